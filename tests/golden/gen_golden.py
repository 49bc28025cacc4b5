"""Generates the golden fixtures in this directory from the REFERENCE itself.

Run here, where the reference checkout exists (the GPU machine has none):

    make -C oracle REF=/root/reference && python tests/golden/gen_golden.py

It loads each preset scene into the reference harness (oracle/_ref, the
reference's unmodified src/*.cc compiled by oracle/Makefile) and records:
  <scene>.sd               the scene-description text the fixtures were made from
  <scene>_trace.npz        rays (2048 x 7) and the reference's world->hit
                           results: hit_f (t,u,v,p,n), hit_i (hit, primitive id),
                           with constant_medium consuming one fresh drand_r
                           stream in ray order
  <scene>_bvh.npz          pre-order BVH topology dumps of every bvh_node line
  <scene>_render.npz       reference renders (main.cpp:109-159 replayed) at low
                           resolution, K runs with distinct per-row drand_r
                           burn-in, as per-pixel means before gamma
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tiny-path-tracer_gb300"))

import pyoracle  # noqa: E402
from tpt import scenes  # noqa: E402

TRACE_SCENES = ["cornell", "one_weekend", "cornell_guiding", "ties", "instances", "next_week"]
RENDERS = {  # scene: (width, height, spp, max_depth, runs)
    "cornell": (48, 48, 64, 50, 8),
    "cornell_guiding": (48, 48, 64, 50, 8),
}
N_RAYS = 2048


def bvh_ids(sd) -> list[int]:
    return [int(l.split()[1]) for l in sd.lines if l.startswith("node ") and l.split()[2] == "bvh_node"]


def main() -> None:
    if not pyoracle.ref_available():
        raise SystemExit("reference harness not built: make -C oracle REF=/path/to/reference")
    for name in TRACE_SCENES:
        sd = scenes.PRESETS[name]()
        text = sd.text()
        with open(os.path.join(HERE, f"{name}.sd"), "w") as f:
            f.write(text)
        ora = pyoracle.Scene(text)
        ref = pyoracle.RefScene(text)
        rays = ora.make_rays(N_RAYS, 20260, 0.5, 0.05)
        hf, hi = ref.trace(rays)
        np.savez_compressed(os.path.join(HERE, f"{name}_trace.npz"), rays=rays, hit_f=hf, hit_i=hi)
        dumps = {}
        for b in bvh_ids(sd):
            boxes, kids = ref.bvh_dump(b)
            dumps[f"boxes_{b}"] = boxes
            dumps[f"kids_{b}"] = kids
        np.savez_compressed(os.path.join(HERE, f"{name}_bvh.npz"), **dumps)
        print(name, "trace + bvh", hi[:, 0].sum(), "hits")
    for name, (w, h, spp, depth, runs) in RENDERS.items():
        text = scenes.PRESETS[name]().text()
        ref = pyoracle.RefScene(text)
        imgs = []
        for r in range(runs):
            img, _ = ref.render(w, h, spp, depth, lean=1, burn_run=r + 1, burn_row=1009)
            imgs.append(img)
        np.savez_compressed(os.path.join(HERE, f"{name}_render.npz"), images=np.stack(imgs),
                            meta=np.array([w, h, spp, depth, runs]))
        print(name, "render", np.stack(imgs).mean())


if __name__ == "__main__":
    main()
