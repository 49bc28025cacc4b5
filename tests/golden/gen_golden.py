"""Generates the golden fixtures in this directory from the REFERENCE itself.

Run where the reference checkout exists (the GPU test machines have none):

    make -C oracle REF=<reference checkout> && python tests/golden/gen_golden.py [scene ...]

It loads each preset scene into the reference harness (oracle/_ref, the
reference's unmodified src/*.cc compiled by oracle/Makefile) and records:
  <scene>.sd               the scene-description text the fixtures were made from
  <scene>_trace.npz        rays (2048 x 7) and the reference's world->hit
                           results: hit_f (t,u,v,p,n), hit_i (hit, primitive id),
                           with constant_medium consuming one fresh drand_r
                           stream in ray order
  <scene>_bvh.npz          pre-order BVH topology dumps of every bvh_node line
  <scene>_edge.npz         known-answer rays at the edges of the primitives'
                           arithmetic (tangent and near-tangent rays, rays
                           from sphere surfaces, rect/box edges and corners,
                           axis-parallel rays) with the reference's results
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

TRACE_SCENES = ["cornell", "one_weekend", "cornell_guiding", "ties", "instances", "next_week",
                "metals", "textures", "motion", "media"]
RENDERS = {  # scene: (width, height, spp, max_depth, runs)
    "cornell": (48, 48, 64, 50, 8),
    "cornell_guiding": (48, 48, 64, 50, 8),
    "metals": (48, 48, 64, 50, 8),
    "textures": (48, 48, 64, 50, 8),
    "motion": (48, 48, 64, 50, 8),
    "media": (48, 48, 64, 50, 8),
}
N_RAYS = 2048


EDGE_SCENES = ["cornell", "one_weekend", "instances", "next_week", "metals", "textures"]


def edge_rays(sd, seed: int) -> np.ndarray:
    """Known-answer rays at the edges of the primitives' arithmetic (float32,
    7 floats each: origin, direction, time): rays tangent to spheres and
    within 1e-6 of tangency, rays leaving or entering a sphere at its
    surface, rays aimed at the edges and corners of rects and boxes, and
    axis-parallel rays through those edges (direction components exactly 0)."""
    rng = np.random.default_rng(seed)
    out = []

    def ray(o, d):
        out.append([*np.asarray(o, np.float32), *np.asarray(d, np.float32), 0.0])

    def unit(v):
        return v / np.linalg.norm(v)

    spheres, rects, boxes = [], [], []
    for l in sd.lines:
        f = l.split()
        if len(f) < 3 or f[0] != "node":
            continue
        if f[2] == "sphere":
            spheres.append((np.array(f[3:6], np.float64), float(f[6])))
        elif f[2] in ("xy_rect", "xz_rect", "yz_rect"):
            rects.append((f[2], [float(v) for v in f[3:8]]))
        elif f[2] == "box":
            boxes.append((np.array(f[3:6], np.float64), np.array(f[6:9], np.float64)))
    for k in rng.permutation(len(spheres))[:40]:
        c, r = spheres[k]
        for _ in range(6):
            u = unit(rng.normal(size=3))
            v = unit(np.cross(u, rng.normal(size=3)))
            for scale in (1.0, 1.0 - 1e-6, 1.0 + 1e-6):
                p = c + r * scale * u
                ray(p - 3.0 * r * v, v * rng.uniform(0.5, 2.0))
        u = unit(rng.normal(size=3))
        ray(c + r * u, u)      # leaving the surface
        ray(c + r * u, -u)     # entering at the surface
    axes = {"xy_rect": (0, 1, 2), "xz_rect": (0, 2, 1), "yz_rect": (1, 2, 0)}
    for kind, (a0, a1, b0, b1, k) in rects:
        ia, ib, ik = axes[kind]
        for (a, b) in [(a0, b0), (a1, b1), (a0, 0.5 * (b0 + b1)), (0.5 * (a0 + a1), b1)]:
            t = np.zeros(3)
            t[ia], t[ib], t[ik] = a, b, k
            o = t + rng.normal(size=3) * 50.0
            ray(o, t - o)
            o2 = t.copy()
            o2[ia] -= 10.0     # axis-parallel through the edge: two direction components exactly 0
            d = np.zeros(3)
            d[ia] = 1.0
            ray(o2, d)
    for lo, hi in boxes[:60]:
        for corner in range(8):
            t = np.where([(corner >> i) & 1 for i in range(3)], hi, lo)
            o = t + rng.normal(size=3) * 40.0
            ray(o, t - o)
    return np.array(out, np.float32)


def bvh_ids(sd) -> list[int]:
    return [int(l.split()[1]) for l in sd.lines if l.startswith("node ") and l.split()[2] == "bvh_node"]


def main(only: list[str]) -> None:
    """Regenerates the fixtures of the scenes named in `only` (all when empty)."""
    if not pyoracle.ref_available():
        raise SystemExit("reference harness not built: make -C oracle REF=/path/to/reference")
    pick = (lambda names: [n for n in names if n in only]) if only else (lambda names: list(names))
    for name in pick(TRACE_SCENES):
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
    for name in pick(EDGE_SCENES):
        text = scenes.PRESETS[name]().text()
        rays = edge_rays(scenes.PRESETS[name](), 77)
        hf, hi = pyoracle.RefScene(text).trace(rays)
        np.savez_compressed(os.path.join(HERE, f"{name}_edge.npz"), rays=rays, hit_f=hf, hit_i=hi)
        print(name, "edge rays", len(rays), hi[:, 0].sum(), "hits")
    for name in pick(RENDERS):
        w, h, spp, depth, runs = RENDERS[name]
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
    main(sys.argv[1:])
