"""Build recipe of the product library: libtpt.so (CUDA kernels for sm_103a +
host scene compiler + C ABI), compiled in-tree into tiny-path-tracer_gb300/_build.

    python tiny-path-tracer_gb300/build.py

The translation units compile in parallel: kernels.cu (path tracing),
learn.cu (tensor-core MLPs of the learned parts) and lbvh.cu (the GPU BVH
builder) with nvcc
(-gencode arch=compute_103a,code=sm_103a; hit arithmetic is written with
unfused round-to-nearest intrinsics, so FMA contraction stays on for the
rest), scene.cc (scene compiler) and config.cc (config.ini, PPM strips) with
g++ (-ffp-contract=off).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libtpt.so")


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_home(nvcc: str) -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def sources() -> list[str]:
    return [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC))]


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(s) <= t for s in sources()) and os.path.getmtime(
        os.path.join(PKG, "..", "include", "tpt.h")) <= t


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    cuda = _cuda_home(nvcc)
    objs, cmds = [], []
    for cu in ("kernels.cu", "learn.cu", "lbvh.cu"):
        obj = os.path.join(OUT, cu.replace(".cu", ".o"))
        objs.append(obj)
        cmds.append([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "-std=c++17",
                     "-Xcompiler", "-fPIC", "-c", os.path.join(CSRC, cu), "-o", obj])
    for cc in ("scene.cc", "config.cc"):
        obj = os.path.join(OUT, cc.replace(".cc", ".o"))
        objs.append(obj)
        cmds.append(["g++", "-std=c++17", "-O3", "-ffp-contract=off", "-fPIC", "-Wall", f"-I{cuda}/include", "-c",
                     os.path.join(CSRC, cc), "-o", obj])
    procs = [subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT) for cmd in cmds]
    for cmd, p in zip(cmds, procs):
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError(f"build failed: {' '.join(cmd)}\n{out.decode(errors='replace')}")
        if verbose and out:
            sys.stdout.write(out.decode(errors="replace"))
    link = [nvcc, "-shared", "-gencode", "arch=compute_103a,code=sm_103a", *objs, "-o", LIB + ".tmp"]
    r = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout.decode(errors="replace"))
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
