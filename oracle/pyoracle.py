"""ctypes bindings of the CPU oracle (liboracle.so) and of the reference
harness (_ref/libtptref.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke() entry point and
by bench.py's CPU-baseline / reference legs, always as the reference that
results are compared against or as the timed CPU baseline - never as the
product path.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libtptref.so")


def build(ref_dir: str | None = None, jobs: int = 4) -> None:
    cmd = ["make", "-C", HERE, f"-j{jobs}"]
    if ref_dir is not None:
        cmd.append(f"REF={ref_dir}")
    subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL)


class RenderParams(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("spp", C.c_int32), ("max_depth", C.c_int32),
                ("semantics", C.c_int32), ("background", C.c_int32), ("sky_scale", C.c_float),
                ("nthreads", C.c_int32), ("seed", C.c_uint64), ("row_begin", C.c_int32),
                ("row_end", C.c_int32)]


class Counters(C.Structure):
    _fields_ = [(n, C.c_int64) for n in ("segments", "aabb_tests", "sphere_tests", "rect_tests",
                                         "instance_xforms", "medium_tests", "lambertian", "metal",
                                         "dielectric", "light_pdf_evals")]

    def as_dict(self) -> dict:
        return {n: int(getattr(self, n)) for n, _ in self._fields_}


class RefRenderParams(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("spp", C.c_int32), ("max_depth", C.c_int32),
                ("lean", C.c_int32), ("burn_run", C.c_int32), ("burn_row", C.c_int32),
                ("row_begin", C.c_int32), ("row_end", C.c_int32)]


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build()
        L = C.CDLL(ORACLE_SO)
        L.oracle_scene_load.restype = C.c_void_p
        L.oracle_scene_load.argtypes = [C.c_char_p, C.c_char_p, C.c_int]
        L.oracle_scene_free.argtypes = [C.c_void_p]
        L.oracle_scene_info.argtypes = [C.c_void_p, C.c_void_p]
        L.oracle_bvh_dump.restype = C.c_int32
        L.oracle_bvh_dump.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_int32]
        L.oracle_world_box.restype = C.c_int32
        L.oracle_world_box.argtypes = [C.c_void_p, C.c_void_p]
        L.oracle_trace.restype = C.c_int32
        L.oracle_trace.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_uint64, C.c_int32, C.c_void_p,
                                   C.c_void_p, C.c_int32, C.c_void_p]
        L.oracle_make_rays.argtypes = [C.c_void_p, C.c_int64, C.c_uint64, C.c_float, C.c_float, C.c_void_p]
        L.oracle_render.restype = C.c_int32
        L.oracle_render.argtypes = [C.c_void_p, C.POINTER(RenderParams), C.c_void_p, C.POINTER(Counters)]
        L.oracle_quantize.argtypes = [C.c_void_p, C.c_int64, C.c_void_p]
        L.oracle_philox.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.oracle_procedural_image.argtypes = [C.c_int32, C.c_int32, C.c_uint32, C.c_void_p]
        L.oracle_lbvh_keys.restype = C.c_int32
        L.oracle_lbvh_keys.argtypes = [C.c_void_p, C.c_int32, C.c_void_p]
        L.oracle_lbvh_build.restype = C.c_int32
        L.oracle_lbvh_build.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_SO)


def reference_dir() -> str | None:
    """The reference checkout the harness was compiled from (recorded by
    oracle/Makefile), if it is still there."""
    try:
        with open(os.path.join(HERE, "_ref", "reference_dir.txt")) as f:
            d = f.read().strip()
    except OSError:
        return None
    return d if os.path.isdir(os.path.join(d, "src")) else None


def ref_lib():
    global _ref
    if _ref is None:
        L = C.CDLL(REF_SO)
        L.ref_scene_load.restype = C.c_void_p
        L.ref_scene_load.argtypes = [C.c_char_p, C.c_char_p, C.c_int]
        L.ref_bvh_dump.restype = C.c_int32
        L.ref_bvh_dump.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_int32]
        L.ref_trace.restype = C.c_int32
        L.ref_trace.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]
        L.ref_render.restype = C.c_double
        L.ref_render.argtypes = [C.c_void_p, C.POINTER(RefRenderParams), C.c_void_p]
        L.ref_hardware_concurrency.restype = C.c_int32
        L.ref_frontend_bvh.restype = C.c_int32
        L.ref_frontend_bvh.argtypes = [C.c_int32, C.c_void_p, C.c_int32]
        L.ref_scene_function_bvhs.restype = C.c_int32
        L.ref_scene_function_bvhs.argtypes = [C.c_char_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32,
                                              C.POINTER(C.c_int32)]
        L.ref_config_parse.restype = None
        L.ref_config_parse.argtypes = [C.c_char_p, C.c_void_p]
        _ref = L
    return _ref


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


class Scene:
    """An SD scene loaded into the oracle."""

    def __init__(self, sd_text: str):
        err = C.create_string_buffer(512)
        self._h = lib().oracle_scene_load(sd_text.encode(), err, 512)
        if not self._h:
            raise ValueError("oracle scene load failed: " + err.value.decode())

    def __del__(self):
        if getattr(self, "_h", None):
            lib().oracle_scene_free(self._h)
            self._h = None

    def info(self) -> np.ndarray:
        out = np.zeros(8, np.int32)
        lib().oracle_scene_info(self._h, _ptr(out))
        return out

    def bvh_dump(self, sd_id: int):
        n = lib().oracle_bvh_dump(self._h, sd_id, None, None, 0)
        if n < 0:
            raise KeyError(sd_id)
        boxes = np.zeros((n, 6), np.float32)
        kids = np.zeros((n, 2), np.int32)
        lib().oracle_bvh_dump(self._h, sd_id, _ptr(boxes), _ptr(kids), n)
        return boxes, kids

    def world_box(self):
        b = np.zeros(6, np.float32)
        ok = lib().oracle_world_box(self._h, _ptr(b))
        return b if ok else None

    def make_rays(self, n: int, seed: int, frac_camera=0.5, frac_axis=0.05) -> np.ndarray:
        rays = np.zeros((n, 7), np.float32)
        lib().oracle_make_rays(self._h, n, seed, frac_camera, frac_axis, _ptr(rays))
        return rays

    def trace(self, rays: np.ndarray, seed: int = 0, media_mode: int = 0, nthreads: int = 0,
              counters: bool = False):
        rays = np.ascontiguousarray(rays, np.float32)
        n = rays.shape[0]
        f = np.zeros((n, 9), np.float32)
        i = np.zeros((n, 2), np.int32)
        cnt = Counters()
        nt = nthreads or min(os.cpu_count() or 1, 16)
        rc = lib().oracle_trace(self._h, _ptr(rays), n, seed, media_mode, _ptr(f), _ptr(i), nt,
                                C.byref(cnt) if counters else None)
        if rc:
            raise RuntimeError("oracle_trace failed")
        return (f, i, cnt.as_dict()) if counters else (f, i)

    def render(self, width, height, spp, max_depth=50, semantics=0, background=0, sky_scale=1.0,
               seed=1, nthreads=0, rows=(0, 0)):
        p = RenderParams(width, height, spp, max_depth, semantics, background, sky_scale,
                         nthreads or (os.cpu_count() or 1), seed, rows[0], rows[1])
        out = np.zeros((height, width, 3), np.float32)
        cnt = Counters()
        rc = lib().oracle_render(self._h, C.byref(p), _ptr(out), C.byref(cnt))
        if rc:
            raise RuntimeError("oracle_render failed")
        return out, cnt.as_dict()


def quantize(mean_rgb: np.ndarray) -> np.ndarray:
    m = np.ascontiguousarray(mean_rgb, np.float32)
    out = np.zeros(m.shape, np.uint8)
    lib().oracle_quantize(_ptr(m), m.size // 3, _ptr(out))
    return out


def philox(ctr, key) -> np.ndarray:
    c = np.asarray(ctr, np.uint32)
    k = np.asarray(key, np.uint32)
    o = np.zeros(4, np.uint32)
    lib().oracle_philox(_ptr(c), _ptr(k), _ptr(o))
    return o


def procedural_image(w: int, h: int, seed: int) -> np.ndarray:
    out = np.zeros((h, w, 3), np.uint8)
    lib().oracle_procedural_image(w, h, seed, _ptr(out))
    return out


def lbvh_keys(boxes: np.ndarray):
    """Unsorted keys of the linear BVH over boxes (n x 6: min xyz, max
    xyz) and the Morton bits per axis (oracle/lbvh.cc)."""
    boxes = np.ascontiguousarray(boxes, np.float32)
    keys = np.zeros(len(boxes), np.uint64)
    bits = lib().oracle_lbvh_keys(_ptr(boxes), len(boxes), _ptr(keys))
    return keys, bits


def lbvh_build(boxes: np.ndarray):
    """The linear BVH over boxes, restated on the CPU (oracle/lbvh.cc):
    pre-order node boxes (m x 6), children (m x 2; >= 0 node, < 0 ~box
    index), skip (m) and the depth in internal-node levels."""
    boxes = np.ascontiguousarray(boxes, np.float32)
    m = max(len(boxes) - 1, 1)
    nb = np.zeros((m, 6), np.float32)
    kids = np.zeros((m, 2), np.int32)
    skip = np.zeros(m, np.int32)
    depth = C.c_int32(0)
    k = lib().oracle_lbvh_build(_ptr(boxes), len(boxes), _ptr(nb), _ptr(kids), _ptr(skip), C.byref(depth))
    if k < 0:
        raise ValueError("lbvh_build needs at least one box")
    return nb, kids, skip, depth.value


def ref_frontend_bvh(n: int):
    """Pre-order node boxes of the reference's bvh_node over n spheres laid
    out with its drand_r (the sequence of tests/frontend/random_bvh.cc)."""
    cap = 2 * n + 2
    out = np.zeros((cap, 6), np.float32)
    k = ref_lib().ref_frontend_bvh(n, out.ctypes.data_as(C.c_void_p), cap)
    return out[:k]


def ref_scene_function_bvhs(name: str):
    """The bvh_nodes one of the reference's own scene functions
    (utils.cc:96-414) builds, run on a fresh thread: a list of (boxes n x 6,
    kids n x 2) per tree in build order, kids -1 for a leaf."""
    nt = C.c_int32()
    n = ref_lib().ref_scene_function_bvhs(name.encode(), None, None, None, 0, C.byref(nt))
    if n < 0:
        raise KeyError(name)
    boxes = np.zeros((max(n, 1), 6), np.float32)
    kids = np.zeros((max(n, 1), 2), np.int32)
    sizes = np.zeros(max(nt.value, 1), np.int32)
    ref_lib().ref_scene_function_bvhs(name.encode(), _ptr(boxes), _ptr(kids), _ptr(sizes), n, C.byref(nt))
    out, off = [], 0
    for k in sizes[:nt.value]:
        out.append((boxes[off:off + k], kids[off:off + k]))
        off += k
    return out


def ref_config_parse(text: str) -> list:
    """config.ini values as the reference's main.cpp reads them (inipp)."""
    out = (C.c_double * 10)()
    ref_lib().ref_config_parse(text.encode(), out)
    return list(out)


class RefScene:
    """An SD scene built from the reference's own classes (harness)."""

    def __init__(self, sd_text: str):
        err = C.create_string_buffer(512)
        self._h = ref_lib().ref_scene_load(sd_text.encode(), err, 512)
        if not self._h:
            raise ValueError("reference scene load failed: " + err.value.decode())

    def bvh_dump(self, sd_id: int):
        n = ref_lib().ref_bvh_dump(self._h, sd_id, None, None, 0)
        if n < 0:
            raise KeyError(sd_id)
        boxes = np.zeros((n, 6), np.float32)
        kids = np.zeros((n, 2), np.int32)
        ref_lib().ref_bvh_dump(self._h, sd_id, _ptr(boxes), _ptr(kids), n)
        return boxes, kids

    def trace(self, rays: np.ndarray):
        rays = np.ascontiguousarray(rays, np.float32)
        n = rays.shape[0]
        f = np.zeros((n, 9), np.float32)
        i = np.zeros((n, 2), np.int32)
        ref_lib().ref_trace(self._h, _ptr(rays), n, _ptr(f), _ptr(i))
        return f, i

    def render(self, width, height, spp, max_depth=50, lean=1, burn_run=0, burn_row=0, rows=(0, 0)):
        p = RefRenderParams(width, height, spp, max_depth, lean, burn_run, burn_row, rows[0], rows[1])
        out = np.zeros((height, width, 3), np.float32)
        secs = ref_lib().ref_render(self._h, C.byref(p), _ptr(out))
        return out, secs
