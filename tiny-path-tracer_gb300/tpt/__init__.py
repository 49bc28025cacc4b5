"""Python binding of the tiny-path-tracer GB300 library (libtpt.so) over its
C ABI (include/tpt.h), via ctypes.

This is a thin host-side mirror of the reference's entry points: a scene is
built from scene-description text (tpt.scenes generates the workloads), a
Context owns a GPU, `trace_closest` is the batched `world->hit`, `render` the
per-pixel sample loop with color().  There is no CPU fallback: loading raises
if the compiled library is missing, and device calls raise TptError when no
GPU is usable.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG, "_build", "libtpt.so")

TPT_MEM_HOST = 0
TPT_MEM_DEVICE = 1
SEMANTICS_REFERENCE = 0
SEMANTICS_PHYSICAL = 1
BACKGROUND_BLACK = 0
BACKGROUND_SKY = 1
ENGINE_AUTO = 0
ENGINE_WAVEFRONT = 1
ENGINE_PERSISTENT = 2
BVH_REFERENCE, BVH_SAH, BVH_LBVH = 0, 1, 2

STATUS = {0: "TPT_OK", 1: "TPT_ERR_INVALID_ARGUMENT", 2: "TPT_ERR_PARSE", 3: "TPT_ERR_UNSUPPORTED",
          4: "TPT_ERR_NO_BOUNDING_BOX", 5: "TPT_ERR_CUDA", 6: "TPT_ERR_OUT_OF_MEMORY",
          7: "TPT_ERR_DEVICE_TIMEOUT", 8: "TPT_ERR_STACK_OVERFLOW", 9: "TPT_ERR_NO_DEVICE",
          10: "TPT_ERR_BAD_HANDLE"}


class TptError(RuntimeError):
    def __init__(self, status: int, msg: str = ""):
        self.status = status
        super().__init__(f"{STATUS.get(status, status)}{': ' + msg if msg else ''}")


class RenderParams(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("spp", C.c_int32), ("max_depth", C.c_int32),
                ("semantics", C.c_int32), ("background", C.c_int32), ("sky_scale", C.c_float),
                ("seed", C.c_uint64), ("engine", C.c_int32), ("block", C.c_int32), ("wave", C.c_int32),
                ("accumulate_fp64", C.c_int32), ("profile", C.c_int32), ("flat_nodes", C.c_int32),
                ("refill", C.c_int32)]


class Config(C.Structure):
    """tpt_config: the config.ini keys of main.cpp:29-56."""
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("sample", C.c_int32), ("recur_depth", C.c_int32),
                ("fov", C.c_float), ("allow_bonus_pic", C.c_int32), ("bonus_pic", C.c_int32),
                ("aperture", C.c_float), ("start_time", C.c_float), ("end_time", C.c_float)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class RenderStats(C.Structure):
    _fields_ = [("samples", C.c_int64), ("segments", C.c_int64), ("iterations", C.c_int32),
                ("kernel_launches", C.c_int32), ("device_ms", C.c_double), ("traverse_ms", C.c_double),
                ("shade_ms", C.c_double), ("traverse_launches", C.c_int32), ("shade_launches", C.c_int32)]

    def as_dict(self) -> dict:
        return {n: getattr(self, n) for n, _ in self._fields_}


class BatchItem(C.Structure):
    _fields_ = [("slot", C.c_int32), ("width", C.c_int32), ("height", C.c_int32), ("spp", C.c_int32),
                ("out_rgb", C.c_void_p)]


class GuideParams(C.Structure):
    _fields_ = [("passes", C.c_int32), ("train_steps", C.c_int32), ("batch", C.c_int32), ("lr", C.c_float),
                ("grid_res", C.c_int32), ("alpha", C.c_float), ("record_cap", C.c_int32), ("seed", C.c_uint64),
                ("light_share", C.c_float), ("warm_start", C.c_int32)]


class GuideStats(C.Structure):
    _fields_ = [("render_ms", C.c_double), ("train_ms", C.c_double), ("final_loss", C.c_float),
                ("records", C.c_int64)]

    def as_dict(self) -> dict:
        return {n: getattr(self, n) for n, _ in self._fields_}


class NrcParams(C.Structure):
    _fields_ = [("passes", C.c_int32), ("train_steps", C.c_int32), ("batch", C.c_int32), ("lr", C.c_float),
                ("terminate_depth", C.c_int32), ("train_stride", C.c_int32), ("record_cap", C.c_int32),
                ("query_cap", C.c_int32), ("seed", C.c_uint64), ("warm_start", C.c_int32),
                ("first_pass_spp", C.c_int32), ("first_train_steps", C.c_int32), ("spread_c", C.c_float)]


class NrcStats(C.Structure):
    _fields_ = [("render_ms", C.c_double), ("infer_ms", C.c_double), ("train_ms", C.c_double),
                ("final_loss", C.c_float), ("records", C.c_int64), ("queries", C.c_int64)]

    def as_dict(self) -> dict:
        return {n: getattr(self, n) for n, _ in self._fields_}


class SceneInfo(C.Structure):
    _fields_ = [(n, C.c_int32) for n in ("n_nodes", "n_leaves", "n_items", "n_blas", "n_materials",
                                         "n_textures", "n_lights", "max_stack")] + [("arena_bytes", C.c_int64)]

    def as_dict(self) -> dict:
        return {n: getattr(self, n) for n, _ in self._fields_}


# Every symbol include/tpt.h declares, with its ctypes signature.
_SIGS = {
    "tpt_status_string": (C.c_char_p, [C.c_int32]),
    "tpt_version": (C.c_char_p, []),
    "tpt_last_error": (C.c_char_p, []),
    "tpt_builder_create": (C.c_int32, [C.c_void_p]),
    "tpt_builder_destroy": (None, [C.c_void_p]),
    "tpt_constant_texture": (C.c_int32, [C.c_void_p, C.c_float, C.c_float, C.c_float]),
    "tpt_checker_texture": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32]),
    "tpt_perlin_noise_texture": (C.c_int32, [C.c_void_p, C.c_float]),
    "tpt_perlin_tables": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "tpt_image_texture": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32]),
    "tpt_lambertian": (C.c_int32, [C.c_void_p, C.c_int32]),
    "tpt_metal": (C.c_int32, [C.c_void_p, C.c_float, C.c_float, C.c_float, C.c_float]),
    "tpt_dielectric": (C.c_int32, [C.c_void_p, C.c_float]),
    "tpt_diffuse_light": (C.c_int32, [C.c_void_p, C.c_int32]),
    "tpt_isotropic": (C.c_int32, [C.c_void_p, C.c_int32]),
    "tpt_sphere": (C.c_int32, [C.c_void_p] + [C.c_float] * 4 + [C.c_int32]),
    "tpt_moving_sphere": (C.c_int32, [C.c_void_p] + [C.c_float] * 9 + [C.c_int32]),
    "tpt_xy_rect": (C.c_int32, [C.c_void_p] + [C.c_float] * 5 + [C.c_int32]),
    "tpt_xz_rect": (C.c_int32, [C.c_void_p] + [C.c_float] * 5 + [C.c_int32]),
    "tpt_yz_rect": (C.c_int32, [C.c_void_p] + [C.c_float] * 5 + [C.c_int32]),
    "tpt_flip_normal": (C.c_int32, [C.c_void_p, C.c_int32]),
    "tpt_box": (C.c_int32, [C.c_void_p] + [C.c_float] * 6 + [C.c_int32]),
    "tpt_translate": (C.c_int32, [C.c_void_p, C.c_int32, C.c_float, C.c_float, C.c_float]),
    "tpt_rotate_y": (C.c_int32, [C.c_void_p, C.c_int32, C.c_float]),
    "tpt_constant_medium": (C.c_int32, [C.c_void_p, C.c_int32, C.c_float, C.c_int32]),
    "tpt_hitable_list": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_int32]),
    "tpt_bvh_node": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_int32, C.c_float, C.c_float]),
    "tpt_builder_set_world": (C.c_int32, [C.c_void_p, C.c_int32]),
    "tpt_builder_set_light_shape": (C.c_int32, [C.c_void_p, C.c_int32]),
    "tpt_builder_set_camera": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p] + [C.c_float] * 6),
    "tpt_scene_compile": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "tpt_scene_from_text": (C.c_int32, [C.c_char_p, C.c_void_p, C.c_char_p, C.c_size_t]),
    "tpt_scene_destroy": (None, [C.c_void_p]),
    "tpt_scene_get_info": (C.c_int32, [C.c_void_p, C.POINTER(SceneInfo)]),
    "tpt_scene_bvh_dump": (C.c_int32, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_int32]),
    "tpt_context_create": (C.c_int32, [C.c_int32, C.c_void_p]),
    "tpt_context_destroy": (None, [C.c_void_p]),
    "tpt_context_set_stream": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "tpt_context_set_option": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int64]),
    "tpt_scene_upload": (C.c_int32, [C.c_void_p, C.c_void_p, C.POINTER(C.c_int32)]),
    "tpt_scene_release": (C.c_int32, [C.c_void_p, C.c_int32]),
    "tpt_bvh_build_boxes": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_void_p]),
    "tpt_trace_closest": (C.c_int32, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int64, C.c_uint64, C.c_void_p,
                                      C.c_void_p, C.c_int32]),
    "tpt_render_params_default": (None, [C.POINTER(RenderParams)]),
    "tpt_render": (C.c_int32, [C.c_void_p, C.c_int32, C.POINTER(RenderParams), C.c_void_p, C.c_int32,
                               C.POINTER(RenderStats)]),
    "tpt_render_noalloc": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_int64, C.POINTER(RenderParams), C.c_void_p,
                                       C.c_void_p]),
    "tpt_render_batch": (C.c_int32, [C.c_void_p, C.POINTER(BatchItem), C.c_int32, C.POINTER(RenderParams),
                                     C.c_int32, C.POINTER(RenderStats)]),
    "tpt_autotune_nrc": (C.c_int32, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_void_p]),
    "tpt_autotune": (C.c_int32, [C.c_void_p, C.c_int32, C.POINTER(RenderParams), C.c_int32,
                                 C.POINTER(C.c_double)]),
    "tpt_mlp_create": (C.c_int32, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_uint64, C.c_void_p]),
    "tpt_mlp_destroy": (None, [C.c_void_p]),
    "tpt_mlp_param_count": (C.c_int64, [C.c_void_p]),
    "tpt_mlp_set_params": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "tpt_mlp_get_params": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "tpt_mlp_get_grad": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "tpt_mlp_forward": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]),
    "tpt_mlp_cache_accumulate": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p,
                                             C.c_void_p, C.c_int64, C.c_void_p]),
    "tpt_mlp_backward_given": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_float,
                                           C.c_void_p]),
    "tpt_mlp_backward_vmf": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_float, C.c_void_p,
                                         C.c_void_p]),
    "tpt_mlp_backward_rel_l2": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_float,
                                            C.c_void_p, C.c_void_p]),
    "tpt_mlp_backward_rel_l2_records": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_int64, C.c_uint32, C.c_uint32,
                                                    C.c_void_p, C.c_void_p, C.c_int64, C.c_float, C.c_void_p,
                                                    C.c_void_p]),
    "tpt_guide_encode": (C.c_int32, [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                     C.c_void_p]),
    "tpt_nrc_encode": (C.c_int32, [C.c_void_p, C.c_int64, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p,
                                   C.c_void_p]),
    "tpt_mlp_adam": (C.c_int32, [C.c_void_p, C.c_float, C.c_float, C.c_void_p]),
    "tpt_mlp_last_error": (C.c_char_p, []),
    "tpt_guide_params_default": (None, [C.POINTER(GuideParams)]),
    "tpt_render_guided": (C.c_int32, [C.c_void_p, C.c_int32, C.POINTER(RenderParams), C.POINTER(GuideParams),
                                      C.c_void_p, C.c_int32, C.POINTER(RenderStats), C.POINTER(GuideStats)]),
    "tpt_guide_records": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_int64, C.POINTER(C.c_int64)]),
    "tpt_nrc_params_default": (None, [C.POINTER(NrcParams)]),
    "tpt_autotune_batch": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_int32, C.POINTER(RenderParams), C.c_int32,
                                       C.POINTER(C.c_double)]),
    "tpt_config_default": (None, [C.POINTER(Config)]),
    "tpt_builder_set_bvh_build": (C.c_int32, [C.c_void_p, C.c_int32]),
    "tpt_scene_from_text_opt": (C.c_int32, [C.c_char_p, C.c_int32, C.POINTER(C.c_void_p), C.c_char_p, C.c_size_t]),
    "tpt_config_parse": (C.c_int32, [C.c_char_p, C.POINTER(Config)]),
    "tpt_config_load": (C.c_int32, [C.c_char_p, C.POINTER(Config)]),
    "tpt_scene_get_camera": (C.c_int32, [C.c_void_p, C.POINTER(C.c_float)]),
    "tpt_scene_set_camera": (C.c_int32, [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                         C.POINTER(C.c_float), C.c_float, C.c_float, C.c_float, C.c_float,
                                         C.c_float, C.c_float]),
    "tpt_render_snapshots": (C.c_int32, [C.c_void_p, C.c_int32, C.POINTER(RenderParams), C.c_int32, C.c_void_p,
                                         C.c_void_p, C.c_int32, C.POINTER(RenderStats)]),
    "tpt_render_range": (C.c_int32, [C.c_void_p, C.c_int32, C.POINTER(RenderParams), C.c_int32, C.c_int32,
                                     C.c_void_p, C.POINTER(RenderStats)]),
    "tpt_resolve_sums": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p,
                                     C.c_int32]),
    "tpt_write_ppm_strip": (C.c_int32, [C.c_char_p, C.POINTER(C.c_void_p), C.c_int32, C.c_int32, C.c_int32]),
    "tpt_read_ppm": (C.c_int32, [C.c_char_p, C.c_void_p, C.c_int64, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "tpt_render_nrc": (C.c_int32, [C.c_void_p, C.c_int32, C.POINTER(RenderParams), C.POINTER(NrcParams),
                                   C.c_void_p, C.c_int32, C.POINTER(RenderStats), C.POINTER(NrcStats)]),
    "tpt_learned_save": (C.c_int32, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int64, C.POINTER(C.c_int64)]),
    "tpt_learned_load": (C.c_int32, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int64]),
    "tpt_quantize": (None, [C.c_void_p, C.c_int64, C.c_void_p]),
    "tpt_write_ppm": (C.c_int32, [C.c_char_p, C.c_void_p, C.c_int32, C.c_int32]),
}

_lib = None


def lib():
    """Loads libtpt.so; raises if it has not been built (no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"libtpt.so not built at {LIB_PATH}: run tiny-path-tracer_gb300/build.py")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(st: int, what: str = "") -> None:
    if st != 0:
        detail = lib().tpt_last_error().decode() if st == 5 else ""
        raise TptError(st, what + (f" ({detail})" if detail else ""))


def _ptr(a):
    if isinstance(a, np.ndarray):
        return a.ctypes.data_as(C.c_void_p)
    return C.c_void_p(int(a))  # raw device pointer


class Scene:
    """A compiled scene (host arena) built from scene-description text."""

    def __init__(self, sd_text: str, bvh: str = "reference"):
        """bvh: "reference" (the reference's tree, closest-hit parity),
        "sah" (binned SAH rebuild of every bvh_node on the host, TPT_BVH_SAH)
        or "lbvh" (linear BVH built on the GPU at upload, TPT_BVH_LBVH)."""
        h = C.c_void_p()
        err = C.create_string_buffer(512)
        mode = {"reference": BVH_REFERENCE, "sah": BVH_SAH, "lbvh": BVH_LBVH}[bvh]
        st = lib().tpt_scene_from_text_opt(sd_text.encode(), mode, C.byref(h), err, 512)
        if st != 0:
            raise TptError(st, err.value.decode())
        self._h = h

    @property
    def handle(self):
        return self._h

    def info(self) -> dict:
        i = SceneInfo()
        check(lib().tpt_scene_get_info(self._h, C.byref(i)))
        return i.as_dict()

    def camera(self) -> dict:
        """The camera inputs (tpt_scene_get_camera)."""
        v = (C.c_float * 15)()
        check(lib().tpt_scene_get_camera(self._h, v), "scene_get_camera")
        v = list(v)
        return {"lookfrom": v[0:3], "lookat": v[3:6], "vup": v[6:9], "vfov": v[9], "aspect": v[10],
                "aperture": v[11], "focus": v[12], "time0": v[13], "time1": v[14]}

    def set_camera(self, lookfrom, lookat, vup, vfov, aspect, aperture, focus, time0, time1) -> None:
        f3 = lambda x: (C.c_float * 3)(*x)
        check(lib().tpt_scene_set_camera(self._h, f3(lookfrom), f3(lookat), f3(vup), vfov, aspect, aperture, focus,
                                         time0, time1), "scene_set_camera")

    def apply_config(self, cfg: dict) -> None:
        """main.cpp:86-90: the camera takes the config's fov, aspect
        (width / height), aperture and shutter; the scene keeps its viewpoint
        and focus distance."""
        c = self.camera()
        self.set_camera(c["lookfrom"], c["lookat"], c["vup"], cfg["fov"], cfg["width"] / cfg["height"],
                        cfg["aperture"], c["focus"], cfg["start_time"], cfg["end_time"])

    def bvh_dump(self, user_id: int):
        n = lib().tpt_scene_bvh_dump(self._h, user_id, None, None, 0)
        if n < 0:
            raise TptError(-n, f"bvh_dump({user_id})")
        boxes = np.zeros((n, 6), np.float32)
        kids = np.zeros((n, 2), np.int32)
        lib().tpt_scene_bvh_dump(self._h, user_id, _ptr(boxes), _ptr(kids), n)
        return boxes, kids

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.tpt_scene_destroy(self._h)
            self._h = None


class Context:
    """One GPU: uploaded scenes, scratch buffers, a stream."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        check(lib().tpt_context_create(device, C.byref(h)), "context_create")
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib().tpt_context_destroy(self._h)
            self._h = None

    def __del__(self):
        if _lib is not None:
            self.close()

    def set_stream(self, stream_ptr: int | None):
        check(lib().tpt_context_set_stream(self._h, C.c_void_p(stream_ptr or 0)))

    def set_flat_nodes(self, n: int) -> None:
        """BVHs of at most n nodes use the stackless walk (0: never)."""
        check(lib().tpt_context_set_option(self._h, 1, n), "set_option")

    def upload(self, scene: Scene) -> int:
        slot = C.c_int32()
        check(lib().tpt_scene_upload(self._h, scene.handle, C.byref(slot)), "scene_upload")
        return slot.value

    def release(self, slot: int) -> None:
        check(lib().tpt_scene_release(self._h, slot))

    def bvh_build_boxes(self, boxes: np.ndarray):
        """The GPU linear-BVH builder over boxes (n x 6: min xyz, max xyz):
        pre-order node boxes (m x 6), children (m x 2; >= 0 node, < 0 ~box
        index), skip (m) and the depth in internal-node levels."""
        boxes = np.ascontiguousarray(boxes, np.float32).reshape(-1, 6)
        n = boxes.shape[0]
        m = max(n - 1, 1)
        nb = np.zeros((m, 6), np.float32)
        kids = np.zeros((m, 2), np.int32)
        skip = np.zeros(m, np.int32)
        depth = C.c_int32(0)
        check(lib().tpt_bvh_build_boxes(self._h, _ptr(boxes), n, _ptr(nb), _ptr(kids), _ptr(skip), C.byref(depth)),
              "bvh_build_boxes")
        return nb, kids, skip, depth.value

    def trace_closest(self, slot: int, rays: np.ndarray, seed: int = 0):
        rays = np.ascontiguousarray(rays, np.float32)
        n = rays.shape[0]
        f = np.zeros((n, 9), np.float32)
        i = np.zeros((n, 2), np.int32)
        check(lib().tpt_trace_closest(self._h, slot, _ptr(rays), n, seed, _ptr(f), _ptr(i), TPT_MEM_HOST),
              "trace_closest")
        return f, i

    def trace_closest_device(self, slot: int, rays_ptr: int, n: int, seed: int, hit_f_ptr: int, hit_i_ptr: int):
        check(lib().tpt_trace_closest(self._h, slot, C.c_void_p(rays_ptr), n, seed, C.c_void_p(hit_f_ptr),
                                      C.c_void_p(hit_i_ptr), TPT_MEM_DEVICE), "trace_closest")

    def render(self, slot: int, width: int, height: int, spp: int, max_depth: int = 50,
               semantics: int = SEMANTICS_REFERENCE, background: int = BACKGROUND_BLACK, sky_scale: float = 1.0,
               seed: int = 1, engine: int = ENGINE_AUTO, block: int = 0, wave: int = 0, fp64: bool = False,
               profile: bool = False, flat_nodes: int = 0, out=None, refill: int = 0):
        p = make_params(width, height, spp, max_depth, semantics, background, sky_scale, seed, engine, block,
                        wave, fp64, profile, flat_nodes, refill)
        st = RenderStats()
        if out is None:
            img = np.zeros((height, width, 3), np.float32)
            check(lib().tpt_render(self._h, slot, C.byref(p), _ptr(img), TPT_MEM_HOST, C.byref(st)), "render")
            return img, st.as_dict()
        check(lib().tpt_render(self._h, slot, C.byref(p), C.c_void_p(int(out)), TPT_MEM_DEVICE, C.byref(st)),
              "render")
        return None, st.as_dict()

    def render_range(self, slot: int, width: int, height: int, sample_begin: int, sample_end: int, accum_ptr: int,
                     max_depth: int = 50, semantics: int = SEMANTICS_REFERENCE, background: int = BACKGROUND_BLACK,
                     sky_scale: float = 1.0, seed: int = 1, block: int = 0, wave: int = 0, flat_nodes: int = 0,
                     engine: int = ENGINE_AUTO, profile: bool = False) -> dict:
        """Samples [sample_begin, sample_end) of every pixel, summed into the
        device float4 accumulators at accum_ptr (width*height*4 floats)."""
        p = make_params(width, height, max(1, sample_end - sample_begin), max_depth, semantics, background,
                        sky_scale, seed, engine, block, wave, False, profile, flat_nodes)
        st = RenderStats()
        check(lib().tpt_render_range(self._h, slot, C.byref(p), sample_begin, sample_end, C.c_void_p(int(accum_ptr)),
                                     C.byref(st)), "render_range")
        return st.as_dict()

    def resolve_sums(self, accum_ptr: int, width: int, height: int, spp: int, out=None):
        """Mean image of summed accumulators: a host array, or written to the
        device pointer `out`."""
        if out is None:
            img = np.zeros((height, width, 3), np.float32)
            check(lib().tpt_resolve_sums(self._h, C.c_void_p(int(accum_ptr)), width, height, spp, _ptr(img),
                                         TPT_MEM_HOST), "resolve_sums")
            return img
        check(lib().tpt_resolve_sums(self._h, C.c_void_p(int(accum_ptr)), width, height, spp,
                                     C.c_void_p(int(out)), TPT_MEM_DEVICE), "resolve_sums")
        return None


def _set_fields(struct, values: dict, name: str) -> None:
    """Sets the named fields of a ctypes struct; a name that is not one of
    its fields raises (setattr alone would add a Python attribute the C side
    never sees)."""
    known = {f for f, _ in type(struct)._fields_}
    unknown = sorted(set(values) - known)
    if unknown:
        raise TypeError(f"{name} has no field(s) {', '.join(unknown)}; fields: {', '.join(sorted(known))}")
    for k, v in values.items():
        setattr(struct, k, v)


def render_guided(ctx: "Context", slot: int, width: int, height: int, spp: int, max_depth: int = 50,
                  background: int = BACKGROUND_BLACK, seed: int = 1, out=None, refill: int = 0, engine: int = 0,
                  **guide):
    """Learned path guiding (physical semantics).  guide: fields of
    tpt_guide_params (passes, train_steps, batch, lr, grid_res, alpha,
    record_cap, seed, light_share, warm_start; another name raises
    TypeError).  out: None (host image returned) or a device pointer.
    Returns (image or None, render stats, guide stats)."""
    p = make_params(width, height, spp, max_depth, SEMANTICS_PHYSICAL, background, 1.0, seed, engine=engine,
                    refill=refill)
    g = GuideParams()
    lib().tpt_guide_params_default(C.byref(g))
    _set_fields(g, guide, "tpt_guide_params")
    img = np.zeros((height, width, 3), np.float32) if out is None else None
    dst, mem = (_ptr(img), TPT_MEM_HOST) if out is None else (C.c_void_p(int(out)), TPT_MEM_DEVICE)
    st, gs = RenderStats(), GuideStats()
    check(lib().tpt_render_guided(ctx._h, slot, C.byref(p), C.byref(g), dst, mem, C.byref(st), C.byref(gs)),
          "render_guided")
    return img, st.as_dict(), gs.as_dict()


NET_GUIDE, NET_CACHE = 0, 1


def learned_save(ctx: "Context", which: int) -> np.ndarray:
    """Checkpoint of the context's guiding network (NET_GUIDE) or radiance
    cache (NET_CACHE): weights, Adam moments and step count
    (tpt_learned_save)."""
    n = C.c_int64()
    check(lib().tpt_learned_save(ctx._h, which, None, 0, C.byref(n)), "learned_save")
    out = np.zeros(n.value, np.float32)
    check(lib().tpt_learned_save(ctx._h, which, _ptr(out), n.value, C.byref(n)), "learned_save")
    return out


def learned_load(ctx: "Context", which: int, state: np.ndarray) -> None:
    """Restores a checkpoint; the next render with warm_start=1 continues
    from it (tpt_learned_load)."""
    state = np.ascontiguousarray(state, np.float32)
    check(lib().tpt_learned_load(ctx._h, which, _ptr(state), state.size), "learned_load")


def config(text: str | None = None, path: str | None = None) -> dict:
    """main.cpp's configuration: the defaults, then `text` (INI) or the file
    at `path` on top (tpt_config_parse / tpt_config_load)."""
    c = Config()
    lib().tpt_config_default(C.byref(c))
    if text is not None:
        check(lib().tpt_config_parse(text.encode(), C.byref(c)), "config_parse")
    if path is not None:
        check(lib().tpt_config_load(path.encode(), C.byref(c)), "config_load")
    return c.as_dict()


def render_snapshots(ctx: "Context", slot: int, width: int, height: int, spp: int, bonus_pic: int, **kw):
    """allow_bonus_pic: (final mean, snapshots [bonus_pic, h, w, 3], stats)."""
    p = make_params(width, height, spp, **kw)
    img = np.zeros((height, width, 3), np.float32)
    snaps = np.zeros((max(bonus_pic, 1), height, width, 3), np.float32)
    st = RenderStats()
    check(lib().tpt_render_snapshots(ctx._h, slot, C.byref(p), bonus_pic, _ptr(img), _ptr(snaps), TPT_MEM_HOST,
                                     C.byref(st)), "render_snapshots")
    return img, snaps[:bonus_pic], st.as_dict()


def write_ppm_strip(path: str, images) -> None:
    """Quantised uint8 images (h, w, 3), side by side in one PPM P3 file."""
    imgs = [np.ascontiguousarray(im, np.uint8) for im in images]
    h, w = imgs[0].shape[:2]
    arr = (C.c_void_p * len(imgs))(*[im.ctypes.data for im in imgs])
    check(lib().tpt_write_ppm_strip(path.encode(), arr, len(imgs), w, h), "write_ppm_strip")


def read_ppm(path: str) -> np.ndarray:
    """A PPM image (P3/P6) as uint8 (h, w, 3), row 0 = top."""
    w, h = C.c_int32(), C.c_int32()
    check(lib().tpt_read_ppm(path.encode(), None, 0, C.byref(w), C.byref(h)), "read_ppm")
    img = np.zeros((h.value, w.value, 3), np.uint8)
    check(lib().tpt_read_ppm(path.encode(), _ptr(img), img.size, C.byref(w), C.byref(h)), "read_ppm")
    return img


def guide_records(ctx: "Context", cap: int = 1 << 22) -> np.ndarray:
    """Training records of the last guided pass: (n, 12) float32 rows of
    (position, weight, normal, 0, direction, 0)."""
    n = C.c_int64()
    check(lib().tpt_guide_records(ctx._h, None, 0, C.byref(n)), "guide_records")
    k = min(int(n.value), cap)
    out = np.zeros((k, 12), np.float32)
    if k:
        check(lib().tpt_guide_records(ctx._h, _ptr(out), k, C.byref(n)), "guide_records")
    return out


def render_nrc(ctx: "Context", slot: int, width: int, height: int, spp: int, max_depth: int = 50,
               semantics: int = SEMANTICS_PHYSICAL, background: int = BACKGROUND_BLACK, seed: int = 1, out=None,
               refill: int = 0, engine: int = 0, **nrc):
    """Neural radiance cache render.  nrc: fields of tpt_nrc_params (another
    name raises TypeError).  out: None (host image returned) or a device
    pointer.
    Returns (image or None, render stats, cache stats)."""
    p = make_params(width, height, spp, max_depth, semantics, background, 1.0, seed, engine=engine, refill=refill)
    n = NrcParams()
    lib().tpt_nrc_params_default(C.byref(n))
    _set_fields(n, nrc, "tpt_nrc_params")
    img = np.zeros((height, width, 3), np.float32) if out is None else None
    dst, mem = (_ptr(img), TPT_MEM_HOST) if out is None else (C.c_void_p(int(out)), TPT_MEM_DEVICE)
    st, ns = RenderStats(), NrcStats()
    check(lib().tpt_render_nrc(ctx._h, slot, C.byref(p), C.byref(n), dst, mem, C.byref(st), C.byref(ns)),
          "render_nrc")
    return img, st.as_dict(), ns.as_dict()


def autotune_batch(ctx: "Context", jobs, outs, spp_divisor=8, max_depth=50, semantics=SEMANTICS_REFERENCE,
                   background=BACKGROUND_BLACK, sky_scale=1.0, seed=1):
    """tpt_autotune_batch over jobs (slot, width, height, spp) rendering into
    the device pointers outs; returns (block, variant, flat_nodes, refill,
    Msamples/s)."""
    n = len(jobs)
    arr = (BatchItem * n)()
    for k, (slot, w, h, spp) in enumerate(jobs):
        arr[k] = BatchItem(slot, w, h, spp, int(outs[k]))
    p = make_params(1, 1, 1, max_depth, semantics, background, sky_scale, seed, ENGINE_PERSISTENT)
    best = C.c_double()
    check(lib().tpt_autotune_batch(ctx._h, arr, n, C.byref(p), spp_divisor, C.byref(best)), "autotune_batch")
    return p.block, p.wave, p.flat_nodes, p.refill, best.value


def render_batch(ctx: "Context", jobs, max_depth=50, semantics=SEMANTICS_REFERENCE, background=BACKGROUND_BLACK,
                 sky_scale=1.0, seed=1, block=0, variant=0, flat_nodes=0, profile=False, outs=None, refill=0):
    """jobs: list of (slot, width, height, spp).  outs: None -> host images are
    returned; else a list of device pointers (one per job)."""
    n = len(jobs)
    arr = (BatchItem * n)()
    host = outs is None
    imgs = []
    for k, (slot, w, h, spp) in enumerate(jobs):
        if host:
            img = np.zeros((h, w, 3), np.float32)
            imgs.append(img)
            ptr = img.ctypes.data
        else:
            ptr = int(outs[k])
        arr[k] = BatchItem(slot, w, h, spp, ptr)
    p = make_params(1, 1, 1, max_depth, semantics, background, sky_scale, seed, ENGINE_PERSISTENT, block, variant,
                    False, profile, flat_nodes, refill)
    st = RenderStats()
    check(lib().tpt_render_batch(ctx._h, arr, n, C.byref(p), TPT_MEM_HOST if host else TPT_MEM_DEVICE,
                                 C.byref(st)), "render_batch")
    return (imgs if host else None), st.as_dict()


def autotune_nrc(ctx: "Context", slot: int, width: int, height: int, probe_spp: int = 16, **kw) -> int:
    """Runs tpt_autotune_nrc; returns the engine the slot's cached renders
    will use (ENGINE_WAVEFRONT or ENGINE_PERSISTENT)."""
    kw.setdefault("semantics", SEMANTICS_PHYSICAL)
    p = make_params(width, height, probe_spp, **kw)
    e = C.c_int32()
    check(lib().tpt_autotune_nrc(ctx._h, slot, C.byref(p), probe_spp, C.byref(e)), "autotune_nrc")
    return e.value


def autotune(ctx: "Context", slot: int, width: int, height: int, probe_spp: int = 4, **kw):
    """Runs tpt_autotune; returns (engine, block, wave, flat_nodes, Msamples/s)."""
    p = make_params(width, height, probe_spp, **kw)
    best = C.c_double()
    check(lib().tpt_autotune(ctx._h, slot, C.byref(p), probe_spp, C.byref(best)), "autotune")
    return p.engine, p.block, p.wave, p.flat_nodes, best.value


def make_params(width, height, spp, max_depth=50, semantics=0, background=0, sky_scale=1.0, seed=1, engine=0,
                block=0, wave=0, fp64=False, profile=False, flat_nodes=0, refill=0) -> RenderParams:
    p = RenderParams()
    lib().tpt_render_params_default(C.byref(p))
    p.width, p.height, p.spp, p.max_depth = width, height, spp, max_depth
    p.semantics, p.background, p.sky_scale, p.seed = semantics, background, sky_scale, seed
    p.engine, p.block, p.wave, p.accumulate_fp64 = engine, block, wave, int(bool(fp64))
    p.profile = int(bool(profile))
    p.flat_nodes = flat_nodes
    p.refill = refill
    return p


def quantize(mean_rgb: np.ndarray) -> np.ndarray:
    m = np.ascontiguousarray(mean_rgb, np.float32)
    out = np.zeros(m.shape, np.uint8)
    lib().tpt_quantize(_ptr(m), m.size // 3, _ptr(out))
    return out


def write_ppm(path: str, rgb8: np.ndarray) -> None:
    h, w, _ = rgb8.shape
    check(lib().tpt_write_ppm(path.encode(), _ptr(np.ascontiguousarray(rgb8)), w, h), "write_ppm")


class Mlp:
    """A tensor-core MLP of the learned parts (device buffers via torch)."""

    def __init__(self, in_dim: int, n_hidden: int, out_dim: int, seed: int = 1, device: int = 0):
        h = C.c_void_p()
        check(lib().tpt_mlp_create(device, in_dim, n_hidden, out_dim, seed, C.byref(h)), "mlp_create")
        self._h = h
        self.shape = (in_dim, n_hidden, out_dim)

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.tpt_mlp_destroy(self._h)
            self._h = None

    @property
    def n_params(self) -> int:
        return int(lib().tpt_mlp_param_count(self._h))

    def get_params(self) -> np.ndarray:
        p = np.zeros(self.n_params, np.float32)
        check(lib().tpt_mlp_get_params(self._h, _ptr(p)))
        return p

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, np.float32)
        check(lib().tpt_mlp_set_params(self._h, _ptr(p)))

    def get_grad(self) -> np.ndarray:
        g = np.zeros(self.n_params, np.float32)
        check(lib().tpt_mlp_get_grad(self._h, _ptr(g)))
        return g

    def forward(self, x_f16_ptr: int, rows: int, y_ptr: int) -> None:
        check(lib().tpt_mlp_forward(self._h, C.c_void_p(x_f16_ptr), rows, C.c_void_p(y_ptr), None), "mlp_forward")

    def cache_accumulate(self, q_ptr: int, count: int, lo, extent, accum_ptr: int, n_pixels: int) -> None:
        """tpt_mlp_cache_accumulate: queries (device, count x 6 float4) ->
        accum (device, n_pixels float4) += throughput x max(cache, 0)."""
        lo_a = np.ascontiguousarray(lo, np.float32)
        ext_a = np.ascontiguousarray(extent, np.float32)
        check(lib().tpt_mlp_cache_accumulate(self._h, C.c_void_p(q_ptr), count, _ptr(lo_a), _ptr(ext_a),
                                             C.c_void_p(accum_ptr), n_pixels, None), "mlp_cache_accumulate")

    def backward_given(self, x_f16_ptr: int, dy_ptr: int, rows: int, scale: float = 1.0) -> None:
        check(lib().tpt_mlp_backward_given(self._h, C.c_void_p(x_f16_ptr), C.c_void_p(dy_ptr), rows, scale, None),
              "mlp_backward")

    def backward_vmf(self, x_f16_ptr: int, target_ptr: int, rows: int, scale: float = 1.0) -> float:
        loss = C.c_float()
        check(lib().tpt_mlp_backward_vmf(self._h, C.c_void_p(x_f16_ptr), C.c_void_p(target_ptr), rows, scale,
                                         C.byref(loss), None), "mlp_backward_vmf")
        return loss.value

    def backward_rel_l2(self, x_f16_ptr: int, target_ptr: int, rows: int, scale: float = 1.0) -> float:
        loss = C.c_float()
        check(lib().tpt_mlp_backward_rel_l2(self._h, C.c_void_p(x_f16_ptr), C.c_void_p(target_ptr), rows, scale,
                                            C.byref(loss), None), "mlp_backward_rel_l2")
        return loss.value

    def backward_rel_l2_records(self, rec_ptr: int, count: int, key: int, step: int, lo, extent, rows: int,
                                scale: float = 1.0) -> float:
        loss = C.c_float()
        lo_a = np.ascontiguousarray(lo, np.float32)
        ext_a = np.ascontiguousarray(extent, np.float32)
        check(lib().tpt_mlp_backward_rel_l2_records(self._h, C.c_void_p(rec_ptr), count, key, step, _ptr(lo_a),
                                                    _ptr(ext_a), rows, scale, C.byref(loss), None),
              "mlp_backward_rel_l2_records")
        return loss.value

    def adam(self, lr: float, inv_loss_scale: float = 1.0) -> None:
        check(lib().tpt_mlp_adam(self._h, lr, inv_loss_scale, None), "mlp_adam")


def _encode(fn: str, records: np.ndarray, stride: int, width: int, lo, extent, with_target: bool):
    import torch

    rec = np.ascontiguousarray(records, np.float32).reshape(-1, stride * 4)
    n = len(rec)
    dr = torch.from_numpy(rec).cuda()
    x = torch.empty((n, width), dtype=torch.float16, device="cuda")
    t = torch.empty((n, 4), dtype=torch.float32, device="cuda") if with_target else None
    lo_a = np.ascontiguousarray(lo, np.float32)
    ext_a = np.ascontiguousarray(extent, np.float32)
    torch.cuda.synchronize()
    if fn == "guide":
        st = lib().tpt_guide_encode(C.c_void_p(dr.data_ptr()), n, _ptr(lo_a), _ptr(ext_a), C.c_void_p(x.data_ptr()),
                                    C.c_void_p(t.data_ptr()) if t is not None else None, None)
    else:
        st = lib().tpt_nrc_encode(C.c_void_p(dr.data_ptr()), n, stride, _ptr(lo_a), _ptr(ext_a),
                                  C.c_void_p(x.data_ptr()), None)
    check(st, fn + "_encode")
    torch.cuda.synchronize()
    return x.cpu().numpy(), (t.cpu().numpy() if t is not None else None)


def guide_encode(records: np.ndarray, lo, extent):
    """Path-guiding input rows (f16, n x 112) and loss targets (n x 4) of
    guide records (n x 3 float4) through the C ABI (a CUDA kernel)."""
    return _encode("guide", records, 3, 112, lo, extent, True)


def nrc_encode(records: np.ndarray, lo, extent, stride: int = 5) -> np.ndarray:
    """Radiance-cache input rows (f16, n x 64) of cache records (n x stride
    float4) through the C ABI (a CUDA kernel)."""
    return _encode("nrc", records, stride, 64, lo, extent, False)[0]


def exported_symbols() -> list[str]:
    return list(_SIGS)
