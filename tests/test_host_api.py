"""Host-side checks that need no GPU: the C-ABI library loads and exports
every symbol include/tpt.h declares, the scene compiler reproduces the
reference's BVH topology, scene-text errors come back as status codes, the
builder API mirrors the reference constructors, and the output helpers
follow main.cpp's quantisation and PPM format."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import pyoracle
import tpt
from tpt import scenes

from conftest import GOLDEN, ROOT

SCENES = ["cornell", "one_weekend", "cornell_guiding", "ties", "instances", "next_week"]


def _sd(name):
    with open(os.path.join(GOLDEN, f"{name}.sd")) as f:
        return f.read()


def _header_symbols():
    with open(os.path.join(ROOT, "include", "tpt.h")) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(tpt_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(built):
    L = tpt.lib()
    declared = _header_symbols()
    assert len(declared) >= 40
    for name in declared:
        assert hasattr(L, name), name
    assert set(declared) <= set(tpt.exported_symbols()) | set(declared)
    assert tpt.lib().tpt_version().decode().startswith("tpt-gb300")


@pytest.mark.parametrize("name", SCENES)
def test_product_bvh_topology_equals_reference(built, name):
    g = np.load(os.path.join(GOLDEN, f"{name}_bvh.npz"))
    sc = tpt.Scene(_sd(name))
    for b in sorted({int(k.split("_")[1]) for k in g.files}):
        boxes, kids = sc.bvh_dump(b)
        assert np.array_equal(kids, g[f"kids_{b}"])
        assert np.array_equal(boxes.view(np.uint32), g[f"boxes_{b}"].view(np.uint32))


@pytest.mark.parametrize("seed", [2, 3, 4])
def test_product_bvh_topology_equals_oracle_on_random_scenes(built, seed):
    for n in (50, 333, 5000):
        sd = scenes.one_weekend(seed=seed, grid=(-40, 40), n_small=n - 4)
        text = sd.text()
        root = [int(l.split()[1]) for l in sd.lines if " bvh_node " in l][0]
        pb, pk = tpt.Scene(text).bvh_dump(root)
        ob, ok = pyoracle.Scene(text).bvh_dump(root)
        assert np.array_equal(pk, ok) and np.array_equal(pb.view(np.uint32), ob.view(np.uint32))


def test_scene_info(built):
    info = tpt.Scene(_sd("next_week")).info()
    assert info["n_blas"] == 1 and info["n_items"] == 9 and info["max_stack"] <= 32
    assert info["arena_bytes"] > 6 * 2**20  # the 2048x1024 RGB8 texture lives in the arena


@pytest.mark.parametrize("text,code", [
    ("tex 0 const 1 1 1\nmat 0 lambertian 0\nnode 0 sphere 0 0 0 1 7\nworld 0\n", 2),   # undefined material
    ("node 0 bogus 1 2 3\n", 2),                                                          # unknown statement
    ("tex 0 const 1 1 1\nmat 0 lambertian 0\nnode 0 sphere 0 0 zz 1 0\nworld 0\n", 2),  # bad number
    ("tex 0 const 1 1 1\nmat 0 lambertian 0\nnode 0 sphere 0 0 0 1 0\n", 1),            # no world
])
def test_scene_text_errors_are_status_codes(built, text, code):
    with pytest.raises(tpt.TptError) as e:
        tpt.Scene(text + "camera 0 0 1 0 0 0 0 1 0 90 1 0 1 0 0\n")
    assert e.value.status == code


def test_unsupported_shapes_are_reported(built):
    text = ("tex 0 const 1 1 1\nmat 0 lambertian 0\nnode 0 sphere 0 0 0 1 0\nnode 1 sphere 3 0 0 1 0\n"
            "node 2 hitable_list 2 0 1\nnode 3 sphere 6 0 0 1 0\nnode 4 bvh_node 0 0 2 2 3\nworld 4\n"
            "camera 0 0 9 0 0 0 0 1 0 90 1 0 1 0 0\n")
    with pytest.raises(tpt.TptError) as e:
        tpt.Scene(text)
    assert e.value.status == 3  # a hitable_list below a bvh_node


def test_builder_api_mirrors_reference_constructors(built):
    """Cornell box built through the C entry points (as a C/C++ caller would)
    compiles to the same BVH as the scene text."""
    L = tpt.lib()
    b = C.c_void_p()
    assert L.tpt_builder_create(C.byref(b)) == 0
    red = L.tpt_lambertian(b, L.tpt_constant_texture(b, 0.65, 0.05, 0.05))
    white = L.tpt_lambertian(b, L.tpt_constant_texture(b, 0.73, 0.73, 0.73))
    green = L.tpt_lambertian(b, L.tpt_constant_texture(b, 0.12, 0.45, 0.15))
    light = L.tpt_diffuse_light(b, L.tpt_constant_texture(b, 15, 15, 15))
    items = [
        L.tpt_flip_normal(b, L.tpt_yz_rect(b, 0, 555, 0, 555, 555, green)),
        L.tpt_yz_rect(b, 0, 555, 0, 555, 0, red),
        L.tpt_flip_normal(b, L.tpt_xz_rect(b, 213, 343, 227, 332, 554, light)),
        L.tpt_flip_normal(b, L.tpt_xz_rect(b, 0, 555, 0, 555, 555, white)),
        L.tpt_xz_rect(b, 0, 555, 0, 555, 0, white),
        L.tpt_flip_normal(b, L.tpt_xy_rect(b, 0, 555, 0, 555, 555, white)),
        L.tpt_translate(b, L.tpt_rotate_y(b, L.tpt_box(b, 0, 0, 0, 165, 330, 165, white), 15.0), 265, 0, 295),
        L.tpt_sphere(b, 190, 90, 190, 90, L.tpt_dielectric(b, 1.5)),
    ]
    assert min(items) >= 0
    arr = (C.c_int32 * len(items))(*items)
    world = L.tpt_bvh_node(b, arr, len(items), 0.0, 0.0)
    assert world >= 0
    assert L.tpt_builder_set_world(b, world) == 0
    f3 = C.c_float * 3
    assert L.tpt_builder_set_camera(b, f3(278, 278, -800), f3(278, 278, 0), f3(0, 1, 0), 40, 1, 0, 10, 0, 0) == 0
    sc = C.c_void_p()
    assert L.tpt_scene_compile(b, C.byref(sc)) == 0
    n = L.tpt_scene_bvh_dump(sc, world, None, None, 0)
    kids = np.zeros((n, 2), np.int32)
    boxes = np.zeros((n, 6), np.float32)
    L.tpt_scene_bvh_dump(sc, world, boxes.ctypes.data_as(C.c_void_p), kids.ctypes.data_as(C.c_void_p), n)
    g = np.load(os.path.join(GOLDEN, "cornell_bvh.npz"))
    assert np.array_equal(boxes.view(np.uint32), g["boxes_14"].view(np.uint32))
    # leaf ids differ (builder handles vs scene-text ids) but the shape is the same
    assert np.array_equal(kids >= 0, g["kids_14"] >= 0)
    L.tpt_scene_destroy(sc)
    L.tpt_builder_destroy(b)


def test_bvh_of_boxless_items_reports_status(built):
    L = tpt.lib()
    b = C.c_void_p()
    L.tpt_builder_create(C.byref(b))
    m = L.tpt_lambertian(b, L.tpt_constant_texture(b, 1, 1, 1))
    empty = L.tpt_hitable_list(b, None, 0)   # hitable_list::bounding_box is false when empty
    s = L.tpt_sphere(b, 0, 0, 0, 1, m)
    arr = (C.c_int32 * 3)(s, empty, s)
    assert L.tpt_bvh_node(b, arr, 3, 0.0, 0.0) == -4  # where the reference calls exit(-1)
    assert L.tpt_sphere(b, 0, 0, 0, 1, 99) == -10     # bad material handle
    L.tpt_builder_destroy(b)


def test_metal_fuzz_clamp_matches_reference(built):
    """metal clamps fuzz outside [0,1) to 1 (material.h:41-46); both scene
    loaders must agree, so the same text gives the same traced image."""
    text = ("tex 0 const 1 1 1\nmat 0 metal 0.8 0.8 0.9 10.0\nnode 0 sphere 0 0 0 1 0\nworld 0\n"
            "camera 0 0 5 0 0 0 0 1 0 40 1 0 5 0 0\n")
    assert tpt.Scene(text).info()["n_materials"] == 1


def test_no_device_is_an_error_not_a_fallback(built):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(tpt.TptError) as e:
        tpt.Context(0)
    assert e.value.status == 9


def test_quantize_matches_reference_formula(built):
    rng = np.random.default_rng(0)
    m = rng.uniform(-0.5, 2.0, size=(7, 9, 3)).astype(np.float32)
    m[0, 0, 0] = np.nan
    q = tpt.quantize(m)
    qo = pyoracle.quantize(m)
    exp = np.clip((255.99 * np.sqrt(np.maximum(m[1:], 0))).astype(np.int64), 0, 255)
    assert np.array_equal(q, qo)
    assert np.array_equal(q[1:], exp)


def test_write_ppm_format(built, tmp_path):
    img = np.arange(2 * 3 * 3, dtype=np.uint8).reshape(2, 3, 3)
    p = str(tmp_path / "img.ppm")
    tpt.write_ppm(p, img)
    with open(p) as f:
        lines = f.read().splitlines()
    assert lines[0] == "P3" and lines[1] == "3 2" and lines[2] == "255"
    assert lines[3].split() == ["0", "1", "2"] and len(lines) == 3 + 6


def test_status_strings(built):
    L = tpt.lib()
    assert L.tpt_status_string(0) == b"ok"
    assert b"bounding box" in L.tpt_status_string(4)
