"""The C++ scene front end (include/tpt_scene.hpp): scene code written
against the reference's class names and constructors compiles unchanged,
and a layout drawn with drand_r gets the reference's BVH bit for bit,
because drand_r and bvh_node share the builder's stream as they share the
thread's mt19937 in the reference.  Host code only (g++ + libtpt.so)."""
import os
import subprocess

import numpy as np
import pytest

import tpt

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def frontend_exe(built, tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("fe") / "random_bvh")
    libdir = os.path.dirname(tpt.LIB_PATH)
    cmd = ["g++", "-std=c++14", "-O2", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "frontend", "random_bvh.cc"), "-o", exe, f"-L{libdir}", "-ltpt",
           f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def _run(exe, n):
    r = subprocess.run([exe, str(n)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    return np.array([[float(v) for v in ln.split()] for ln in r.stdout.strip().splitlines()], np.float32)


@pytest.mark.parametrize("n", [1, 2, 7, 500])
def test_frontend_bvh_matches_reference(frontend_exe, n):
    import pyoracle

    ours = _run(frontend_exe, n)
    assert ours.ndim == 2 and ours.shape[1] == 6 and len(ours) >= 1
    if not pyoracle.ref_available():
        pytest.skip("reference harness not built (no reference checkout)")
    ref = pyoracle.ref_frontend_bvh(n)
    np.testing.assert_array_equal(ours, ref)


def test_frontend_is_deterministic(frontend_exe):
    np.testing.assert_array_equal(_run(frontend_exe, 50), _run(frontend_exe, 50))


# The reference's own scene functions (src/utils.cc): every function that
# builds a scene, cut from the file between the first and the last of them,
# minus the perlin_noise definitions in between (the front end has no host
# perlin class; its perlin_noise_texture draws the same tables).
SCENE_FUNCTIONS = ["random_scene", "two_checker_spheres", "two_perlin_spheres", "light_spheres",
                   "sphere_cornell_box", "cornell_box", "cornell_box_smoke", "oneweek_final"]


def _cut_scene_functions(utils_cc: str) -> str:
    lines = utils_cc.splitlines()

    def start(sig):
        return next(i for i, l in enumerate(lines) if l.startswith(sig))

    def end_of(i):
        return next(j for j in range(i, len(lines)) if lines[j] == "}")

    a = start("hitable *random_scene()")
    b = start("std::array<vec3, 256> perlin_noise::random_vec3_")
    c = start("hitable *two_perlin_spheres()")
    d = end_of(start("hitable *oneweek_final()"))
    return "\n".join(lines[a:b] + lines[c:d + 1]) + "\n"


@pytest.fixture(scope="module")
def reference_scenes_exe(built, tmp_path_factory):
    import pyoracle

    ref = pyoracle.reference_dir() if pyoracle.ref_available() else None
    if ref is None:
        pytest.skip("no reference checkout (the harness records where it was built from)")
    d = tmp_path_factory.mktemp("refscenes")
    with open(os.path.join(ref, "src", "utils.cc")) as f:
        (d / "reference_scene_functions.inc").write_text(_cut_scene_functions(f.read()))
    exe = str(d / "reference_scenes")
    libdir = os.path.dirname(tpt.LIB_PATH)
    cmd = ["g++", "-std=c++14", "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"), "-I", str(d),
           os.path.join(ROOT, "tests", "frontend", "reference_scenes.cc"), "-o", exe, f"-L{libdir}", "-ltpt",
           f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def _trees(exe, name):
    r = subprocess.run([exe, name], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    trees, cur = [], None
    for ln in r.stdout.splitlines():
        f = ln.split()
        if f[0] == "tree":
            cur = []
            trees.append(cur)
        else:
            cur.append([float(v) for v in f])
    return [(np.array(t, np.float32)[:, :6], np.array(t)[:, 6:].astype(np.int32)) for t in trees]


@pytest.mark.parametrize("name", SCENE_FUNCTIONS)
def test_reference_scene_functions_compile_and_give_reference_bvhs(reference_scenes_exe, name):
    """The reference's scene functions (utils.cc:96-154,226-414), compiled
    unchanged against tpt_scene.hpp (vec3 arithmetic, drand_r, the scene
    classes; stbi_load replaced by a stand-in image), build and compile into
    a GPU scene; every bvh_node they create has the reference's topology and
    boxes node for node, including the trees built after perlin textures and
    moving spheres have consumed the drand_r stream."""
    import pyoracle

    ours = _trees(reference_scenes_exe, name)
    ref = pyoracle.ref_scene_function_bvhs(name)
    assert len(ours) == len(ref)
    for (ob, ok), (rb, rk) in zip(ours, ref):
        np.testing.assert_array_equal(ok, rk)
        np.testing.assert_array_equal(ob, rb)
