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
