"""The CPU oracle against golden vectors produced by the reference itself
(tests/golden/gen_golden.py runs the reference's own sources).  Bit-exact
for closest hits and BVH topology; statistical for renders."""
import os

import numpy as np
import pytest

import pyoracle
from tpt import scenes

from conftest import GOLDEN, zcheck

SCENES = ["cornell", "one_weekend", "cornell_guiding", "ties", "instances", "next_week",
          "metals", "textures", "motion", "media"]
RENDERS = ["cornell", "cornell_guiding", "metals", "textures", "motion", "media"]


def _sd(name):
    with open(os.path.join(GOLDEN, f"{name}.sd")) as f:
        return f.read()


@pytest.mark.parametrize("name", SCENES)
def test_generators_reproduce_golden_scene_text(name):
    assert scenes.PRESETS[name]().text() == _sd(name)


@pytest.mark.parametrize("name", SCENES)
def test_oracle_bvh_topology_equals_reference(built, name):
    g = np.load(os.path.join(GOLDEN, f"{name}_bvh.npz"))
    ora = pyoracle.Scene(_sd(name))
    ids = sorted({int(k.split("_")[1]) for k in g.files})
    assert ids
    for b in ids:
        boxes, kids = ora.bvh_dump(b)
        assert np.array_equal(kids, g[f"kids_{b}"]), f"bvh {b} children"
        assert np.array_equal(boxes.view(np.uint32), g[f"boxes_{b}"].view(np.uint32)), f"bvh {b} boxes"


@pytest.mark.parametrize("name", SCENES)
def test_oracle_closest_hit_bit_exact(built, name):
    g = np.load(os.path.join(GOLDEN, f"{name}_trace.npz"))
    ora = pyoracle.Scene(_sd(name))
    f, i = ora.trace(g["rays"], media_mode=1)  # the reference's drand_r order for media
    assert np.array_equal(i, g["hit_i"])
    assert np.array_equal(f.view(np.uint32), g["hit_f"].view(np.uint32))


def test_golden_covers_edge_cases():
    """The fixtures hold misses, hits, axis-parallel rays and exact ties."""
    g = np.load(os.path.join(GOLDEN, "ties_trace.npz"))
    hit = g["hit_i"][:, 0] == 1
    assert 0 < hit.sum() < len(hit)
    rays = np.load(os.path.join(GOLDEN, "cornell_trace.npz"))["rays"]
    assert ((rays[:, 3:6] == 0).any(axis=1)).sum() > 10


def test_ties_known_answers(built):
    """Exact ties: coincident spheres in a BVH -> the right child (hitable.cc:71);
    coincident spheres in a list -> the earlier (strict '<'); coincident rects
    in a list -> the later (t may equal t_max)."""
    sd = scenes.tie_scene()
    ora = pyoracle.Scene(sd.text())
    rays = np.array([[0, 0, 5, 0, 0, -1, 0], [3, 0, 5, 0, 0, -1, 0], [-6, 0, 5, 0, 0, -1, 0]], np.float32)
    f, i = ora.trace(rays)
    bvh_root = 2  # node ids: 0,1 spheres in the BVH, 2 the BVH
    boxes, kids = ora.bvh_dump(bvh_root)
    right_child = -(kids[0, 1] + 1)
    assert i[0, 1] == right_child
    assert i[1, 1] == 3   # earlier of the list pair (nodes 3, 4)
    assert i[2, 1] == 7   # later of the rect pair (nodes 6, 7)
    if pyoracle.ref_available():
        rf, ri = pyoracle.RefScene(sd.text()).trace(rays)
        assert np.array_equal(ri, i)


@pytest.mark.parametrize("name", RENDERS)
def test_oracle_render_matches_reference_statistics(built, name):
    """Oracle renders against the reference's renders at the same resolution
    and spp: the image means agree within 4 sigma of the reference's run to
    run spread, and per-pixel means agree in a chi-square sense."""
    g = np.load(os.path.join(GOLDEN, f"{name}_render.npz"))
    ref = g["images"].astype(np.float64)
    w, h, spp, depth, runs = [int(v) for v in g["meta"]]
    ora = pyoracle.Scene(_sd(name))
    mine = np.stack([ora.render(w, h, spp, depth, seed=100 + k)[0] for k in range(runs)]).astype(np.float64)
    m_ref = ref.mean(axis=(1, 2, 3))
    m_ora = mine.mean(axis=(1, 2, 3))
    se = np.sqrt(m_ref.var(ddof=1) / runs + m_ora.var(ddof=1) / runs)
    assert abs(m_ref.mean() - m_ora.mean()) < 4 * se + 1e-6, (m_ref.mean(), m_ora.mean(), se)
    # per pixel: difference of run means over its standard error
    zcheck(mine, ref)


@pytest.mark.parametrize("name", ["cornell", "one_weekend", "instances", "next_week", "metals", "textures"])
def test_oracle_edge_rays_match_reference(built, name):
    """Known-answer rays at the edges of the primitives' arithmetic
    (tangent and near-tangent to spheres, from sphere surfaces, at rect and
    box edges and corners, axis-parallel through rect edges - where the
    reference's 0/0 gives t = NaN), frozen from the reference itself: the
    oracle reproduces every result bit for bit."""
    g = np.load(os.path.join(GOLDEN, f"{name}_edge.npz"))
    ora = pyoracle.Scene(_sd(name))
    f, i = ora.trace(g["rays"], media_mode=1, nthreads=1)  # the reference's drand_r order for media
    assert np.array_equal(i, g["hit_i"])
    hit = g["hit_i"][:, 0] == 1
    assert np.array_equal(f[hit], g["hit_f"][hit], equal_nan=True)
