"""Closest-hit parity on the GPU: tpt_trace_closest (CUDA traversal) against
the CPU oracle, which is itself pinned bit-exact to the reference
(test_oracle_golden.py / golden fixtures), and against the reference's own
hit records.  Bar: primitive ids bit-exact; t, point, normal and uv within
1e-5 relative.  Floors for components near zero: a point component is
measured against max(|p|, 1), a normal component against the normal's
length, and u, v (in [0, 1]) get an absolute floor of 1e-6 (eight ulps at
1.0; the device's atan2f / asinf differ from the host's by an ulp or two).
Measured on a GB300 over 200k rays per scene: ids, points and normals are
bit-identical, t differs in the last bit on a few instanced or medium hits,
u and v differ by at most 1.2e-7."""
import numpy as np
import pytest

import pyoracle
import tpt
from tpt import scenes

pytestmark = pytest.mark.gpu

RTOL = 1e-5
SCENES = ["cornell", "one_weekend", "cornell_guiding", "ties", "instances", "next_week",
          "metals", "textures", "motion", "media"]


def _compare(f, i, of, oi, medium_ids=()):
    assert np.array_equal(i, oi), f"id mismatch on {(i != oi).any(axis=1).sum()} rays"
    hit = oi[:, 0] == 1
    # t: the float-float sphere root reproduces the double root
    np.testing.assert_allclose(f[hit, 0], of[hit, 0], rtol=RTOL, atol=0)
    geo = hit & ~np.isin(oi[:, 1], list(medium_ids))
    p_gpu, p_ora = f[geo, 3:6], of[geo, 3:6]
    assert (np.abs(p_gpu - p_ora) <= RTOL * np.maximum(1.0, np.abs(p_ora))).all(), "hit point"
    fin = np.isfinite(of[geo, 6:9]).all(axis=1)
    n_gpu, n_ora = f[geo][fin, 6:9], of[geo][fin, 6:9]
    n_len = np.linalg.norm(n_ora, axis=1, keepdims=True)
    assert (np.abs(n_gpu - n_ora) <= RTOL * n_len).all(), "normal"
    uv_ok = np.isfinite(of[geo, 1:3])
    d_uv = np.abs(f[geo, 1:3] - of[geo, 1:3])
    assert (d_uv[uv_ok] <= RTOL * np.abs(of[geo, 1:3])[uv_ok] + 1e-6).all(), "uv"


@pytest.mark.parametrize("flat", [0, 48, 1 << 20], ids=["stack", "auto", "stackless"])
@pytest.mark.parametrize("name", SCENES)
def test_trace_matches_oracle(ctx, name, flat):
    sd = scenes.PRESETS[name]()
    text = sd.text()
    ctx.set_flat_nodes(flat)
    slot = ctx.upload(tpt.Scene(text))
    ora = pyoracle.Scene(text)
    rays = ora.make_rays(200_000, 11, 0.5, 0.05)
    f, i = ctx.trace_closest(slot, rays, seed=5)
    of, oi = ora.trace(rays, seed=5, media_mode=0)
    med = [int(l.split()[1]) for l in sd.lines if " constant_medium " in l]
    _compare(f, i, of, oi, med)
    ctx.release(slot)
    ctx.set_flat_nodes(48)


def test_trace_one_million_rays_one_weekend(ctx):
    """The 10^6-ray parity batch: 50% camera rays of the one-weekend camera,
    50% random rays (origins in the scene box, 5% axis-parallel)."""
    sd = scenes.one_weekend()
    text = sd.text()
    slot = ctx.upload(tpt.Scene(text))
    ora = pyoracle.Scene(text)
    rays = ora.make_rays(1_000_000, 1234, 0.5, 0.05)
    f, i = ctx.trace_closest(slot, rays)
    of, oi = ora.trace(rays)
    _compare(f, i, of, oi)
    assert oi[:, 0].sum() > 400_000
    ctx.release(slot)


@pytest.mark.parametrize("name", SCENES)
def test_trace_matches_reference_golden(ctx, name):
    """GPU closest hits against the reference's own outputs (golden fixtures).
    A constant_medium draws its free-flight distance from drand_r inside
    hit() (hitable.cc:116), which the GPU replaces by a Philox draw, so in
    scenes with media only the rays whose answer does not depend on that draw
    are compared: those where the oracle gives the same record with the
    reference's mt19937 stream and with the Philox draws."""
    import os
    from conftest import GOLDEN
    with open(os.path.join(GOLDEN, f"{name}.sd")) as fh:
        text = fh.read()
    g = np.load(os.path.join(GOLDEN, f"{name}_trace.npz"))
    slot = ctx.upload(tpt.Scene(text))
    f, i = ctx.trace_closest(slot, g["rays"])
    keep = np.ones(len(i), bool)
    if " constant_medium " in text:
        ora = pyoracle.Scene(text)
        f0, i0 = ora.trace(g["rays"], media_mode=0)
        f1, i1 = ora.trace(g["rays"], media_mode=1)
        keep = (i0 == i1).all(axis=1) & (f0[:, 0].view(np.uint32) == f1[:, 0].view(np.uint32))
        assert keep.mean() > 0.8
    _compare(f[keep], i[keep], g["hit_f"][keep], g["hit_i"][keep])
    ctx.release(slot)


def test_trace_device_pointers(ctx):
    import torch
    sd = scenes.cornell()
    text = sd.text()
    slot = ctx.upload(tpt.Scene(text))
    ora = pyoracle.Scene(text)
    rays = ora.make_rays(10_000, 3, 0.5, 0.05)
    dr = torch.from_numpy(rays).cuda()
    hf = torch.empty((10_000, 9), dtype=torch.float32, device="cuda")
    hi = torch.empty((10_000, 2), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    ctx.trace_closest_device(slot, dr.data_ptr(), 10_000, 0, hf.data_ptr(), hi.data_ptr())
    f, i = ctx.trace_closest(slot, rays)
    assert np.array_equal(hi.cpu().numpy(), i)
    assert np.array_equal(hf.cpu().numpy().view(np.uint32), f.view(np.uint32))
    ctx.release(slot)


def _in_rect_plane(sd, rays):
    """Rays whose origin lies on the plane of a rect or box face of the
    scene with the direction parallel to it: the reference computes t = 0/0
    = NaN there and the NaN then steers its comparisons (a NaN t_max accepts
    any later hit), so the winner depends on the order of its recursive
    calls; the flattened GPU traversal rejects NaN hits instead (a known,
    documented divergence)."""
    axis_of = {"xy_rect": 2, "xz_rect": 1, "yz_rect": 0}
    planes = []
    for l in sd.lines:
        f = l.split()
        if len(f) > 2 and f[2] in axis_of:
            planes.append((axis_of[f[2]], float(f[7])))
        elif len(f) > 2 and f[2] == "box":
            for a in range(3):
                planes += [(a, float(f[3 + a])), (a, float(f[6 + a]))]
    o, d = rays[:, 0:3], rays[:, 3:6]
    m = np.zeros(len(rays), bool)
    for a, k in planes:
        m |= (o[:, a] == np.float32(k)) & (d[:, a] == 0)
    return m


@pytest.mark.parametrize("flat", [0, 1 << 20], ids=["stack", "stackless"])
@pytest.mark.parametrize("name", ["cornell", "one_weekend", "instances", "next_week", "metals", "textures"])
def test_trace_edge_rays(ctx, name, flat):
    """The known-answer edge rays (tests/golden/<scene>_edge.npz, frozen from
    the reference; the oracle reproduces them bit for bit on the CPU):
    tangent and near-tangent rays, rays from sphere surfaces, rect and box
    edges and corners.  Compared with the oracle in the GPU's medium mode
    (free flight from (ray, medium)), except the rays lying in a rect's
    plane (_in_rect_plane)."""
    import os

    g = np.load(os.path.join(os.path.dirname(__file__), "golden", f"{name}_edge.npz"))
    sd = scenes.PRESETS[name]()
    text = sd.text()
    ctx.set_flat_nodes(flat)
    slot = ctx.upload(tpt.Scene(text))
    f, i = ctx.trace_closest(slot, g["rays"], seed=5)
    ctx.release(slot)
    ctx.set_flat_nodes(48)
    of, oi = pyoracle.Scene(text).trace(g["rays"], seed=5, media_mode=0)
    med = [int(l.split()[1]) for l in sd.lines if " constant_medium " in l]
    keep = ~_in_rect_plane(sd, g["rays"])
    assert keep.sum() > 0.6 * len(keep)
    _compare(f[keep], i[keep], of[keep], oi[keep], med)
