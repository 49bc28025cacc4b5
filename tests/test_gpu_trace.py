"""Closest-hit parity on the GPU: tpt_trace_closest (CUDA traversal) against
the CPU oracle, which is itself pinned bit-exact to the reference
(test_oracle_ref.py / golden fixtures).  Bar: primitive ids bit-exact; t,
uv, point and normal within 1e-5 relative (absolute floor 1e-5 for
components near zero and 2e-4 for points far from the origin)."""
import numpy as np
import pytest

import pyoracle
import tpt
from tpt import scenes

pytestmark = pytest.mark.gpu

RTOL = 1e-5


def _compare(f, i, of, oi, medium_ids=()):
    assert np.array_equal(i, oi), f"id mismatch on {(i != oi).any(axis=1).sum()} rays"
    hit = oi[:, 0] == 1
    # t exact-ish: the float-float sphere root reproduces the double root
    np.testing.assert_allclose(f[hit, 0], of[hit, 0], rtol=RTOL, atol=1e-6)
    geo = hit & ~np.isin(oi[:, 1], list(medium_ids))
    scale = np.maximum(1.0, np.abs(of[geo, 3:6]))
    assert (np.abs(f[geo, 3:6] - of[geo, 3:6]) <= 2e-5 * scale + 1e-5).all(), "hit point"
    fin = np.isfinite(of[geo, 6:9]).all(axis=1)
    n_gpu, n_ora = f[geo][fin, 6:9], of[geo][fin, 6:9]
    assert (np.abs(n_gpu - n_ora) <= 1e-4).all(), "normal"
    uv_ok = np.isfinite(of[geo, 1:3])
    d_uv = np.abs(f[geo, 1:3] - of[geo, 1:3])
    assert (d_uv[uv_ok] <= 1e-4).all(), "uv"


@pytest.mark.parametrize("name", ["cornell", "one_weekend", "cornell_guiding", "ties", "instances", "next_week"])
def test_trace_matches_oracle(ctx, name):
    sd = scenes.PRESETS[name]()
    text = sd.text()
    slot = ctx.upload(tpt.Scene(text))
    ora = pyoracle.Scene(text)
    rays = ora.make_rays(200_000, 11, 0.5, 0.05)
    f, i = ctx.trace_closest(slot, rays, seed=5)
    of, oi = ora.trace(rays, seed=5, media_mode=0)
    med = [int(l.split()[1]) for l in sd.lines if " constant_medium " in l]
    _compare(f, i, of, oi, med)
    ctx.release(slot)


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
