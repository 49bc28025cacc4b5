"""Render parity on the GPU.

Statistical: per-pixel means of K GPU renders against K renders of the
REFERENCE (golden fixtures made by running the reference's own sample loop)
and against the CPU oracle: the z-scores of per-pixel mean differences must
look like unit-variance noise, image means must agree within 4 standard
errors, and the relMSE of GPU and reference renders against a high-spp
FP64-accumulated image must agree within 3 sigma.

Deterministic: every camera sample owns a counter-based RNG stream, so the
wavefront and persistent engines, any wave size and any block size give the
same per-sample radiance; with FP64 accumulation their images agree to
rounding of the summation order."""
import os

import numpy as np
import pytest

import pyoracle
import tpt
from tpt import scenes

from conftest import GOLDEN, zcheck as _zcheck

pytestmark = pytest.mark.gpu

EPS = 1e-2  # relMSE denominator epsilon


def relmse(x, ref):
    return float(np.mean((x - ref) ** 2 / (ref * ref + EPS)))


def _sd(name):
    with open(os.path.join(GOLDEN, f"{name}.sd")) as f:
        return f.read()


@pytest.mark.parametrize("name", ["cornell", "cornell_guiding", "metals", "textures", "motion", "media"])
def test_render_matches_reference_renders(ctx, name):
    """Against the reference's own renders: the Cornell boxes, and the
    Cornell room holding metals (fuzz 0, 0.35, a clamped 1.6, a metal box),
    checker / perlin / image textures, moving spheres under a shutter, and
    media (which absorb in the reference's semantics)."""
    g = np.load(os.path.join(GOLDEN, f"{name}_render.npz"))
    ref = g["images"].astype(np.float64)
    w, h, spp, depth, runs = [int(v) for v in g["meta"]]
    slot = ctx.upload(tpt.Scene(_sd(name)))
    mine = np.stack([ctx.render(slot, w, h, spp, max_depth=depth, seed=1000 + k)[0] for k in range(runs)])
    _zcheck(mine.astype(np.float64), ref)
    # converged image: FP64-accumulated, 1024x the spp
    hi, _ = ctx.render(slot, w, h, spp * 1024, max_depth=depth, seed=7, fp64=True)
    hi = hi.astype(np.float64)
    r_gpu = np.array([relmse(m, hi) for m in mine])
    r_ref = np.array([relmse(m, hi) for m in ref])
    se = np.sqrt(r_gpu.var(ddof=1) / runs + r_ref.var(ddof=1) / runs)
    assert abs(r_gpu.mean() - r_ref.mean()) < 3 * se + 1e-6, (r_gpu.mean(), r_ref.mean(), se)
    ctx.release(slot)


@pytest.mark.parametrize("name,semantics,background", [
    ("one_weekend", 0, 1), ("next_week", 0, 0), ("instances", 0, 1), ("cornell", 1, 0), ("next_week", 1, 0)])
def test_render_matches_oracle(ctx, name, semantics, background):
    text = scenes.PRESETS[name]().text()
    slot = ctx.upload(tpt.Scene(text))
    ora = pyoracle.Scene(text)
    w = h = 24
    spp, depth, k = 32, 50, 6
    mine = np.stack([ctx.render(slot, w, h, spp, depth, semantics=semantics, background=background,
                                seed=50 + i)[0] for i in range(k)]).astype(np.float64)
    ref = np.stack([ora.render(w, h, spp, depth, semantics=semantics, background=background,
                               seed=900 + i)[0] for i in range(k)]).astype(np.float64)
    _zcheck(mine, ref)
    ctx.release(slot)


def test_engines_waves_and_blocks_agree(ctx):
    text = scenes.cornell().text()
    slot = ctx.upload(tpt.Scene(text))
    args = dict(width=37, height=23, spp=16, max_depth=50, seed=3, fp64=True)
    a, sa = ctx.render(slot, engine=tpt.ENGINE_WAVEFRONT, **args)
    b, sb = ctx.render(slot, engine=tpt.ENGINE_PERSISTENT, **args)
    c, sc = ctx.render(slot, engine=tpt.ENGINE_WAVEFRONT, wave=96, block=64, **args)
    d, _ = ctx.render(slot, engine=tpt.ENGINE_PERSISTENT, block=64, wave=8, **args)
    e, _ = ctx.render(slot, engine=tpt.ENGINE_WAVEFRONT, block=256, flat_nodes=1, **args)
    np.testing.assert_allclose(a, e, rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(a, b, rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(a, c, rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(a, d, rtol=1e-6, atol=1e-7)
    assert sa["segments"] == sb["segments"] == sc["segments"]
    assert sa["samples"] == 37 * 23 * 16
    ctx.release(slot)


def test_edge_parameters(ctx):
    text = scenes.cornell().text()
    slot = ctx.upload(tpt.Scene(text))
    one, st = ctx.render(slot, 1, 1, 1, max_depth=50, seed=1)
    assert one.shape == (1, 1, 3) and st["samples"] == 1
    # depth 0: only emission at the first hit (utils.cc:65: depth < max_depth fails)
    d0, st0 = ctx.render(slot, 32, 32, 8, max_depth=0, seed=1)
    assert st0["segments"] == 32 * 32 * 8
    # every sample is 15 (camera ray on the light) or 0: pixel means are k*15/8
    assert np.allclose(d0 * 8 / 15.0, np.round(d0 * 8 / 15.0), atol=1e-4)
    assert (d0 == 15.0).any()
    with pytest.raises(tpt.TptError):
        ctx.render(slot, 0, 10, 1)
    with pytest.raises(tpt.TptError):
        ctx.render(slot + 99, 8, 8, 1)
    ctx.release(slot)


def test_nan_samples_are_zeroed(ctx):
    """The reference main's light list holds a sphere; shading points inside
    it give NaN light pdfs (sphere.cc:101-102 guards only the solid angle) and
    NaN directions from sphere::random; de_nan zeroes those samples."""
    sd = scenes.SD()
    wm = sd.lambertian(sd.const(0.5, 0.5, 0.5))
    lm = sd.diffuse_light(sd.const(4, 4, 4))
    floor = sd.rect("xz_rect", -50, 50, -50, 50, 0, wm)
    lamp = sd.flip(sd.rect("xz_rect", -2, 2, -2, 2, 10, lm))
    sd.world(sd.bvh([floor, lamp], 0, 0))
    dummy = sd.lambertian(sd.const(0, 0, 0))
    sd.lights(sd.hlist([sd.rect("xz_rect", -2, 2, -2, 2, 10, dummy), sd.sphere((0, 0, 0), 30, dummy)]))
    sd.camera((0, 5, 20), (0, 0, 0), (0, 1, 0), 60, 1.0, 0.0, 10.0)
    slot = ctx.upload(tpt.Scene(sd.text()))
    img, _ = ctx.render(slot, 16, 16, 16, max_depth=10, seed=2)
    assert np.isfinite(img).all()
    ctx.release(slot)


def test_quantized_output_matches_reference_formula(ctx):
    text = scenes.cornell().text()
    slot = ctx.upload(tpt.Scene(text))
    img, _ = ctx.render(slot, 20, 20, 4, seed=9)
    q = tpt.quantize(img)
    exp = np.clip((255.99 * np.sqrt(img)).astype(np.int64), 0, 255)
    assert np.array_equal(q, exp)
    ctx.release(slot)
