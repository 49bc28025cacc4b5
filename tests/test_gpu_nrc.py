"""Neural radiance cache on the GPU: with the cache never queried the
renderer is the plain tracer (statistically identical images); online
training lowers the cache loss; and the cached render's relMSE against a
high-spp FP64 plain render is below the plain tracer's at equal spp (the
cache trades a small bias for much less variance and shorter paths).  Both
engines (wavefront, persistent) carry the cached renderer."""
import numpy as np
import pytest

import tpt
from tpt import scenes

pytestmark = pytest.mark.gpu
EPS = 1e-2


def relmse(x, ref):
    return float(np.mean((x - ref) ** 2 / (ref * ref + EPS)))


def _slot(ctx):
    return ctx.upload(tpt.Scene(scenes.next_week(image_size=(256, 128)).text()))


@pytest.mark.parametrize("engine", [tpt.ENGINE_WAVEFRONT, tpt.ENGINE_PERSISTENT], ids=["wavefront", "persistent"])
def test_uncached_nrc_render_equals_plain_tracer(ctx, engine):
    slot = _slot(ctx)
    w = h = 24
    k = 6
    a = np.stack([tpt.render_nrc(ctx, slot, w, h, 32, seed=10 + i, passes=2, terminate_depth=1 << 20,
                                 spread_c=0.0, train_steps=4, batch=1024, engine=engine)[0]
                  for i in range(k)]).astype(np.float64)
    b = np.stack([ctx.render(slot, w, h, 32, semantics=tpt.SEMANTICS_PHYSICAL, seed=200 + i)[0]
                  for i in range(k)]).astype(np.float64)
    ma, mb = a.mean(axis=(1, 2, 3)), b.mean(axis=(1, 2, 3))
    se = np.sqrt(ma.var(ddof=1) / k + mb.var(ddof=1) / k)
    assert abs(ma.mean() - mb.mean()) < 4 * se + 1e-7, (ma.mean(), mb.mean(), se)
    ctx.release(slot)


@pytest.mark.parametrize("engine", [tpt.ENGINE_WAVEFRONT, tpt.ENGINE_PERSISTENT], ids=["wavefront", "persistent"])
def test_cache_training_lowers_loss_and_renders(ctx, engine):
    slot = _slot(ctx)
    _, _, n1 = tpt.render_nrc(ctx, slot, 64, 64, 16, passes=2, train_steps=1, batch=8192, seed=3, engine=engine)
    img, st, n2 = tpt.render_nrc(ctx, slot, 64, 64, 16, passes=2, train_steps=300, batch=8192, seed=3,
                                 engine=engine)
    assert n1["records"] > 1000 and n2["queries"] > 0
    assert n2["final_loss"] < n1["final_loss"], (n1, n2)
    assert np.isfinite(img).all() and img.mean() > 0
    ctx.release(slot)


def test_cached_render_gains_at_equal_spp(ctx):
    slot = _slot(ctx)
    w = h = 48
    ref, _ = ctx.render(slot, w, h, 4096, semantics=tpt.SEMANTICS_PHYSICAL, seed=999, fp64=True)
    plain = relmse(ctx.render(slot, w, h, 64, semantics=tpt.SEMANTICS_PHYSICAL, seed=5)[0], ref)
    cached, st, ns = tpt.render_nrc(ctx, slot, w, h, 64, passes=4, train_steps=64, seed=5)
    r = relmse(cached, ref)
    print("relMSE plain", plain, "nrc", r, ns)
    # what the trained cache gains: lower error than the plain tracer at equal spp
    assert r < plain
    ctx.release(slot)


@pytest.mark.parametrize("engine", [tpt.ENGINE_WAVEFRONT, tpt.ENGINE_PERSISTENT], ids=["wavefront", "persistent"])
def test_first_pass_has_its_own_spp(ctx, engine):
    """The uncached first pass takes first_pass_spp samples per pixel and the
    other passes share the rest, rounded up: 5 + 3 x ceil(27 / 3) = 32."""
    slot = _slot(ctx)
    w, h = 40, 24
    for first, passes, spp, total in ((5, 4, 32, 32), (5, 4, 30, 32), (0, 4, 30, 32), (3, 1, 16, 16)):
        _, st, _ = tpt.render_nrc(ctx, slot, w, h, spp, passes=passes, first_pass_spp=first, train_steps=2,
                                  batch=1024, seed=4, engine=engine)
        assert st["samples"] == w * h * total, (first, passes, spp, st["samples"])
    ctx.release(slot)


@pytest.mark.parametrize("engine", [tpt.ENGINE_WAVEFRONT, tpt.ENGINE_PERSISTENT], ids=["wavefront", "persistent"])
def test_path_spread_rule_ends_paths_between_the_fixed_depths(ctx, engine):
    """Paths are a deterministic function of (pixel, sample, depth) draws, so
    the segment counts order exactly.  The spread rule only adds earlier ends
    (at diffuse vertices past the camera hit), so with a huge c it never
    fires (the same segments as with the rule off); with a tiny c it fires
    after every non-specular bounce, so paths are at least as long as with
    terminate_depth 1 and at most as long as with the rule off."""
    slot = _slot(ctx)
    w = h = 48

    def segs(**kw):
        return tpt.render_nrc(ctx, slot, w, h, 16, passes=2, first_pass_spp=4, train_steps=2, batch=1024, seed=6,
                              engine=engine, **kw)[1]["segments"]

    off = segs(terminate_depth=3, spread_c=0.0)
    assert segs(terminate_depth=3, spread_c=1e30) == off
    tiny = segs(terminate_depth=3, spread_c=1e-12)
    one = segs(terminate_depth=1, spread_c=0.0)
    default = segs(terminate_depth=3, spread_c=0.01)
    assert one <= tiny <= default <= off, (one, tiny, default, off)
    assert tiny < off
    ctx.release(slot)


def test_cache_engine_autotune(ctx):
    """tpt_autotune_nrc picks an engine for the slot's cached renders, which
    the next TPT_ENGINE_AUTO cached render uses (an explicit engine still
    wins), and a zero probe is refused."""
    import ctypes as C

    slot = _slot(ctx)
    e = tpt.autotune_nrc(ctx, slot, 48, 48, probe_spp=4)
    assert e in (tpt.ENGINE_WAVEFRONT, tpt.ENGINE_PERSISTENT)
    img, st, ns = tpt.render_nrc(ctx, slot, 48, 48, 16, passes=2, first_pass_spp=4, train_steps=4, batch=1024, seed=2)
    assert np.isfinite(img).all() and ns["queries"] > 0
    p = tpt.make_params(48, 48, 4, 50, tpt.SEMANTICS_PHYSICAL)
    assert tpt.lib().tpt_autotune_nrc(ctx._h, slot, C.byref(p), 0, None) == 1
    ctx.release(slot)


def test_nrc_argument_errors(ctx):
    import ctypes as C

    slot = _slot(ctx)
    img = np.zeros((8, 8, 3), np.float32)
    p = tpt.make_params(8, 8, 4, 50, tpt.SEMANTICS_PHYSICAL)
    for field, bad in (("passes", 0), ("terminate_depth", -1), ("train_stride", 0), ("query_cap", 16),
                       ("batch", 8), ("first_pass_spp", -1), ("first_train_steps", -1), ("spread_c", -1.0),
                       ("spread_c", float("nan"))):
        n = tpt.NrcParams()
        tpt.lib().tpt_nrc_params_default(C.byref(n))
        setattr(n, field, bad)
        assert tpt.lib().tpt_render_nrc(ctx._h, slot, C.byref(p), C.byref(n), img.ctypes.data_as(C.c_void_p),
                                        tpt.TPT_MEM_HOST, None, None) == 1, field
    ctx.release(slot)
