"""Checkpoint and resume of the learned parts (tpt_learned_save /
tpt_learned_load, warm_start): a saved network (weights, Adam moments, step
count) loads bit for bit into another context; a guide restored from a
checkpoint guides from the first pass, so a one-pass render has a lower
error than the plain tracer at equal spp; a restored radiance cache is
queried from the first pass, which shortens the paths."""
import numpy as np
import pytest

import tpt
from tpt import scenes

pytestmark = pytest.mark.gpu

EPS = 1e-2


def relmse(x, ref):
    return float(np.mean((x - ref) ** 2 / (ref * ref + EPS)))


def test_save_needs_a_trained_network(built):
    ctx = tpt.Context(0)
    with pytest.raises(tpt.TptError) as e:
        tpt.learned_save(ctx, tpt.NET_GUIDE)
    assert e.value.status == 10  # TPT_ERR_BAD_HANDLE
    with pytest.raises(tpt.TptError):
        tpt.learned_load(ctx, tpt.NET_CACHE, np.zeros(7, np.float32))  # wrong size
    with pytest.raises(tpt.TptError) as e:  # and the failed load left no network behind
        tpt.learned_save(ctx, tpt.NET_CACHE)
    assert e.value.status == 10
    ctx.close()


@pytest.mark.parametrize("which", [tpt.NET_GUIDE, tpt.NET_CACHE], ids=["guide", "cache"])
def test_checkpoint_round_trip(built, which):
    a, b = tpt.Context(0), tpt.Context(0)
    sd = scenes.cornell_guiding() if which == tpt.NET_GUIDE else scenes.next_week()
    slot = a.upload(tpt.Scene(sd.text()))
    if which == tpt.NET_GUIDE:
        tpt.render_guided(a, slot, 32, 32, 32, passes=4, train_steps=8, batch=4096, seed=3)
    else:
        tpt.render_nrc(a, slot, 32, 32, 16, passes=4, train_steps=8, batch=4096, seed=3)
    state = tpt.learned_save(a, which)
    assert np.isfinite(state).all() and state[-1] > 0  # Adam steps taken
    tpt.learned_load(b, which, state)
    again = tpt.learned_save(b, which)
    assert np.array_equal(state.view(np.uint32), again.view(np.uint32))
    a.close()
    b.close()


def test_warm_guide_guides_from_the_first_pass(ctx):
    slot = ctx.upload(tpt.Scene(scenes.cornell_guiding().text()))
    w = h = 64
    ref, _ = ctx.render(slot, w, h, 16384, semantics=tpt.SEMANTICS_PHYSICAL, seed=999, fp64=True)
    tpt.render_guided(ctx, slot, w, h, 256, seed=7, passes=8, train_steps=32)
    state = tpt.learned_save(ctx, tpt.NET_GUIDE)
    other = tpt.Context(0)
    s2 = other.upload(tpt.Scene(scenes.cornell_guiding().text()))
    plain, warm = [], []
    for i in range(4):
        plain.append(relmse(other.render(s2, w, h, 256, semantics=tpt.SEMANTICS_PHYSICAL, seed=50 + i)[0], ref))
        tpt.learned_load(other, tpt.NET_GUIDE, state)
        # one pass: every sample is guided by the restored network
        warm.append(relmse(tpt.render_guided(other, s2, w, h, 256, seed=50 + i, passes=1, warm_start=1)[0], ref))
    print("relMSE plain", plain, "warm", warm)
    # medians: at 64x64 a single rare light path can dominate one image's relMSE
    assert np.median(warm) < 0.9 * np.median(plain)
    other.close()
    ctx.release(slot)


def test_warm_cache_is_queried_from_the_first_pass(ctx):
    slot = ctx.upload(tpt.Scene(scenes.next_week().text()))
    w = h = 64
    tpt.render_nrc(ctx, slot, w, h, 64, seed=7)
    state = tpt.learned_save(ctx, tpt.NET_CACHE)
    other = tpt.Context(0)
    s2 = other.upload(tpt.Scene(scenes.next_week().text()))
    img_c, st_c, ns_c = tpt.render_nrc(other, s2, w, h, 32, seed=5, passes=1)
    tpt.learned_load(other, tpt.NET_CACHE, state)
    img_w, st_w, ns_w = tpt.render_nrc(other, s2, w, h, 32, seed=5, passes=1, warm_start=1)
    assert ns_c["queries"] == 0 and ns_w["queries"] > 0
    assert st_w["segments"] < 0.8 * st_c["segments"]
    assert np.isfinite(img_w).all()
    assert abs(img_w.mean() - img_c.mean()) < 0.2 * img_c.mean()
    other.close()
    ctx.release(slot)
