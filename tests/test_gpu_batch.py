"""Batched rendering (one persistent launch over many scenes, replayed from a
CUDA graph) and the autotuner.  The items of a batch agree statistically
with the CPU oracle's renders of their scenes, and an item must equal
tpt_render of the same scene with the same parameters: both draw each
sample from the same counter-based stream, so images differ only by float
accumulation order."""
import numpy as np
import pytest

import tpt
from tpt import scenes

pytestmark = pytest.mark.gpu


def _slots(ctx):
    sds = [scenes.cornell(), scenes.one_weekend(seed=5), scenes.instance_scene(), scenes.next_week(image_size=(64, 32)),
           scenes.cornell_guiding()]
    return [ctx.upload(tpt.Scene(sd.text())) for sd in sds]


def test_batch_items_equal_individual_renders(ctx):
    slots = _slots(ctx)
    jobs = [(slots[0], 40, 30, 8), (slots[1], 17, 23, 16), (slots[2], 32, 32, 4), (slots[3], 24, 24, 8),
            (slots[4], 50, 10, 12), (slots[0], 8, 8, 64)]
    imgs, st = tpt.render_batch(ctx, jobs, max_depth=50, background=tpt.BACKGROUND_SKY, seed=77)
    assert st["samples"] == sum(w * h * s for _, w, h, s in jobs)
    for (slot, w, h, spp), img in zip(jobs, imgs):
        ref, _ = ctx.render(slot, w, h, spp, 50, background=tpt.BACKGROUND_SKY, seed=77,
                            engine=tpt.ENGINE_PERSISTENT)
        np.testing.assert_allclose(img, ref, rtol=1e-5, atol=1e-6)
    # replay of the captured graph gives the same images
    imgs2, _ = tpt.render_batch(ctx, jobs, max_depth=50, background=tpt.BACKGROUND_SKY, seed=77)
    for a, b in zip(imgs, imgs2):
        np.testing.assert_allclose(a, b, rtol=1e-5, atol=1e-6)
    for s in set(slots):
        ctx.release(s)


def test_batch_device_outputs_and_errors(ctx):
    import torch

    slots = _slots(ctx)
    outs = [torch.zeros((16, 16, 3), device="cuda") for _ in range(2)]
    torch.cuda.synchronize()
    jobs = [(slots[0], 16, 16, 4), (slots[1], 16, 16, 4)]
    _, st = tpt.render_batch(ctx, jobs, seed=3, outs=[o.data_ptr() for o in outs])
    imgs, _ = tpt.render_batch(ctx, jobs, seed=3)
    for o, i in zip(outs, imgs):
        np.testing.assert_allclose(o.cpu().numpy(), i, rtol=1e-5, atol=1e-6)
    with pytest.raises(tpt.TptError):
        tpt.render_batch(ctx, [(slots[0] + 100, 8, 8, 1)])
    with pytest.raises(tpt.TptError):
        tpt.render_batch(ctx, [(slots[0], 0, 8, 1)])
    for s in set(slots):
        ctx.release(s)


def test_autotune_picks_a_config_that_auto_renders_use(ctx):
    slot = ctx.upload(tpt.Scene(scenes.cornell().text()))
    eng, block, wave, flat, msps = tpt.autotune(ctx, slot, 120, 120, probe_spp=2)
    assert eng in (tpt.ENGINE_WAVEFRONT, tpt.ENGINE_PERSISTENT) and block in (64, 128, 256) and msps > 0
    a, _ = ctx.render(slot, 40, 40, 8, seed=5, fp64=True)  # engine AUTO -> tuned
    b, _ = ctx.render(slot, 40, 40, 8, seed=5, fp64=True, engine=eng, block=block, wave=wave, flat_nodes=flat)
    np.testing.assert_allclose(a, b, rtol=1e-6, atol=1e-7)
    ctx.release(slot)


def test_batch_autotuner_and_variant_5(ctx):
    import torch

    slots = _slots(ctx)
    jobs = [(slots[0], 40, 30, 16), (slots[1], 17, 23, 16), (slots[3], 24, 24, 8)]
    outs = [torch.empty((h, w, 3), dtype=torch.float32, device="cuda") for _, w, h, _ in jobs]
    block, variant, flat, refill, msps = tpt.autotune_batch(ctx, jobs, [o.data_ptr() for o in outs], spp_divisor=4,
                                                            background=tpt.BACKGROUND_SKY, seed=3)
    assert block in (64, 128) and variant in (4, 5, 6) and flat in (16, 48) and refill == 1 and msps > 0
    # every variant renders the same images (register caps change spills, not arithmetic)
    ref, _ = tpt.render_batch(ctx, jobs, background=tpt.BACKGROUND_SKY, seed=3, block=128, variant=4)
    got, _ = tpt.render_batch(ctx, jobs, background=tpt.BACKGROUND_SKY, seed=3, block=64, variant=5)
    for a, b in zip(ref, got):
        np.testing.assert_allclose(a, b, rtol=1e-5, atol=1e-6)
    for s in set(slots):
        ctx.release(s)


def test_batch_items_match_oracle_renders(ctx):
    """Parity of the batched launch itself against the CPU oracle: three of
    the 64-scene batch's random-sphere scenes (the smallest, a middle and the
    largest sphere count) rendered together in one persistent launch, K runs
    with distinct seeds, each item compared with K oracle renders of its
    scene (per-pixel z statistics and image means, tests/conftest.py
    zcheck)."""
    import pyoracle
    from conftest import zcheck

    sds = scenes.batch_scenes()
    order = sorted(range(len(sds)), key=lambda k: sds[k].meta["n_spheres"])
    pick = [sds[order[0]], sds[order[len(order) // 2]], sds[order[-1]]]
    assert pick[0].meta["n_spheres"] < 200 and pick[-1].meta["n_spheres"] > 4500
    slots = [ctx.upload(tpt.Scene(sd.text())) for sd in pick]
    w = h = 24
    spp, k = 32, 6
    jobs = [(s, w, h, spp) for s in slots]
    runs = [tpt.render_batch(ctx, jobs, max_depth=50, background=tpt.BACKGROUND_SKY, seed=300 + r)[0]
            for r in range(k)]
    for j, sd in enumerate(pick):
        ora = pyoracle.Scene(sd.text())
        ref = np.stack([ora.render(w, h, spp, 50, background=1, seed=600 + r)[0] for r in range(k)])
        mine = np.stack([runs[r][j] for r in range(k)])
        zcheck(mine.astype(np.float64), ref.astype(np.float64))
    for s in slots:
        ctx.release(s)


@pytest.mark.parametrize("refill", [1, 16])
def test_stepped_walk_matches_the_batch_kernel(ctx, refill):
    """Sphere-only batches also run on the stepped-walk kernel (register
    variants 14-16): the same samples, nodes, tests and tie order as the
    whole-segment kernel - for one-BVH scenes (the stepped walk) and for a
    scene whose world is a list (its segments go through trace_closest).
    The shading arithmetic keeps FMA contraction, which ptxas applies per
    kernel, so a scattered direction can differ in its last bit between the
    two kernels and, rarely, a long path then takes another turn (built with
    -fmad=false the two kernels agree on every pixel to summation order,
    measured on a GB300).  The check: equal sample counts, segment counts
    within 0.2 %, and all but 1 % of the pixels equal to summation order."""
    sds = [scenes.one_weekend(seed=5), scenes.batch_scenes(count=3)[2]]
    lst = scenes.SD()
    m = lst.lambertian(lst.const(0.5, 0.5, 0.5))
    lst.world(lst.hlist([lst.sphere((0, -1000, 0), 1000, m), lst.sphere((0, 1, 0), 1, lst.dielectric(1.5)),
                         lst.sphere((2, 1, 0), 1, lst.metal(0.7, 0.6, 0.5, 0.1))]))
    lst.camera((13, 2, 3), (0, 0, 0), (0, 1, 0), 20.0, 1.0, 0.1, 10.0)
    sds.append(lst)
    slots = [ctx.upload(tpt.Scene(sd.text())) for sd in sds]
    jobs = [(slots[0], 40, 30, 8), (slots[1], 33, 17, 12), (slots[2], 24, 24, 6)]
    kw = dict(max_depth=50, background=tpt.BACKGROUND_SKY, seed=21)
    ref, st0 = tpt.render_batch(ctx, jobs, block=64, variant=4, **kw)
    got, st1 = tpt.render_batch(ctx, jobs, block=64, variant=14, refill=refill, **kw)
    assert st0["samples"] == st1["samples"]
    assert abs(st0["segments"] - st1["segments"]) <= 2e-3 * st0["segments"], (st0["segments"], st1["segments"])
    for a, b in zip(got, ref):
        same = np.abs(a - b) <= 1e-5 * np.abs(b) + 1e-6
        assert same.all(axis=2).mean() >= 0.99, same.all(axis=2).mean()
    for s in slots:
        ctx.release(s)


def test_batch_autotuner_offers_the_stepped_walk_for_sphere_scenes(ctx):
    """A sphere-only batch: the autotuner also times the stepped walk (variants
    14-16, 16 or 24 waiting lanes) and its winner renders."""
    import torch

    sds = scenes.batch_scenes(count=4)
    slots = [ctx.upload(tpt.Scene(sd.text())) for sd in sds]
    jobs = [(s, 48, 48, 8) for s in slots]
    outs = [torch.empty((48, 48, 3), dtype=torch.float32, device="cuda") for _ in jobs]
    block, variant, flat, refill, msps = tpt.autotune_batch(ctx, jobs, [o.data_ptr() for o in outs], spp_divisor=2,
                                                            background=tpt.BACKGROUND_SKY, seed=3)
    assert msps > 0 and (variant in (4, 5, 6) or (variant in (14, 15) and refill in (16, 20, 24)))
    imgs, st = tpt.render_batch(ctx, jobs, background=tpt.BACKGROUND_SKY, seed=3, block=block, variant=variant,
                                flat_nodes=flat, refill=refill)
    assert st["samples"] == 4 * 48 * 48 * 8 and all(np.isfinite(i).all() for i in imgs)
    for s in slots:
        ctx.release(s)
