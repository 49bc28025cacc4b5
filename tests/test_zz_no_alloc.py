"""tpt_render_noalloc: the render entry point for callers that cannot allocate
device memory (a plugin whose host owns all GPU memory through its own
pool, real-time loops that must not hit an allocation's implicit
synchronisation).  The caller supplies the scene buffer and the image
buffer; the accumulators live in a fixed device array inside the library.

Checked through the C ABI against tpt_render (persistent engine, same seed,
same parameters) on two calls in a row with different sizes and seeds, so a
second call that did not clear the shared scratch would fail.  Tolerance:
the float accumulation order differs between the two calls' atomics, so
images agree to rtol 1e-5 / atol 1e-6, the tolerance of the other parity
tests."""
import ctypes as C

import numpy as np
import pytest

import tpt
from tpt import scenes

pytestmark = pytest.mark.gpu


def _noalloc(scene, arena, params, out):
    return tpt.lib().tpt_render_noalloc(scene.handle, C.c_void_p(arena.data_ptr()), arena.numel(),
                                        C.byref(params), C.c_void_p(out.data_ptr()), None)


def test_noalloc_matches_render_on_two_calls(ctx):
    import torch

    scene = tpt.Scene(scenes.cornell().text())
    slot = ctx.upload(scene)
    arena = torch.zeros(scene.info()["arena_bytes"], dtype=torch.uint8, device="cuda")
    for (w, h, spp, seed) in [(64, 48, 16, 11), (40, 40, 8, 12)]:
        out = torch.full((h, w, 3), -1.0, dtype=torch.float32, device="cuda")
        p = tpt.make_params(w, h, spp, 50, seed=seed, engine=tpt.ENGINE_PERSISTENT)
        torch.cuda.synchronize()
        assert _noalloc(scene, arena, p, out) == 0, tpt.lib().tpt_last_error()
        got = out.cpu().numpy()
        ref, _ = ctx.render(slot, w, h, spp, 50, seed=seed, engine=tpt.ENGINE_PERSISTENT)
        np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-6)
        assert got.max() > 0
    ctx.release(slot)


def test_noalloc_rejects_oversized_images(built):
    import torch

    scene = tpt.Scene(scenes.cornell().text())
    arena = torch.zeros(scene.info()["arena_bytes"], dtype=torch.uint8, device="cuda")
    out = torch.zeros(16, dtype=torch.float32, device="cuda")
    p = tpt.make_params(1025, 1024, 1, 50)
    assert _noalloc(scene, arena, p, out) == 1
    assert b"TPT_NOALLOC_MAX_PIXELS" in tpt.lib().tpt_last_error()
    small = torch.zeros(16, dtype=torch.uint8, device="cuda")
    assert _noalloc(scene, small, tpt.make_params(8, 8, 1, 50), out) == 1
    assert b"arena" in tpt.lib().tpt_last_error()
    p = tpt.make_params(2, 2, 1, 50)
    p.accumulate_fp64 = 1
    assert _noalloc(scene, arena, p, out) == 1
    assert b"accumulate_fp64" in tpt.lib().tpt_last_error()
    p = tpt.make_params(2, 2, 1, 50, block=96 + 1)
    assert _noalloc(scene, arena, p, out) == 1
    assert b"block" in tpt.lib().tpt_last_error()


def test_noalloc_builds_gpu_bvh_in_the_callers_buffer(ctx):
    """A TPT_BVH_LBVH scene: every call rebuilds the trees on the GPU inside
    the caller's arena buffer; two calls in a row give tpt_render's image of
    the same scene uploaded through the library's own allocations."""
    import torch

    scene = tpt.Scene(scenes.one_weekend().text(), bvh="lbvh")
    slot = ctx.upload(scene)
    arena = torch.zeros(scene.info()["arena_bytes"], dtype=torch.uint8, device="cuda")
    for (w, h, spp, seed) in [(48, 32, 8, 21), (32, 32, 4, 22)]:
        out = torch.full((h, w, 3), -1.0, dtype=torch.float32, device="cuda")
        p = tpt.make_params(w, h, spp, 50, seed=seed, engine=tpt.ENGINE_PERSISTENT, background=tpt.BACKGROUND_SKY)
        torch.cuda.synchronize()
        assert _noalloc(scene, arena, p, out) == 0, tpt.lib().tpt_last_error()
        got = out.cpu().numpy()
        ref, _ = ctx.render(slot, w, h, spp, 50, seed=seed, engine=tpt.ENGINE_PERSISTENT,
                            background=tpt.BACKGROUND_SKY)
        np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-6)
        assert got.max() > 0
    ctx.release(slot)
