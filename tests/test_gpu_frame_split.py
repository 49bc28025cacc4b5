"""A frame split by sample ranges on the GPU (tpt_render_range,
tpt_resolve_sums): shares rendered in turn and summed equal the whole
frame's accumulators, because every sample draws from its own (pixel,
sample index) stream; only the float summation order differs."""
import numpy as np
import pytest

import tpt
from tpt import frame_split, scenes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("world", [2, 3])
def test_shares_sum_to_the_whole_frame(ctx, world):
    import torch

    slot = ctx.upload(tpt.Scene(scenes.cornell().text()))
    w, h, spp = 48, 40, 37
    whole = torch.empty(w * h * 4, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    ctx.render_range(slot, w, h, 0, spp, whole.data_ptr(), seed=9)
    total = torch.zeros_like(whole)
    part = torch.empty_like(whole)
    segs = 0
    for r in range(world):
        b, e = frame_split.sample_range(r, world, spp)
        segs += ctx.render_range(slot, w, h, b, e, part.data_ptr(), seed=9)["samples"]
        total += part
    assert segs == w * h * spp
    a, b = total.cpu().numpy(), whole.cpu().numpy()
    np.testing.assert_allclose(a, b, rtol=1e-5, atol=1e-5 * np.abs(b).max())
    # the resolved mean equals tpt_render's frame of the same seed and spp
    img = ctx.resolve_sums(total.data_ptr(), w, h, spp)
    ref, _ = ctx.render(slot, w, h, spp, seed=9, engine=tpt.ENGINE_PERSISTENT)
    np.testing.assert_allclose(img, ref, rtol=1e-5, atol=1e-6)
    ctx.release(slot)


def test_range_arguments(ctx):
    import torch

    slot = ctx.upload(tpt.Scene(scenes.cornell().text()))
    acc = torch.ones(8 * 8 * 4, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    st = ctx.render_range(slot, 8, 8, 5, 5, acc.data_ptr())  # an empty share clears its accumulators
    assert st["samples"] == 0 and float(acc.abs().max()) == 0.0
    with pytest.raises(tpt.TptError):
        ctx.render_range(slot, 8, 8, 6, 5, acc.data_ptr())
    with pytest.raises(tpt.TptError):
        ctx.render_range(slot, 8, 8, 0, 4, acc.data_ptr() + 4)  # not 16-byte aligned
    ctx.release(slot)
