"""allow_bonus_pic snapshots (main.cpp:111-131,192-216): snapshot k is the
running mean of each pixel's first (k+1) * (spp / bonus_pic) samples, and the
final image the mean of all spp; both must equal plain renders with those spp
(same sample streams; float accumulation order differs, rtol 1e-5)."""
import numpy as np
import pytest

import tpt
from tpt import scenes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("spp,bonus", [(20, 4), (22, 4), (9, 9)])
def test_snapshots_equal_partial_renders(ctx, spp, bonus):
    slot = ctx.upload(tpt.Scene(scenes.cornell().text()))
    w, h = 48, 40
    final, snaps, st = tpt.render_snapshots(ctx, slot, w, h, spp, bonus, seed=3, engine=tpt.ENGINE_PERSISTENT)
    assert snaps.shape == (bonus, h, w, 3) and st["samples"] == w * h * spp
    sl = spp // bonus
    for k in range(bonus):
        ref, _ = ctx.render(slot, w, h, (k + 1) * sl, seed=3, engine=tpt.ENGINE_PERSISTENT)
        np.testing.assert_allclose(snaps[k], ref, rtol=1e-5, atol=1e-6)
    ref, _ = ctx.render(slot, w, h, spp, seed=3, engine=tpt.ENGINE_PERSISTENT)
    np.testing.assert_allclose(final, ref, rtol=1e-5, atol=1e-6)
    assert final.max() > 0
    ctx.release(slot)


def test_snapshot_arguments(ctx):
    slot = ctx.upload(tpt.Scene(scenes.cornell().text()))
    with pytest.raises(tpt.TptError):
        tpt.render_snapshots(ctx, slot, 8, 8, 4, 5)   # slice would be 0: the reference divides by zero
    final, snaps, _ = tpt.render_snapshots(ctx, slot, 8, 8, 4, 0)
    assert snaps.shape[0] == 0 and np.isfinite(final).all()
    ctx.release(slot)
