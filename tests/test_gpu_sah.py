"""The alternative topologies - SAH built on the host (TPT_BVH_SAH) and the
linear BVH built on the GPU (TPT_BVH_LBVH): the closest hit of every ray is
the reference's (checked against the CPU oracle, which builds the
reference's own tree) except which primitive wins where several report
exactly the same t - the scene built from coincident primitives ("ties") is
left out - and renders agree with the reference topology's."""
import numpy as np
import pytest

import pyoracle
import tpt
from tpt import scenes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("bvh", ["sah", "lbvh"])
@pytest.mark.parametrize("flat", [0, 1 << 20], ids=["stack", "stackless"])
@pytest.mark.parametrize("name", ["one_weekend", "next_week", "instances", "cornell_guiding"])
def test_closest_hits_match_oracle(ctx, name, flat, bvh):
    sd = scenes.PRESETS[name]()
    text = sd.text()
    ctx.set_flat_nodes(flat)
    slot = ctx.upload(tpt.Scene(text, bvh=bvh))
    ora = pyoracle.Scene(text)
    rays = ora.make_rays(200_000, 21, 0.5, 0.05)
    f, i = ctx.trace_closest(slot, rays, seed=5)
    of, oi = ora.trace(rays, seed=5, media_mode=0)
    ctx.set_flat_nodes(48)
    ctx.release(slot)
    # media draw their free flight from (ray, medium id): independent of the visit order
    assert np.array_equal(i[:, 0], oi[:, 0]), "hit / miss differs"
    hit = oi[:, 0] == 1
    np.testing.assert_allclose(f[hit, 0], of[hit, 0], rtol=1e-5, atol=1e-6)
    # a different primitive only where two primitives report the very same t
    # (boxes standing on the floor, adjacent ground boxes sharing a face):
    # which one wins such a tie is a property of the tree
    differ = hit & (i[:, 1] != oi[:, 1])
    assert (f[differ, 0] == of[differ, 0]).all(), "a primitive differs without a tie in t"
    assert differ.mean() < 1e-2, differ.sum()


@pytest.mark.parametrize("bvh", ["sah", "lbvh"])
def test_render_matches_reference_topology(ctx, bvh):
    sd = scenes.one_weekend()
    a = ctx.upload(tpt.Scene(sd.text()))
    b = ctx.upload(tpt.Scene(sd.text(), bvh=bvh))
    k, w, h = 6, 48, 48
    ra = np.stack([ctx.render(a, w, h, 16, background=tpt.BACKGROUND_SKY, seed=10 + j)[0] for j in range(k)])
    rb = np.stack([ctx.render(b, w, h, 16, background=tpt.BACKGROUND_SKY, seed=10 + j)[0] for j in range(k)])
    # identical sample streams and identical closest hits: images agree up to
    # the float accumulation order
    np.testing.assert_allclose(rb, ra, rtol=1e-4, atol=1e-5)
    ctx.release(a)
    ctx.release(b)
