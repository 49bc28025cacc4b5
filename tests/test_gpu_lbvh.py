"""The GPU linear-BVH builder (TPT_BVH_LBVH, csrc/lbvh.cu) against its CPU
restatement in the oracle (oracle/lbvh.cc): node boxes, children, skip
indices and depth bit for bit, on box sets that exercise the shared-memory
sort (up to 16384 keys) and the global-memory sort above it, identical
boxes, a flat layout, a huge outlier and one or two primitives.  The
scene-level closest-hit parity of LBVH scenes is in tests/test_gpu_sah.py;
here also: the no-allocation entry point builds the same trees as
tpt_scene_upload, and a batch of LBVH scenes renders as the reference
topology does."""
import ctypes as C

import numpy as np
import pytest

import pyoracle
import tpt
from tpt import scenes

pytestmark = pytest.mark.gpu


def _spheres(rng, n, spread=50.0):
    c = rng.uniform(-spread, spread, (n, 3)).astype(np.float32)
    r = rng.uniform(0.05, 2.0, (n, 1)).astype(np.float32)
    return np.hstack([c - r, c + r])


def _cases():
    rng = np.random.default_rng(11)
    out = {f"spheres{n}": _spheres(rng, n) for n in (1, 2, 3, 31, 1000, 5000, 16384, 20000)}
    out["identical"] = np.tile(np.array([[1, 2, 3, 4, 5, 6]], np.float32), (300, 1))
    flat = _spheres(rng, 2000)
    flat[:, 1], flat[:, 4] = -0.5, 0.5
    out["flat"] = flat
    grid = _spheres(rng, 3000, 11.0)
    out["outlier"] = np.vstack([grid, [[-1000, -2000, -1000, 1000, 0, 1000]]]).astype(np.float32)
    out["clustered"] = np.vstack([_spheres(rng, 1500, 1e-3), _spheres(rng, 1500, 1e4)])
    return out


CASES = _cases()


@pytest.mark.parametrize("name", list(CASES))
def test_builder_matches_oracle(ctx, name):
    boxes = CASES[name]
    gb, gk, gs, gd = ctx.bvh_build_boxes(boxes)
    ob, ok, os_, od = pyoracle.lbvh_build(boxes)
    assert np.array_equal(gk, ok), "children differ"
    assert np.array_equal(gs, os_), "skip indices differ"
    assert np.array_equal(gb.view(np.uint32), ob.view(np.uint32)), "node boxes differ"
    assert gd == od


def test_builder_rejects_empty(ctx):
    with pytest.raises(tpt.TptError):
        ctx.bvh_build_boxes(np.zeros((0, 6), np.float32))


def test_noalloc_builds_the_uploaded_tree(ctx):
    import torch

    scene = tpt.Scene(scenes.one_weekend().text(), bvh="lbvh")
    slot = ctx.upload(scene)
    arena = torch.zeros(scene.info()["arena_bytes"], dtype=torch.uint8, device="cuda")
    w, h, spp, seed = 64, 48, 8, 21
    out = torch.full((h, w, 3), -1.0, dtype=torch.float32, device="cuda")
    p = tpt.make_params(w, h, spp, 50, background=tpt.BACKGROUND_SKY, seed=seed, engine=tpt.ENGINE_PERSISTENT)
    torch.cuda.synchronize()
    st = tpt.lib().tpt_render_noalloc(scene.handle, C.c_void_p(arena.data_ptr()), arena.numel(), C.byref(p),
                                      C.c_void_p(out.data_ptr()), None)
    assert st == 0, tpt.lib().tpt_last_error()
    ref, _ = ctx.render(slot, w, h, spp, 50, background=tpt.BACKGROUND_SKY, seed=seed,
                        engine=tpt.ENGINE_PERSISTENT)
    np.testing.assert_allclose(out.cpu().numpy(), ref, rtol=1e-5, atol=1e-6)
    ctx.release(slot)


def test_lbvh_batch_matches_reference_topology(ctx):
    sds = scenes.batch_scenes(seed=3, count=4)
    ref = [ctx.upload(tpt.Scene(sd.text())) for sd in sds]
    lb = [ctx.upload(tpt.Scene(sd.text(), bvh="lbvh")) for sd in sds]
    dims = [(40, 32, 8), (24, 24, 4), (32, 16, 8), (16, 16, 16)]
    ia, _ = tpt.render_batch(ctx, [(s, *d) for s, d in zip(ref, dims)], background=tpt.BACKGROUND_SKY, seed=4)
    ib, _ = tpt.render_batch(ctx, [(s, *d) for s, d in zip(lb, dims)], background=tpt.BACKGROUND_SKY, seed=4)
    for a, b in zip(ia, ib):
        # the same sample streams and closest hits: images agree up to the
        # float accumulation order
        np.testing.assert_allclose(b, a, rtol=1e-4, atol=1e-5)
    for s in ref + lb:
        ctx.release(s)


def test_nested_bvh_nodes_trace_as_the_reference(ctx):
    """bvh_nodes nested in a bvh_node: the rebuilt topologies flatten them
    into one tree and still report the reference's closest hits."""
    rng = np.random.default_rng(5)
    sd = scenes.SD()
    m = sd.lambertian(sd.const(0.5, 0.5, 0.5))
    inner = []
    for g in range(2):
        sph = [sd.sphere(rng.uniform(-5, 5, 3) + [10 * g, 0, 0], float(rng.uniform(0.2, 1.0)), m) for _ in range(40)]
        inner.append(sd.bvh(sph))
    sd.world(sd.bvh(inner + [sd.box((-1, -1, -1), (1, 1, 1), m)]))
    sd.camera((0, 0, 30), (5, 0, 0), (0, 1, 0), 40.0, 1.0, 0.0, 10.0)
    text = sd.text()
    ora = pyoracle.Scene(text)
    rays = ora.make_rays(20_000, 31, 0.5, 0.05)
    of, oi = ora.trace(rays, seed=5, media_mode=0)
    for bvh in ("sah", "lbvh"):
        slot = ctx.upload(tpt.Scene(text, bvh=bvh))
        f, i = ctx.trace_closest(slot, rays, seed=5)
        ctx.release(slot)
        assert np.array_equal(i[:, 0], oi[:, 0]), bvh
        hit = oi[:, 0] == 1
        np.testing.assert_allclose(f[hit, 0], of[hit, 0], rtol=1e-5, atol=1e-6)
        differ = hit & (i[:, 1] != oi[:, 1])
        assert (f[differ, 0] == of[differ, 0]).all(), bvh  # only exact ties may pick another primitive


def test_moving_spheres_under_rebuilt_topologies(ctx):
    """Moving spheres (boxes over the bvh_node's shutter interval) under the
    rebuilt topologies: the reference's closest hits at each ray's time."""
    rng = np.random.default_rng(9)
    sd = scenes.SD()
    m = sd.lambertian(sd.const(0.4, 0.6, 0.5))
    items = []
    for _ in range(60):
        c0 = rng.uniform(-6, 6, 3)
        items.append(sd.moving_sphere(c0, c0 + rng.uniform(-1, 1, 3), 0.0, 1.0, float(rng.uniform(0.2, 0.8)), m))
    items += [sd.sphere(rng.uniform(-6, 6, 3), float(rng.uniform(0.2, 0.8)), m) for _ in range(20)]
    sd.world(sd.bvh(items, 0.0, 1.0))
    sd.camera((0, 2, 25), (0, 0, 0), (0, 1, 0), 40.0, 1.0, 0.0, 10.0, 0.0, 1.0)
    text = sd.text()
    ora = pyoracle.Scene(text)
    rays = ora.make_rays(20_000, 17, 0.5, 0.05)
    of, oi = ora.trace(rays, seed=5, media_mode=0)
    assert (oi[:, 0] == 1).mean() > 0.05  # the batch does hit the spheres
    for bvh in ("sah", "lbvh"):
        slot = ctx.upload(tpt.Scene(text, bvh=bvh))
        f, i = ctx.trace_closest(slot, rays, seed=5)
        ctx.release(slot)
        assert np.array_equal(i[:, 0], oi[:, 0]), bvh
        hit = oi[:, 0] == 1
        np.testing.assert_allclose(f[hit, 0], of[hit, 0], rtol=1e-5, atol=1e-6)
        differ = hit & (i[:, 1] != oi[:, 1])
        assert (f[differ, 0] == of[differ, 0]).all(), bvh


def _chain_points():
    """Centroids whose Morton codes have one bit each, at 57 positions: the
    radix tree over them is a chain of depth 57."""
    pts = [[0.0, 0.0, 0.0]]
    for a in range(3):
        for k in range(2, 21):
            p = [0.0, 0.0, 0.0]
            p[a] = float(2 ** k)
            pts.append(p)
    pts.append([2.0 ** 21] * 3)
    return np.array(pts, np.float32)


def test_too_deep_lbvh_fails_at_upload(ctx):
    pts = _chain_points()
    boxes = np.hstack([pts - 0.25, pts + 0.25]).astype(np.float32)
    _, _, _, depth = ctx.bvh_build_boxes(boxes)
    assert depth == pyoracle.lbvh_build(boxes)[3] == 57
    sd = scenes.SD()
    m = sd.lambertian(sd.const(0.5, 0.5, 0.5))
    sd.world(sd.bvh([sd.sphere(p, 0.25, m) for p in pts]))
    sd.camera((0, 0, -10), (0, 0, 0), (0, 1, 0), 40.0, 1.0, 0.0, 10.0)
    text = sd.text()
    # the traversal stack holds 32 entries: the upload refuses the tree
    with pytest.raises(tpt.TptError) as e:
        ctx.upload(tpt.Scene(text, bvh="lbvh"))
    assert e.value.status == 8  # TPT_ERR_STACK_OVERFLOW
    assert b"LBVH of depth 57" in tpt.lib().tpt_last_error()
    # the reference's median-split tree over the same spheres is shallow
    slot = ctx.upload(tpt.Scene(text))
    ctx.release(slot)
