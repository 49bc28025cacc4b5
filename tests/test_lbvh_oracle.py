"""The CPU restatement of the GPU linear-BVH builder (oracle/lbvh.cc), checked
against a second, independent restatement written here: numpy float32 keys
(the same IEEE single operations, no fused multiply-add) and the binary radix
tree built top-down (split each range where the highest differing key bit
flips), which for unique keys is the tree Karras 2012 builds bottom-up.  The
GPU builder is then checked bit for bit against oracle/lbvh.cc
(tests/test_gpu_lbvh.py).  Also: the host compiler reserves the node slots
of a TPT_BVH_LBVH scene."""
import numpy as np
import pytest

import pyoracle


def _index_bits(n):
    b = 1
    while (1 << b) < n:
        b += 1
    return b


def _spread3(q):
    r = 0
    for b in range(21):
        r |= ((q >> b) & 1) << (3 * b)
    return r


def np_keys(boxes):
    boxes = np.asarray(boxes, np.float32)
    n = len(boxes)
    c = (boxes[:, :3] + boxes[:, 3:]) * np.float32(0.5)
    cmin, cmax = c.min(axis=0), c.max(axis=0)
    ib = _index_bits(n)
    mb = min(21, (64 - ib) // 3)
    cells = np.float32(1 << mb)
    keys = []
    for i in range(n):
        m = 0
        for a in range(3):
            ext = np.float32(cmax[a] - cmin[a])
            q = 0
            if ext > 0:
                t = np.float32(np.float32(c[i, a] - cmin[a]) * np.float32(cells / ext))
                q = (1 << mb) - 1 if t >= cells else (int(t) if t >= 0 else 0)
            m |= _spread3(q) << (2 - a)
        keys.append((m << ib) | i)
    return keys, mb


def topdown_tree(boxes):
    """Radix tree over the sorted unique keys, top-down, in pre-order."""
    boxes = np.asarray(boxes, np.float32)
    keys, _ = np_keys(boxes)
    order = sorted(keys)
    ib = _index_bits(len(boxes))
    prim = [k & ((1 << ib) - 1) for k in order]
    nodes = []  # [box(6), kids(2), skip]

    def build(a, b, depth):
        me = len(nodes)
        nodes.append(None)
        if a == b:  # one primitive: left == right
            nodes[me] = [boxes[prim[a]].copy(), [~prim[a], ~prim[a]], me + 1]
            return me, depth
        hb = (order[a] ^ order[b]).bit_length() - 1
        s = a
        while not (order[s + 1] >> hb) & 1:
            s += 1
        kids, md, bx = [], depth, []
        for lo, hi in ((a, s), (s + 1, b)):
            if lo == hi:
                kids.append(~prim[lo])
                bx.append(boxes[prim[lo]])
            else:
                k, d = build(lo, hi, depth + 1)
                kids.append(k)
                md = max(md, d)
                bx.append(nodes[k][0])
        box = np.concatenate([np.minimum(bx[0][:3], bx[1][:3]), np.maximum(bx[0][3:], bx[1][3:])])
        nodes[me] = [box, kids, len(nodes)]
        return me, md

    _, depth = build(0, len(boxes) - 1, 1)
    return (np.array([n[0] for n in nodes], np.float32), np.array([n[1] for n in nodes], np.int32),
            np.array([n[2] for n in nodes], np.int32), depth)


def _cases():
    rng = np.random.default_rng(7)
    out = {}
    for n in (1, 2, 3, 5, 16, 17, 100, 300):
        c = rng.uniform(-50, 50, (n, 3)).astype(np.float32)
        r = rng.uniform(0.1, 3, (n, 1)).astype(np.float32)
        out[f"spheres{n}"] = np.hstack([c - r, c + r])
    out["identical"] = np.tile(np.array([[0, 0, 0, 1, 1, 1]], np.float32), (40, 1))
    flat = rng.uniform(-5, 5, (64, 3)).astype(np.float32)
    flat[:, 1] = 2.0
    out["plane"] = np.hstack([flat - 0.5, flat + 0.5])
    g = rng.uniform(-11, 11, (120, 3)).astype(np.float32)
    g[:, 1] = 0.2
    grid = np.hstack([g - 0.2, g + 0.2])
    out["ground_sphere"] = np.vstack([grid, [[-1000, -2000, -1000, 1000, 0, 1000]]]).astype(np.float32)
    return out


CASES = _cases()


@pytest.mark.parametrize("name", list(CASES))
def test_oracle_keys_match_numpy(built, name):
    keys, bits = pyoracle.lbvh_keys(CASES[name])
    ref, mb = np_keys(CASES[name])
    assert bits == mb
    assert [int(k) for k in keys] == ref
    assert len(set(ref)) == len(ref)


@pytest.mark.parametrize("name", list(CASES))
def test_oracle_tree_matches_topdown(built, name):
    boxes = CASES[name]
    nb, kids, skip, depth = pyoracle.lbvh_build(boxes)
    tb, tk, ts, td = topdown_tree(boxes)
    assert np.array_equal(kids, tk)
    assert np.array_equal(skip, ts)
    assert np.array_equal(nb.view(np.uint32), tb.view(np.uint32))
    assert depth == td
    # every primitive is a leaf exactly once
    leaves = sorted(~k for k in kids.ravel() if k < 0)
    expect = [0, 0] if len(boxes) == 1 else list(range(len(boxes)))
    assert leaves == expect


def test_host_compiler_reserves_lbvh_slots(built):
    import tpt
    from tpt import scenes

    for name in ("one_weekend", "next_week", "instances"):
        text = scenes.PRESETS[name]().text()
        sah = tpt.Scene(text, bvh="sah").info()
        lb = tpt.Scene(text, bvh="lbvh").info()
        # n - 1 internal nodes per bvh_node, as the SAH tree (a binary tree
        # with one primitive per leaf)
        assert lb["n_nodes"] == sah["n_nodes"]
        assert lb["n_leaves"] == sah["n_leaves"]
        assert lb["arena_bytes"] > sah["arena_bytes"]  # build inputs and scratch


def nested_bvh_scene():
    """Spheres in two bvh_nodes nested inside a third, plus a box: the LBVH
    and SAH rebuilds flatten the nesting into one tree over the primitives."""
    from tpt import scenes

    rng = np.random.default_rng(5)
    sd = scenes.SD()
    m = sd.lambertian(sd.const(0.5, 0.5, 0.5))
    inner = []
    for g in range(2):
        sph = [sd.sphere(rng.uniform(-5, 5, 3) + [10 * g, 0, 0], float(rng.uniform(0.2, 1.0)), m) for _ in range(40)]
        inner.append(sd.bvh(sph))
    outer = sd.bvh(inner + [sd.box((-1, -1, -1), (1, 1, 1), m)])
    sd.world(outer)
    sd.camera((0, 0, 30), (5, 0, 0), (0, 1, 0), 40.0, 1.0, 0.0, 10.0)
    return sd.text()


def test_nested_bvh_nodes_become_one_tree(built):
    import tpt

    text = nested_bvh_scene()
    for bvh in ("sah", "lbvh"):
        info = tpt.Scene(text, bvh=bvh).info()
        assert info["n_leaves"] == 81 and info["n_nodes"] == 80, (bvh, info)  # n - 1 nodes over 81 primitives
    ref = tpt.Scene(text).info()
    assert ref["n_leaves"] == 81 and ref["n_nodes"] > 80  # the reference keeps the nesting (n == 1 nodes too)


def test_unknown_topology_is_rejected(built):
    import ctypes as C

    import tpt

    h = C.c_void_p()
    err = C.create_string_buffer(256)
    st = tpt.lib().tpt_scene_from_text_opt(nested_bvh_scene().encode(), 3, C.byref(h), err, 256)
    assert st == 1 and not h.value  # TPT_ERR_INVALID_ARGUMENT, no scene
