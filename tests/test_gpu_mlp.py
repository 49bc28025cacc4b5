"""Tensor-core MLP kernels of the learned parts against the float64 CPU
reference (oracle/mlp_ref.py): forward outputs, weight gradients of a given
output gradient (the backward and weight-gradient GEMM kernels), and one Adam
step.  Tolerance: activations are rounded to f16 between layers on the GPU
(the reference rounds them the same way), products accumulate in f32."""
import numpy as np
import pytest

import mlp_ref
import tpt

pytestmark = pytest.mark.gpu

SHAPES = [(32, 2, 16), (112, 3, 48), (64, 5, 16)]
# Measured on a GB300 (largest error over the shapes and layers): forward
# 3.8e-4 of the output's largest magnitude, weight gradients 4.2e-4 of the
# layer's largest magnitude (given output gradient), 1.5e-4 (vMF loss),
# 8.5e-5 (relative L2 loss), loss sums 4e-6.  The remaining differences are
# f32 summation order and f16 roundings of activations and gradients that
# fall on the other side of a rounding boundary.
FWD_RTOL = 2e-3    # of the output's largest magnitude
GRAD_RTOL = 2e-3   # per layer, of the gradient's largest magnitude
LOSS_RTOL = 1e-4


def _inputs(rows, in_dim, seed):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-1, 1, size=(rows, in_dim)).astype(np.float16)
    return x


@pytest.mark.parametrize("shape", SHAPES)
def test_mlp_forward_matches_reference(built, shape):
    import torch

    in_dim, nh, out_dim = shape
    net = tpt.Mlp(in_dim, nh, out_dim, seed=3)
    p = net.get_params()
    p16 = p.astype(np.float16).astype(np.float32)
    rows = 4096
    x = _inputs(rows, in_dim, 1)
    xd = torch.from_numpy(x).cuda()
    yd = torch.empty((rows, out_dim), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    net.forward(xd.data_ptr(), rows, yd.data_ptr())
    torch.cuda.synchronize()
    y = yd.cpu().numpy()
    yr, _ = mlp_ref.forward(p16, x.astype(np.float64), in_dim, nh, out_dim)
    scale = np.abs(yr).max()
    print("forward", shape, np.abs(y - yr).max() / scale)
    assert np.abs(y - yr).max() < FWD_RTOL * scale, (np.abs(y - yr).max(), scale)


@pytest.mark.parametrize("shape", SHAPES)
def test_mlp_weight_gradients_match_reference(built, shape):
    import torch

    in_dim, nh, out_dim = shape
    net = tpt.Mlp(in_dim, nh, out_dim, seed=5)
    p = net.get_params()
    p16 = p.astype(np.float16).astype(np.float32)
    rows = 2048
    x = _inputs(rows, in_dim, 2)
    rng = np.random.default_rng(9)
    dy = rng.uniform(-1, 1, size=(rows, out_dim)).astype(np.float32) / rows
    xd = torch.from_numpy(x).cuda()
    dyd = torch.from_numpy(dy).cuda()
    torch.cuda.synchronize()
    net.backward_given(xd.data_ptr(), dyd.data_ptr(), rows, scale=256.0)
    torch.cuda.synchronize()
    g = net.get_grad() / 256.0
    _, acts = mlp_ref.forward(p16, x.astype(np.float64), in_dim, nh, out_dim)
    gr = mlp_ref.backward(p16, acts, dy.astype(np.float16).astype(np.float64) * 256 / 256, in_dim, nh, out_dim)
    # per layer relative error
    off = 0
    for (o, i) in mlp_ref.shapes(in_dim, nh, out_dim):
        a, b = g[off:off + o * i], gr[off:off + o * i]
        off += o * i
        print("given layer", shape, (o, i), np.abs(a - b).max() / np.abs(b).max())
        assert np.abs(a - b).max() < GRAD_RTOL * np.abs(b).max(), (o, i, np.abs(a - b).max(), np.abs(b).max())
    # Adam moves the weights against the gradient and clears it
    net.adam(1e-3, 1.0 / 256.0)
    p2 = net.get_params()
    moved = np.sign(p2 - p)
    big = np.abs(gr) > 1e-3 * np.abs(gr).max()
    assert (moved[big] == -np.sign(gr[big])).mean() > 0.97
    assert np.abs(net.get_grad()).max() == 0.0


def test_vmf_loss_gradient_matches_reference(built):
    """The guiding loss on the GPU (weighted vMF-mixture NLL) against the
    analytic float64 gradient of oracle/mlp_ref.py, itself checked against
    finite differences in tests/test_learn_ref.py."""
    import torch

    net = tpt.Mlp(112, 3, 48, seed=11)
    p16 = net.get_params().astype(np.float16).astype(np.float32)
    rows = 1024
    rng = np.random.default_rng(4)
    x = rng.uniform(0, 1, size=(rows, 112)).astype(np.float16)
    w = rng.normal(size=(rows, 3))
    w /= np.linalg.norm(w, axis=1, keepdims=True)
    wt = rng.uniform(0.1, 2.0, size=rows)
    target = np.concatenate([w, wt[:, None]], axis=1).astype(np.float32)
    xd = torch.from_numpy(x).cuda()
    td = torch.from_numpy(target).cuda()
    torch.cuda.synchronize()
    scale = 64.0 / rows
    loss = net.backward_vmf(xd.data_ptr(), td.data_ptr(), rows, scale)
    g = net.get_grad() / scale
    y, acts = mlp_ref.forward(p16, x.astype(np.float64), 112, 3, 48)
    dy = mlp_ref.vmf_nll_grad(y, w, wt)
    gr = mlp_ref.backward(p16, acts, dy.astype(np.float32).astype(np.float64), 112, 3, 48)
    ref_loss = mlp_ref.vmf_nll(y, w, wt).sum()
    print("vmf loss", loss, ref_loss)
    assert abs(loss - ref_loss) < LOSS_RTOL * abs(ref_loss)
    off = 0
    for (o, i) in mlp_ref.shapes(112, 3, 48):
        a, b = g[off:off + o * i], gr[off:off + o * i]
        off += o * i
        print("vmf layer", (o, i), np.abs(a - b).max() / np.abs(b).max())
        assert np.abs(a - b).max() < GRAD_RTOL * np.abs(b).max(), (o, i, np.abs(a - b).max(), np.abs(b).max())


def _records(n, seed, width):
    """Cache (width 5) or guide (width 3) records: positions mostly inside
    the box [-1, 3]^3, some outside; unit directions and normals; roughness
    and albedo in [0, 1]; a few non-finite entries."""
    rng = np.random.default_rng(seed)
    r = np.zeros((n, width, 4), np.float32)
    r[:, 0, :3] = rng.uniform(-1.5, 3.5, size=(n, 3))
    for k in (1, 2):
        d = rng.normal(size=(n, 3))
        r[:, k, :3] = d / np.linalg.norm(d, axis=1, keepdims=True)
    r[:, 0, 3] = rng.uniform(-0.1, 1.1, size=n)
    if width == 5:
        r[:, 3, :3] = rng.uniform(0, 1, size=(n, 3))
        r[:, 4] = rng.uniform(0, 4, size=(n, 4))
        r[::97, 3, 1] = np.inf
        r[::89, 0, 3] = np.nan
    else:
        r[::97, 0, 3] = -1.0       # negative weight: unusable
        r[::89, 2, 0] = np.nan     # non-finite direction: unusable
    r[::101, 0, 0] = np.nan
    return r


LO, EXT = np.array([-1, -1, -1], np.float32), np.array([4, 4, 4], np.float32)


def test_nrc_encoder_matches_reference(built):
    """The cache's input encoding (learn.cu nrc_encode) against its float32
    restatement (mlp_ref.nrc_encode): identical f16 rows, except that the
    direction one-blobs may differ by one f16 ulp where the device's acosf /
    atan2f and the host's differ in the last float bit."""
    rec = _records(20000, 1, 5)
    x = tpt.nrc_encode(rec, LO, EXT).astype(np.float32)
    xr = mlp_ref.nrc_encode(rec, LO, EXT).astype(np.float32)
    exact = np.r_[0:36, 52:64]
    assert np.array_equal(x[:, exact], xr[:, exact])
    d = np.abs(x[:, 36:52] - xr[:, 36:52])
    assert d.max() <= 2.0 ** -11 and (d > 0).mean() < 1e-3, (d.max(), (d > 0).mean())


def test_cache_query_accumulate_matches_reference(built):
    """The cached renderer's query evaluation (one tcgen05 kernel: encode,
    forward, throughput x max(cache, 0) added to the pixel's sum) against the
    float64 reference of the same steps (mlp_ref.nrc_encode, mlp_ref.forward),
    with queries colliding on pixels and some non-finite features; a count
    that is not a multiple of the 128-row tile."""
    import torch

    net = tpt.Mlp(64, 5, 16, seed=7)
    p16 = net.get_params().astype(np.float16).astype(np.float32)
    n, npix = 50_001, 3_000
    rec = _records(n, 4, 5)
    rng = np.random.default_rng(9)
    q = np.zeros((n, 6, 4), np.float32)
    q[:, :4] = rec[:, :4]
    q[:, 4, :3] = rng.uniform(0, 2, size=(n, 3))
    pix = rng.integers(0, npix, size=n).astype(np.int32)
    q[:, 4, 3] = pix.view(np.float32)
    acc0 = rng.uniform(0, 1, size=(npix, 4)).astype(np.float32)
    qd = torch.from_numpy(q.reshape(n, 24)).cuda()
    ad = torch.from_numpy(acc0.copy()).cuda()
    torch.cuda.synchronize()
    net.cache_accumulate(qd.data_ptr(), n, LO, EXT, ad.data_ptr(), npix)
    torch.cuda.synchronize()
    acc = ad.cpu().numpy().astype(np.float64)
    y, _ = mlp_ref.forward(p16, mlp_ref.nrc_encode(q, LO, EXT).astype(np.float64), 64, 5, 16)
    L = q[:, 4, :3].astype(np.float64) * np.maximum(y[:, :3], 0.0)
    L = np.where(np.isnan(L), 0.0, L)
    ref = acc0.astype(np.float64)
    np.add.at(ref[:, :3], pix, L)
    assert np.array_equal(acc[:, 3], acc0[:, 3])  # w untouched
    err = np.abs(acc[:, :3] - ref[:, :3])
    scale = np.abs(ref[:, :3] - acc0[:, :3]).max()
    print("cache accumulate", err.max() / scale)
    assert err.max() < FWD_RTOL * scale, (err.max(), scale)
    # a query naming a pixel past the buffer is skipped and reported
    q2 = q[:256].copy()
    q2[7, 4, 3] = np.int32(npix).view(np.float32)
    qd2 = torch.from_numpy(q2.reshape(256, 24)).cuda()
    before = ad.clone()
    with pytest.raises(tpt.TptError):
        net.cache_accumulate(qd2.data_ptr(), 256, LO, EXT, ad.data_ptr(), npix)
    got = (ad - before).cpu().numpy().astype(np.float64)[:, :3]
    ok = np.arange(256) != 7
    want = np.zeros((npix, 3))
    np.add.at(want, pix[:256][ok], L[:256][ok])
    assert np.abs(got - want).max() < FWD_RTOL * scale, np.abs(got - want).max()


def test_guide_encoder_matches_reference(built):
    """The guide's input encoding and loss targets (learn.cu
    guide_record_row) against mlp_ref.guide_encode: bit-identical, unusable
    records included."""
    rec = _records(20000, 2, 3)
    x, t = tpt.guide_encode(rec, LO, EXT)
    xr, tr = mlp_ref.guide_encode(rec, LO, EXT)
    assert np.array_equal(x.view(np.uint16), xr.view(np.uint16))
    assert np.array_equal(t, tr.astype(np.float32))


def test_rel_l2_loss_gradient_matches_reference(built):
    """The radiance cache's training signal on the GPU (the relative L2
    loss, learn.cu LossRelL2, through the fused training kernels) against
    the float64 gradient of mlp_ref.rel_l2_grad pushed through the
    reference backward; the loss sum against mlp_ref.rel_l2."""
    import torch

    net = tpt.Mlp(64, 5, 16, seed=13)
    p16 = net.get_params().astype(np.float16).astype(np.float32)
    rows = 2048
    rec = _records(rows, 3, 5)
    x = tpt.nrc_encode(rec, LO, EXT)
    rng = np.random.default_rng(5)
    target = np.concatenate([rng.uniform(0, 2, size=(rows, 3)), np.ones((rows, 1))], axis=1).astype(np.float32)
    xd = torch.from_numpy(x).cuda()
    td = torch.from_numpy(target).cuda()
    torch.cuda.synchronize()
    scale = 1024.0 / rows
    loss = net.backward_rel_l2(xd.data_ptr(), td.data_ptr(), rows, scale)
    g = net.get_grad() / scale
    y, acts = mlp_ref.forward(p16, x.astype(np.float64), 64, 5, 16)
    dy = mlp_ref.rel_l2_grad(y, target.astype(np.float64), 16)
    gr = mlp_ref.backward(p16, acts, dy.astype(np.float32).astype(np.float64), 64, 5, 16)
    ref_loss = mlp_ref.rel_l2(y, target).sum()
    print("rel_l2 loss", loss, ref_loss)
    assert abs(loss - ref_loss) < LOSS_RTOL * abs(ref_loss)
    off = 0
    for (o, i) in mlp_ref.shapes(64, 5, 16):
        a, b = g[off:off + o * i], gr[off:off + o * i]
        off += o * i
        err = np.abs(a - b).max() / np.abs(b).max()
        print("rel_l2 layer", (o, i), err)
        assert err < GRAD_RTOL, (o, i, err)


def _record_index(rows, count, key, step):
    """The cache's row sampler (learn.cu nrc_record_index), in uint32 arithmetic."""
    r = np.arange(rows, dtype=np.uint64)
    m = np.uint64(0xFFFFFFFF)
    h = ((r * np.uint64(0x9E3779B1)) & m) ^ np.uint64((step * 0x85EBCA77) & 0xFFFFFFFF) ^ np.uint64(key)
    h ^= h >> np.uint64(15)
    h = (h * np.uint64(0x2C1B3C6D)) & m
    h ^= h >> np.uint64(12)
    h = (h * np.uint64(0x297A2D39)) & m
    h ^= h >> np.uint64(15)
    return (h % np.uint64(count)).astype(np.int64)


def test_cache_training_from_records_matches_the_encoded_batch(built):
    """The cached renderer's training step, which samples and encodes its rows
    inside the tensor-core training kernel (tpt_mlp_backward_rel_l2_records),
    gives the gradient and loss of the same rows encoded first
    (tpt_nrc_encode) and trained through tpt_mlp_backward_rel_l2, and both
    match the float64 reference."""
    import torch

    rows, count, key, step = 4000, 2500, 0x1234567, 7
    rec = _records(count, 6, 5)
    idx = _record_index(rows, count, key, step)
    sampled = rec[idx]
    target = sampled[:, 4].copy()
    target[~np.isfinite(target).all(axis=1)] = 0
    x = tpt.nrc_encode(sampled, LO, EXT)
    a = tpt.Mlp(64, 5, 16, seed=21)
    b = tpt.Mlp(64, 5, 16, seed=21)
    dr = torch.from_numpy(np.ascontiguousarray(rec)).cuda()
    xd = torch.from_numpy(x).cuda()
    td = torch.from_numpy(np.ascontiguousarray(target)).cuda()
    torch.cuda.synchronize()
    scale = 1024.0 / rows
    la = a.backward_rel_l2_records(dr.data_ptr(), count, key, step, LO, EXT, rows, scale)
    lb = b.backward_rel_l2(xd.data_ptr(), td.data_ptr(), rows, scale)
    ga, gb = a.get_grad(), b.get_grad()
    assert abs(la - lb) <= 1e-6 * abs(lb)
    np.testing.assert_allclose(ga, gb, rtol=1e-5, atol=1e-6 * np.abs(gb).max())
    p16 = a.get_params().astype(np.float16).astype(np.float32)
    y, acts = mlp_ref.forward(p16, x.astype(np.float64), 64, 5, 16)
    gr = mlp_ref.backward(p16, acts, mlp_ref.rel_l2_grad(y, target.astype(np.float64), 16).astype(np.float32)
                          .astype(np.float64), 64, 5, 16)
    assert np.abs(ga / scale - gr).max() < GRAD_RTOL * np.abs(gr).max()
