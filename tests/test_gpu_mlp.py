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
    assert np.abs(y - yr).max() < 2e-2 * scale + 1e-3, (np.abs(y - yr).max(), scale)


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
        assert np.abs(a - b).max() < 3e-2 * np.abs(b).max() + 1e-6, (o, i, np.abs(a - b).max(), np.abs(b).max())
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
    assert abs(loss - ref_loss) < 2e-2 * abs(ref_loss)
    off = 0
    for (o, i) in mlp_ref.shapes(112, 3, 48):
        a, b = g[off:off + o * i], gr[off:off + o * i]
        off += o * i
        assert np.abs(a - b).max() < 5e-2 * np.abs(b).max() + 1e-6, (o, i, np.abs(a - b).max(), np.abs(b).max())
