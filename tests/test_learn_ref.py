"""CPU checks of the learned parts' reference (no GPU): the analytic vMF
mixture gradient against central finite differences, the mixture's
normalisation over the sphere, and the MLP reference backward against finite
differences."""
import numpy as np

import mlp_ref


def test_vmf_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    y = rng.normal(size=(4, 48))
    w = rng.normal(size=(4, 3))
    w /= np.linalg.norm(w, axis=1, keepdims=True)
    wt = rng.uniform(0.5, 2, 4)
    g = mlp_ref.vmf_nll_grad(y, w, wt)
    eps = 1e-6
    for i in range(4):
        for j in range(40):
            yp, ym = y.copy(), y.copy()
            yp[i, j] += eps
            ym[i, j] -= eps
            num = (mlp_ref.vmf_nll(yp[i:i + 1], w[i:i + 1], wt[i:i + 1]) -
                   mlp_ref.vmf_nll(ym[i:i + 1], w[i:i + 1], wt[i:i + 1]))[0] / (2 * eps)
            assert abs(num - g[i, j]) < 1e-6 * max(1.0, abs(g[i, j]))
    assert np.all(g[:, 40:] == 0)


def test_vmf_mixture_integrates_to_one():
    rng = np.random.default_rng(1)
    y = rng.normal(size=(1, 48)) * 2
    pi, kappa, mu = mlp_ref.vmf_params(y)
    # quadrature on a fine (cos theta, phi) grid
    n = 800
    ct = (np.arange(n) + 0.5) / n * 2 - 1
    ph = (np.arange(2 * n) + 0.5) / (2 * n) * 2 * np.pi
    C, P = np.meshgrid(ct, ph, indexing="ij")
    st = np.sqrt(1 - C ** 2)
    dirs = np.stack([st * np.cos(P), st * np.sin(P), C], axis=-1).reshape(-1, 3)
    pdf = mlp_ref.vmf_pdf(pi[0], kappa[0], mu[0], dirs)
    integral = pdf.sum() * (2.0 / n) * (2 * np.pi / (2 * n))
    assert abs(integral - 1.0) < 2e-3


def test_mlp_reference_backward_matches_finite_differences():
    rng = np.random.default_rng(2)
    in_dim, nh, out_dim = 32, 2, 16
    n_par = sum(o * i for o, i in mlp_ref.shapes(in_dim, nh, out_dim))
    p = rng.normal(size=n_par) * 0.3
    x = rng.normal(size=(8, in_dim))
    dy = rng.normal(size=(8, out_dim))
    y, acts = mlp_ref.forward(p, x, in_dim, nh, out_dim, f16_acts=False)
    g = mlp_ref.backward(p, acts, dy, in_dim, nh, out_dim)
    eps = 1e-6
    for k in rng.choice(n_par, size=40, replace=False):
        pp, pm = p.copy(), p.copy()
        pp[k] += eps
        pm[k] -= eps
        yp, _ = mlp_ref.forward(pp, x, in_dim, nh, out_dim, f16_acts=False)
        ym, _ = mlp_ref.forward(pm, x, in_dim, nh, out_dim, f16_acts=False)
        num = ((yp - ym) * dy).sum() / (2 * eps)
        assert abs(num - g[k]) < 1e-5 * max(1.0, abs(g[k]))
