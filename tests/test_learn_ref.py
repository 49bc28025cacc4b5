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


def test_rel_l2_gradient_matches_finite_differences():
    """The cache loss's gradient holds the denominator constant: finite
    differences of (y - t)^2 / (d^2 + 0.01) with d frozen at y."""
    rng = np.random.default_rng(3)
    y = rng.uniform(-0.5, 3.0, size=(6, 16))
    t = np.concatenate([rng.uniform(0, 3, size=(6, 3)), np.ones((6, 1))], axis=1)
    g = mlp_ref.rel_l2_grad(y, t, 16)
    eps = 1e-6
    den = y[:, :3] ** 2 + mlp_ref.REL_L2_EPS
    for i in range(6):
        for c in range(3):
            yp, ym = y[i, c] + eps, y[i, c] - eps
            num = ((yp - t[i, c]) ** 2 - (ym - t[i, c]) ** 2) / den[i, c] / (2 * eps)
            assert abs(num - g[i, c]) < 1e-6 * max(1.0, abs(g[i, c]))
    assert np.all(g[:, 3:] == 0)
    assert np.allclose(mlp_ref.rel_l2(y, t), ((y[:, :3] - t[:, :3]) ** 2 / den).sum(1))


def test_encoders_known_answers():
    """One-blob and triangle-wave values at hand-checked points."""
    ob = mlp_ref.one_blob(np.array([0.0, 0.5, 1.0, np.nan]), 4)
    assert np.allclose(ob[0], [0.5, 0, 0, 0]) and np.allclose(ob[1], [0, 0.5, 0.5, 0])
    assert np.allclose(ob[2], [0, 0, 0, 0.5]) and np.allclose(ob[3], ob[0])
    rec = np.zeros((1, 5, 4), np.float32)
    rec[0, 0] = [0.25, 0.5, 0.75, 0.5]   # position (box [0,1]^3), roughness
    rec[0, 1, :3] = [0, 0, 1]            # outgoing direction +z: theta 0
    rec[0, 2, :3] = [1, 0, 0]            # normal +x: theta 1/2, phi 0
    rec[0, 3, :3] = [0.1, 0.2, np.inf]   # albedo, a non-finite channel -> 0
    x = mlp_ref.nrc_encode(rec, [0, 0, 0], [1, 1, 1]).astype(np.float32)[0]
    # |2 frac(2^k 0.25) - 1|: 0.5, 0, 1, 1, ...
    assert np.allclose(x[0:4], [0.5, 0.0, 1.0, 1.0])
    assert np.allclose(x[36:40], [0.5, 0, 0, 0]) and np.allclose(x[44:48], [0, 0.5, 0.5, 0])
    assert np.allclose(x[56:59], [0.1, 0.2, 0.0], atol=1e-3) and np.all(x[59:] == 0)
    g, t = mlp_ref.guide_encode(np.array([[[0.5, 0.5, 0.5, 2.0], [0, 1, 0, 0], [0, 0, -1, 0]],
                                          [[np.nan, 0, 0, 1.0], [0, 1, 0, 0], [0, 0, 1, 0]]]), [0, 0, 0], [1, 1, 1])
    assert g[0, 15] == 0.5 and g[0, 16] == 0.5 and g[0, 97] == 1 and np.allclose(t[0], [0, 0, -1, 2])
    assert t[1, 3] == 0 and g[1, 0] == 0.5 and g[1, 98] == 1  # unusable record: corner, +z, zero weight
