"""CPU reference of the learned parts' networks and losses (numpy, float64).

TEST INFRASTRUCTURE ONLY: the tests compare the GPU kernels of
tiny-path-tracer_gb300/csrc/learn.cu against it.  The MLP is in -> [64 ReLU] x
n_hidden -> out, no biases, weights row-major [out][in] per layer,
concatenated.  The GPU stores weights and activations in f16 and
accumulates in f32; callers pass f16-rounded weights and inputs, and compare
with a tolerance that covers the f16 rounding of activations.
"""
from __future__ import annotations

import numpy as np

HID = 64


def shapes(in_dim: int, n_hidden: int, out_dim: int):
    dims = [in_dim] + [HID] * n_hidden + [out_dim]
    return [(dims[i + 1], dims[i]) for i in range(len(dims) - 1)]


def split(params: np.ndarray, in_dim: int, n_hidden: int, out_dim: int):
    out, off = [], 0
    for (o, i) in shapes(in_dim, n_hidden, out_dim):
        out.append(params[off:off + o * i].reshape(o, i).astype(np.float64))
        off += o * i
    return out


def forward(params, x, in_dim, n_hidden, out_dim, f16_acts=True):
    """Returns (y, activations) with activations[l] = input of layer l."""
    W = split(params, in_dim, n_hidden, out_dim)
    h = x.astype(np.float64)
    acts = [h]
    for l, w in enumerate(W):
        z = h @ w.T
        if l < len(W) - 1:
            h = np.maximum(z, 0.0)
            if f16_acts:
                h = h.astype(np.float16).astype(np.float64)
            acts.append(h)
        else:
            return z, acts


def backward(params, acts, dy, in_dim, n_hidden, out_dim):
    """Weight gradients (concatenated) of sum(dy * y)."""
    W = split(params, in_dim, n_hidden, out_dim)
    grads = [None] * len(W)
    dz = dy.astype(np.float64)
    for l in range(len(W) - 1, -1, -1):
        grads[l] = dz.T @ acts[l]
        if l > 0:
            dh = dz @ W[l]
            dz = dh * (acts[l] > 0)
    return np.concatenate([g.reshape(-1) for g in grads])


# ---- vMF mixture (path guiding) ------------------------------------------
def vmf_params(y: np.ndarray, lobes: int = 8):
    """Raw outputs -> (pi, kappa, mu).  Per lobe 5 outputs: weight logit,
    kappa pre-activation (softplus + 1e-2), mean direction (normalised)."""
    y = y[..., : 5 * lobes].reshape(y.shape[:-1] + (lobes, 5)).astype(np.float64)
    logits = y[..., 0]
    pi = np.exp(logits - logits.max(axis=-1, keepdims=True))
    pi /= pi.sum(axis=-1, keepdims=True)
    kappa = np.logaddexp(0.0, y[..., 1]) + 1e-2
    m = y[..., 2:5]
    mu = m / np.maximum(np.linalg.norm(m, axis=-1, keepdims=True), 1e-12)
    return pi, kappa, mu


def vmf_pdf(pi, kappa, mu, w):
    """Mixture density at unit directions w (solid-angle measure)."""
    cos = (mu * w[..., None, :]).sum(-1)
    norm = kappa / (2 * np.pi * (1 - np.exp(-2 * kappa)))
    return (pi * norm * np.exp(kappa * (cos - 1))).sum(-1)


def vmf_nll(y, w, weight, lobes: int = 8):
    pi, kappa, mu = vmf_params(y, lobes)
    return -(weight * np.log(vmf_pdf(pi, kappa, mu, w)))


def vmf_nll_grad(y, w, weight, lobes: int = 8):
    """Analytic d(nll)/dy for one batch (rows), matching the GPU loss."""
    y = y.astype(np.float64)
    pi, kappa, mu = vmf_params(y, lobes)
    cos = (mu * w[:, None, :]).sum(-1)
    e2 = np.exp(-2 * kappa)
    f = kappa / (2 * np.pi * (1 - e2)) * np.exp(kappa * (cos - 1))
    p = (pi * f).sum(-1, keepdims=True)
    r = pi * f / p
    g = np.zeros_like(y)
    yl = y[:, : 5 * lobes].reshape(-1, lobes, 5)
    dlogit = pi - r
    dlogf_dk = 1.0 / kappa - 2 * e2 / (1 - e2) + (cos - 1)
    dk = -r * dlogf_dk * (1.0 / (1.0 + np.exp(-yl[..., 1])))
    m = yl[..., 2:5]
    mn = np.maximum(np.linalg.norm(m, axis=-1, keepdims=True), 1e-12)
    dmu = -(r * kappa)[..., None] * (w[:, None, :] - cos[..., None] * mu) / mn
    gl = np.concatenate([dlogit[..., None], dk[..., None], dmu], axis=-1)
    g[:, : 5 * lobes] = (gl * weight[:, None, None]).reshape(-1, 5 * lobes)
    return g
