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


# ---- radiance cache loss ---------------------------------------------------
REL_L2_EPS = 0.01


def rel_l2(y, t):
    """Relative L2 of Mueller et al. 2021 ("Real-time Neural Radiance Caching
    for Path Tracing", eq. 3) per row: sum over rgb of
    (y - t)^2 / (y^2 + 0.01)."""
    y = y[:, :3].astype(np.float64)
    t = t[:, :3].astype(np.float64)
    return ((y - t) ** 2 / (y * y + REL_L2_EPS)).sum(-1)


def rel_l2_grad(y, t, out_dim):
    """d(loss)/dy with the denominator held constant (a stop-gradient on the
    prediction in the denominator, as the paper prescribes)."""
    g = np.zeros((y.shape[0], out_dim))
    yy = y[:, :3].astype(np.float64)
    g[:, :3] = 2.0 * (yy - t[:, :3]) / (yy * yy + REL_L2_EPS)
    return g


# ---- input encodings (float32 arithmetic as the GPU encoders do) -----------
F32 = np.float32


def one_blob(u, bins):
    """One-blob encoding (Mueller et al. 2019, "Neural Importance Sampling",
    sec. 4.3) of u in [0, 1] over `bins` bins, triangular kernel one bin
    wide; NaN encodes as 0."""
    u = np.nan_to_num(np.asarray(u, F32), nan=0.0)
    x = (np.clip(u, F32(0), F32(1)) * F32(bins)).astype(F32)
    centres = (np.arange(bins, dtype=F32) + F32(0.5))
    return np.maximum(F32(0), F32(1) - np.abs(x[:, None] - centres[None, :])).astype(F32)


def dir_blob(d):
    """Unit direction -> (theta / pi, phi / 2 pi in [0, 1)) one-blobs, 4 + 4 bins."""
    d = np.asarray(d, F32)
    th = (np.arccos(np.clip(d[:, 2], F32(-1), F32(1))) * F32(1.0 / np.pi)).astype(F32)
    ph = (np.arctan2(d[:, 1], d[:, 0]) * F32(0.5 / np.pi)).astype(F32)
    ph = np.where(ph < 0, ph + F32(1), ph).astype(F32)
    return np.concatenate([one_blob(th, 4), one_blob(ph, 4)], axis=1)


def _inv_ext(ext):
    return (F32(1) / np.asarray(ext, F32)).astype(F32)


def nrc_encode(rec, lo, ext):
    """Radiance-cache input rows (n x 64, f16) of records (n x >=4 x 4
    float32): position as a 12-octave triangle wave |2 frac(2^k x) - 1| per
    axis (36), outgoing direction and normal one-blobs (8 + 8), a 4-bin
    roughness one-blob, the albedo (non-finite -> 0), zero padding."""
    rec = np.asarray(rec, F32)
    n = rec.shape[0]
    out = np.zeros((n, 64), F32)
    c = ((rec[:, 0, :3] - np.asarray(lo, F32)) * _inv_ext(ext)).astype(F32)
    c = np.where(np.isfinite(c), np.clip(c, F32(0), F32(1)), F32(0)).astype(F32)
    for a in range(3):
        s = c[:, a].copy()
        for k in range(12):
            fr = (s - np.floor(s)).astype(F32)
            out[:, a * 12 + k] = np.abs(F32(2) * fr - F32(1))
            s = (s * F32(2)).astype(F32)
    out[:, 36:44] = dir_blob(rec[:, 1, :3])
    out[:, 44:52] = dir_blob(rec[:, 2, :3])
    out[:, 52:56] = one_blob(rec[:, 0, 3], 4)
    alb = rec[:, 3, :3]
    out[:, 56:59] = np.where(np.isfinite(alb), np.clip(alb, F32(-65504), F32(65504)), F32(0))
    return out.astype(np.float16)


def guide_encode(rec, lo, ext):
    """Path-guiding input rows (n x 112, f16) and loss targets (n x 4) of
    records (n x 3 x 4: position + weight, normal, direction): the position
    normalised to the box as 32-bin one-blobs per axis (96), the normal (3),
    zero padding.  An unusable record (non-finite, negative weight) becomes
    a zero-weight row at the box corner with normal and direction +z."""
    rec = np.asarray(rec, F32).copy()
    bad = ~(np.isfinite(rec).all(axis=(1, 2)) & (rec[:, 0, 3] >= 0))
    rec[bad, 0] = [*np.asarray(lo, F32), 0]
    rec[bad, 1] = [0, 0, 1, 0]
    rec[bad, 2] = [0, 0, 1, 0]
    xn = ((rec[:, 0, :3] - np.asarray(lo, F32)) * _inv_ext(ext)).astype(F32)
    out = np.zeros((rec.shape[0], 112), F32)
    for a in range(3):
        out[:, 32 * a:32 * (a + 1)] = one_blob(xn[:, a], 32)
    out[:, 96:99] = rec[:, 1, :3]
    target = np.concatenate([rec[:, 2, :3], rec[:, 0, 3:4]], axis=1)
    return out.astype(np.float16), target
