"""CPU oracle of the path-guiding network (test infrastructure only).

The guiding network has no counterpart in the reference: this is the FP64
statement of what the device kernels compute, written from the mathematics,
and the checker of their forward pass, backward pass, loss gradient and
mixture density.

Numerics emulated from the device: inputs, weights, hidden activations and
output gradients are rounded to BF16 (round to nearest even) where the
tensor cores read them; sums are exact (FP64) here and FP32 on the device.
"""
import numpy as np

IN, WIDTH, OUT, LOBES = 128, 64, 64, 8
LOG_KAPPA_MIN, LOG_KAPPA_MAX = -4.0, 9.0


def bf16(x):
    """Rounds to the nearest BF16 value (ties to even), returned as float64."""
    x32 = np.ascontiguousarray(x, dtype=np.float32)
    bits = x32.view(np.uint32).astype(np.uint64)
    bits = (bits + 0x7FFF + ((bits >> 16) & 1)) & 0xFFFF0000
    return bits.astype(np.uint32).view(np.float32).astype(np.float64)


def split(weights, hidden):
    """The flat weight vector as matrices [64 out][in]."""
    w = np.asarray(weights, dtype=np.float64)
    mats, off = [], 0
    for l in range(hidden + 1):
        k = IN if l == 0 else WIDTH
        mats.append(w[off:off + WIDTH * k].reshape(WIDTH, k))
        off += WIDTH * k
    return mats


def forward(weights, hidden, x, rounding=True):
    """Outputs (n, 64) and the per-layer inputs and pre-activations."""
    r = bf16 if rounding else (lambda a: np.asarray(a, dtype=np.float64))
    mats = split(weights, hidden)
    h = r(x)
    inputs, pre = [], []
    for l, W in enumerate(mats):
        inputs.append(h)
        z = h @ r(W).T
        pre.append(z)
        if l < hidden:
            h = r(np.maximum(z, 0.0))
    return z, inputs, pre


def backward(weights, hidden, x, dout, rounding=True):
    """Gradient of sum(dout * outputs) with respect to the flat weights."""
    r = bf16 if rounding else (lambda a: np.asarray(a, dtype=np.float64))
    mats = split(weights, hidden)
    _, inputs, pre = forward(weights, hidden, x, rounding)
    grads = [None] * len(mats)
    dz = np.asarray(dout, dtype=np.float64)
    for l in range(hidden, -1, -1):
        dzr = r(dz)
        grads[l] = dzr.T @ inputs[l]
        if l > 0:
            dx = dzr @ r(mats[l])
            dz = dx * (pre[l - 1] > 0)
    return np.concatenate([g.ravel() for g in grads])


BINS_OF = [32, 32, 32, 6, 6, 6, 6]  # position axes, then normal and outgoing angles


def one_blob(s):
    """Encoded inputs (n, 128) of scalars s (n, 7) in [0, 1]: each scalar's
    Gaussian bins one after another, then a constant 1, then zeros."""
    s = np.asarray(s, dtype=np.float64)
    parts = []
    for i, bins in enumerate(BINS_OF):
        centres = (np.arange(bins) + 0.5) / bins
        x = (s[:, i:i + 1] - centres[None, :]) * bins
        parts.append(np.exp(-0.5 * x * x))
    enc = np.concatenate(parts, axis=1)
    out = np.zeros((len(s), IN))
    out[:, :enc.shape[1]] = enc
    out[:, enc.shape[1]] = 1.0
    return out


def decode(raw):
    """Mixture (mu (n, 8, 3), kappa (n, 8), w (n, 8)) from raw outputs (n, 64)."""
    o = np.asarray(raw, dtype=np.float64)[:, :5 * LOBES].reshape(-1, LOBES, 5)
    m = o[:, :, 0:3]
    ln = np.linalg.norm(m, axis=2, keepdims=True)
    mu = np.where(ln > 1e-10, m / np.maximum(ln, 1e-300), np.array([0.0, 1.0, 0.0]))
    kappa = np.exp(np.clip(o[:, :, 3], LOG_KAPPA_MIN, LOG_KAPPA_MAX))
    logit = o[:, :, 4]
    e = np.exp(logit - logit.max(axis=1, keepdims=True))
    return mu, kappa, e / e.sum(axis=1, keepdims=True)


def vmf(mu, kappa, w):
    """vMF densities of directions w (n, 3) under lobes (n, 8, 3), (n, 8)."""
    norm = kappa / (2 * np.pi * -np.expm1(-2 * kappa))
    return norm * np.exp(kappa * ((mu * w[:, None, :]).sum(axis=2) - 1))


def pdf(raw, w):
    mu, kappa, wt = decode(raw)
    return (wt * vmf(mu, kappa, np.asarray(w, dtype=np.float64))).sum(axis=1)


def loss(raw, w, c):
    return -np.asarray(c, dtype=np.float64) * np.log(pdf(raw, w))


def loss_grad(raw, w, c):
    """d loss / d raw (n, 64), analytically."""
    raw = np.asarray(raw, dtype=np.float64)
    w = np.asarray(w, dtype=np.float64)
    c = np.asarray(c, dtype=np.float64)
    n = len(raw)
    mu, kappa, wt = decode(raw)
    v = vmf(mu, kappa, w)
    q = (wt * v).sum(axis=1)
    resp = wt * v / q[:, None]
    o = raw[:, :5 * LOBES].reshape(n, LOBES, 5)
    ln = np.linalg.norm(o[:, :, 0:3], axis=2)
    mw = (mu * w[:, None, :]).sum(axis=2)
    dmu = (kappa / ln)[:, :, None] * (w[:, None, :] - mw[:, :, None] * mu)
    ls = o[:, :, 3]
    inside = (ls > LOG_KAPPA_MIN) & (ls < LOG_KAPPA_MAX)
    dls = np.where(inside, 1 - 2 * kappa / np.expm1(2 * kappa) + kappa * (mw - 1), 0.0)
    g = np.zeros((n, LOBES, 5))
    g[:, :, 0:3] = -c[:, None, None] * resp[:, :, None] * dmu
    g[:, :, 3] = -c[:, None] * resp * dls
    g[:, :, 4] = -c[:, None] * (resp - wt)
    out = np.zeros((n, OUT))
    out[:, :5 * LOBES] = g.reshape(n, 5 * LOBES)
    return out
