"""CPU oracle of the learned warm start's network -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline import this
module, and only as the checker; nothing in the product path calls it.

The reference has no learned component, so there is nothing to pin against:
this restates the standard mathematics of the engine's MLP in numpy, in
FP64, rounding to BF16 at exactly the points where the device kernels hold
BF16 values (the GEMM operands), so that device and oracle differ only by
FP32 accumulation order:

  forward, layer l:  z = bf16(a_l) @ bf16(W_l)^T + b_l
                     a_{l+1} = bf16(gelu(fp32(z)))         (hidden layers)
                     y = z                                  (output layer)
  loss:              L = sum_{b,o} w_o (y - t)^2 / (B O)
                     dY = bf16(2 w_o (y - t) / (B O))
  backward:          dW_l = dZ_l^T @ a_l,  db_l = sum_b dZ_l
                     dZ_{l-1} = bf16((dZ_l @ bf16(W_l)) * gelu'(fp32(z_l)))
  Adam (Kingma & Ba 2015, bias-corrected), GELU(z) = z Phi(z) (erf form).

Parameter layout (shared with the device): for each layer l, W_l
[width[l+1]][width[l]] row-major, then b_l [width[l+1]].

Also restated: the MLP rows of a mean field (unitary 2-D DFT + density) and
the initial fields of a row (inverse DFT, per-quadrature sigma).
"""
from __future__ import annotations

import math

import numpy as np

try:  # scipy is present on both machines; the fallback keeps the module importable
    from scipy.special import erf as _erf
except Exception:  # pragma: no cover
    _erf = np.vectorize(math.erf)


def bf16(x) -> np.ndarray:
    """Round to the nearest BF16 (ties to even) from FP32, returned as float64."""
    f = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = f.view(np.uint32).astype(np.uint64)
    r = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def fp32(x) -> np.ndarray:
    return np.asarray(x, dtype=np.float32).astype(np.float64)


def gelu(z):
    return 0.5 * z * (1.0 + _erf(z / math.sqrt(2.0)))


def gelu_grad(z):
    return 0.5 * (1.0 + _erf(z / math.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / math.sqrt(2.0 * math.pi)


def offsets(widths):
    out, off = [], 0
    for k, n in zip(widths[:-1], widths[1:]):
        out.append((off, off + n * k))
        off += n * k + n
    return out, off


def unpack(params, widths):
    offs, _ = offsets(widths)
    ws, bs = [], []
    for (wo, bo), k, n in zip(offs, widths[:-1], widths[1:]):
        ws.append(np.asarray(params[wo:wo + n * k], dtype=np.float64).reshape(n, k))
        bs.append(np.asarray(params[bo:bo + n], dtype=np.float64))
    return ws, bs


def init_params(widths, seed=0):
    """Glorot-uniform weights, zero biases (numpy generator; the device's
    own initialiser uses a different generator, tests set parameters)."""
    rng = np.random.default_rng(seed)
    _, n = offsets(widths)
    p = np.zeros(n, dtype=np.float32)
    for (wo, _), k, m in zip(offsets(widths)[0], widths[:-1], widths[1:]):
        a = math.sqrt(6.0 / (k + m))
        p[wo:wo + m * k] = rng.uniform(-a, a, m * k)
    return p


def forward(params, widths, x, emulate_bf16=True):
    """Returns y and the cache (layer inputs a_l, pre-activations z_l)."""
    r = bf16 if emulate_bf16 else (lambda v: np.asarray(v, dtype=np.float64))
    f = fp32 if emulate_bf16 else (lambda v: np.asarray(v, dtype=np.float64))
    ws, bs = unpack(params, widths)
    a = r(x)
    acts, zs = [a], [None]
    nl = len(ws)
    for l in range(nl):
        z = a @ r(ws[l]).T + bs[l]
        if l + 1 < nl:
            zs.append(f(z))
            a = r(gelu(f(z)))
            acts.append(a)
        else:
            return z, (acts, zs)


def backward(params, widths, x, t, w=None, emulate_bf16=True):
    """Returns (loss, gradient array in the parameter layout, y)."""
    r = bf16 if emulate_bf16 else (lambda v: np.asarray(v, dtype=np.float64))
    y, (acts, zs) = forward(params, widths, x, emulate_bf16)
    B, O = y.shape
    wo = np.ones(O) if w is None else np.asarray(w, dtype=np.float64)
    e = y - np.asarray(t, dtype=np.float64)
    loss = float((wo * e * e).sum() / (B * O))
    d = r(2.0 * wo * e / (B * O))
    ws, _ = unpack(params, widths)
    offs, n = offsets(widths)
    g = np.zeros(n)
    for l in range(len(ws) - 1, -1, -1):
        wo_, bo_ = offs[l]
        k, m = widths[l], widths[l + 1]
        g[wo_:wo_ + m * k] = (d.T @ acts[l]).reshape(-1)
        g[bo_:bo_ + m] = d.sum(axis=0)
        if l > 0:
            d = r((d @ r(ws[l])) * gelu_grad(zs[l]))
    return loss, g, y


def adam(params, grads, m, v, step, lr, beta1=0.9, beta2=0.999, eps=1e-8):
    """One Adam step (step counts from 1); returns new (params, m, v)."""
    m = beta1 * m + (1 - beta1) * grads
    v = beta2 * v + (1 - beta2) * grads * grads
    mh = m / (1 - beta1 ** step)
    vh = v / (1 - beta2 ** step)
    return params - lr * mh / (np.sqrt(vh) + eps), m, v


def targets(mean, abs2, nx, ny, frames=1):
    """MLP rows [P][2N+1] from mean fields [P][N] complex and <|a|^2> [P][N]
    (sums over `frames` frames): unitary DFT (Re, Im interleaved) + density."""
    mean = np.asarray(mean, dtype=np.complex128) / frames
    P, N = mean.shape
    ak = np.fft.fft2(mean.reshape(P, nx, ny), norm="ortho").reshape(P, N)
    rows = np.zeros((P, 2 * N + 1))
    rows[:, 0:2 * N:2] = ak.real
    rows[:, 1:2 * N:2] = ak.imag
    rows[:, 2 * N] = np.asarray(abs2, dtype=np.float64).mean(axis=1) / frames - 0.5
    return rows


def standardize(t, squash=0.0, floor_frac=0.05):
    """Squash (asinh(v / squash) when squash > 0), then per-column mean and
    standard deviation (ddof 1, floored at floor_frac x the largest), and
    loss weights clamp((std / max std)^2, 1e-4, 1). Returns (t', mean, std, w)."""
    t = np.asarray(t, dtype=np.float64)
    if squash > 0:
        t = np.arcsinh(t / squash)
    mu = t.mean(0)
    sd = t.std(0, ddof=1) if t.shape[0] > 1 else np.zeros(t.shape[1])
    m = max(sd.max(), 1e-30)
    w = np.clip((sd / m) ** 2, 1e-4, 1.0)
    sd = np.maximum(sd, max(floor_frac * m, 1e-30))
    return (t - mu) / sd, mu, sd, w


def fields(rows, nx, ny, mean=None, std=None, squash=0.0, max_incoherent=np.inf):
    """Initial fields (beta_init, beta_sigma) [P][N] complex of MLP rows."""
    rows = np.asarray(rows, dtype=np.float64)
    if mean is not None:
        rows = rows * np.asarray(std, dtype=np.float64) + np.asarray(mean, dtype=np.float64)
    if squash > 0:
        rows = squash * np.sinh(rows)
    N = nx * ny
    P = rows.shape[0]
    ak = rows[:, 0:2 * N:2] + 1j * rows[:, 1:2 * N:2]
    b = np.fft.ifft2(ak.reshape(P, nx, ny), norm="ortho").reshape(P, N)
    dens = rows[:, 2 * N][:, None]
    inc = np.minimum(np.maximum(dens - np.abs(b) ** 2, 0.0), max_incoherent)
    sg = np.sqrt((inc + 0.5) * 0.5)
    return b, sg.astype(np.complex128)
