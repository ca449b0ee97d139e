"""Ensemble observables from the engine's FP64 moment blocks.

The reference saves raw fields only (its analysis tools are not part of the
project); these are the standard truncated-Wigner estimators. For Wigner
samples a of the field: <a^+ a> = <|a|^2>_W - 1/2,
<a^+2 a^2> = <|a|^4>_W - 2 <|a|^2>_W + 1/2, g2 = <a^+2 a^2> / <a^+ a>^2,
n_k = <|a_k|^2>_W - 1/2 with the unitary FFT a_k = FFT(a) / sqrt(N).

Moment blocks come from twmc_run / twmc_batch_reduce: block b holds FP64 sums
over trajectories [b T / B, (b + 1) T / B) of |a|^2, |a|^4 and |a_k|^2.
Standard errors use the batch means of the B blocks; g2 uses a
delete-one-block jackknife.
"""
from __future__ import annotations

import numpy as np


def block_sizes(ntraj: int, nblocks: int) -> np.ndarray:
    b = np.arange(nblocks + 1)
    edges = (b * ntraj) // nblocks
    return np.diff(edges)


def observables(moments: np.ndarray, ntraj: int) -> dict:
    """moments: (..., B, N, 3) FP64 block sums -> dict of (..., N) arrays."""
    m = np.asarray(moments, dtype=np.float64)
    B = m.shape[-3]
    cnt = block_sizes(ntraj, B).astype(np.float64)
    used = cnt > 0
    m = m[..., used, :, :]
    cnt = cnt[used]
    B = len(cnt)
    shape = (1,) * (m.ndim - 3) + (B, 1)
    c = cnt.reshape(shape)
    tot = m.sum(axis=-3)
    m2, m4, mk = tot[..., 0] / ntraj, tot[..., 1] / ntraj, tot[..., 2] / ntraj
    n = m2 - 0.5
    a2a2 = m4 - 2.0 * m2 + 0.5
    with np.errstate(divide="ignore", invalid="ignore"):
        g2 = a2a2 / n**2
    nk = mk - 0.5
    # batch means
    bm2 = m[..., 0] / c
    bm4 = m[..., 1] / c
    bmk = m[..., 2] / c
    def se(x):
        if B < 2:
            return np.full(x.shape[:-2] + x.shape[-1:], np.nan)
        return x.std(axis=-2, ddof=1) / np.sqrt(B)
    n_se = se(bm2)
    nk_se = se(bmk)
    # jackknife over blocks for g2
    g2_se = np.full_like(n, np.nan)
    if B >= 2:
        s2, s4 = m[..., 0].sum(axis=-2), m[..., 1].sum(axis=-2)
        jk = []
        for b in range(B):
            t = ntraj - cnt[b]
            j2 = (s2 - m[..., b, :, 0]) / t
            j4 = (s4 - m[..., b, :, 1]) / t
            with np.errstate(divide="ignore", invalid="ignore"):
                jk.append((j4 - 2 * j2 + 0.5) / (j2 - 0.5) ** 2)
        jk = np.stack(jk, axis=-2)
        g2_se = np.sqrt((B - 1) / B * ((jk - jk.mean(axis=-2, keepdims=True)) ** 2).sum(axis=-2))
    return {"n": n, "n_se": n_se, "a2a2": a2a2, "g2": g2, "g2_se": g2_se, "nk": nk, "nk_se": nk_se,
            "bm2": bm2}


def time_to_steady_state(times: np.ndarray, nbar: np.ndarray, nbar_se: np.ndarray, tail: float = 0.25,
                         hold: int = 2):
    """Earliest save time at which the spatially averaged n is within
    max(1 SE, 1e-3 n_inf) of n_inf (the mean of the last `tail` of the
    frames) and stays within twice that band for the next `hold` frames.

    First entry rather than "never leaves again": with a one-SE band, noise
    alone takes about a third of the steady frames outside it. Returns
    (time, n_inf); the last save time if the band is never reached."""
    times = np.asarray(times)
    nbar = np.asarray(nbar)
    k0 = int(np.floor((1.0 - tail) * len(nbar)))
    n_inf = float(np.mean(nbar[k0:]))
    tol = np.maximum(np.asarray(nbar_se), 1e-3 * abs(n_inf)) * np.ones_like(nbar)
    dev = np.abs(nbar - n_inf)
    for k in range(len(nbar)):
        nxt = slice(k + 1, min(len(nbar), k + 1 + hold))
        if dev[k] <= tol[k] and np.all(dev[nxt] <= 2.0 * tol[nxt]):
            return float(times[k]), n_inf
    return float(times[-1]), n_inf


def frame_observables(frames: np.ndarray, nblocks: int = 32) -> dict:
    """The same estimators from raw fields (T, F, N) complex, blocked like the
    engine's moment blocks (block b = trajectories [b T / B, (b + 1) T / B))."""
    x = np.asarray(frames)
    T = x.shape[0]
    ab2 = np.abs(x) ** 2
    edges = (np.arange(nblocks + 1) * T) // nblocks
    m = np.zeros((x.shape[1], nblocks, x.shape[2], 3))
    for b in range(nblocks):
        s = slice(edges[b], edges[b + 1])
        m[:, b, :, 0] = ab2[s].sum(0)
        m[:, b, :, 1] = (ab2[s] ** 2).sum(0)
    return observables(m, T)


def _z(a, sa, b, sb):
    with np.errstate(divide="ignore", invalid="ignore"):
        return (np.asarray(a) - np.asarray(b)) / np.sqrt(np.asarray(sa) ** 2 + np.asarray(sb) ** 2)


def compare(a: dict, b: dict, frames=slice(1, None), keys=("n", "g2", "nk")) -> dict:
    """Difference of two ensembles' observables in units of their combined
    standard error, z = (a - b) / sqrt(se_a^2 + se_b^2), per frame and site
    (frames: which save frames; frame 0 is the shared initial state).

    For each observable: max |z| and the mean of z^2 over frames and sites,
    and for n also the site-averaged density (its SE from the batch means of
    the site-averaged block densities). For independent ensembles of the same
    process z is close to N(0, 1): mean z^2 about 1. Ensembles sharing noise
    streams are positively correlated, so their z is smaller."""
    out = {}
    for k in keys:
        if k not in a or k not in b:
            continue
        z = _z(a[k][frames], a[k + "_se"][frames], b[k][frames], b[k + "_se"][frames])
        z = z[np.isfinite(z)]
        if z.size == 0:
            continue
        out[k] = {"max_abs_z": float(np.abs(z).max()), "mean_z2": float(np.mean(z ** 2)), "count": int(z.size)}

    def nbar(o):
        bm = o["bm2"][frames].mean(axis=-1)  # (F, B) site-averaged block <|a|^2>
        B = bm.shape[-1]
        return o["n"][frames].mean(axis=-1), bm.std(axis=-1, ddof=1) / np.sqrt(B)

    na, sa = nbar(a)
    nb, sb = nbar(b)
    zb = _z(na, sa, nb, sb)
    out["n_site_avg"] = {"max_abs_z": float(np.abs(zb).max()), "mean_z2": float(np.mean(zb ** 2)),
                         "count": int(zb.size),
                         "max_rel_diff": float(np.max(np.abs(na - nb) / np.maximum(np.abs(nb), 1e-300)))}
    return out
