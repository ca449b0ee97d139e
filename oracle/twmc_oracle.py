"""Independent numpy restatement of the reference's TWMC hot path.

TEST INFRASTRUCTURE ONLY (the oracle). It cross-checks oracle/twmc_oracle.cpp
with a second implementation that shares no code with it: numpy's pocketfft
instead of the hand-written FFT, a dense coupling matrix instead of the CSR
triplets, and a vectorised Philox4x32-10 written from the SC'11 paper's round
function. Parity with the reference is unpinned by reference outputs (the
reference cannot be built here); see the header of twmc_oracle.cpp.

Follows (paths relative to the reference project root):
  TWMCBaseSolver::Compute   src/TWMC/Solvers/TWMCBaseSolver.cpp:206-280
  TWMCLiebSolver::Compute   src/TWMC/Solvers/TWMCLiebSolver.cpp:222-294
  coupling triplets         src/TWMC/Solvers/TWMCLiebSolver.cpp:52-85
"""
from __future__ import annotations

import numpy as np

M0 = np.uint64(0xD2511F53)
M1 = np.uint64(0xCD9E8D57)
W0 = np.uint64(0x9E3779B9)
W1 = np.uint64(0xBB67AE85)
MASK = np.uint64(0xFFFFFFFF)
# fixed key of the Wiener stream (stream 0): hex digits of pi
WIENER_KEY = (0x243F6A88, 0x85A308D3)


def philox4x32_10(ctr, key):
    """Vectorised Philox4x32-10. ctr: (..., 4) uint32, key: (..., 2) uint32."""
    c = np.asarray(ctr, dtype=np.uint64)
    k = np.asarray(key, dtype=np.uint64)
    c0, c1, c2, c3 = (c[..., i].copy() for i in range(4))
    k0, k1 = k[..., 0].copy(), k[..., 1].copy()
    for _ in range(10):
        p0 = M0 * c0
        p1 = M1 * c2
        hi0, lo0 = p0 >> np.uint64(32), p0 & MASK
        hi1, lo1 = p1 >> np.uint64(32), p1 & MASK
        c0, c1, c2, c3 = hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0
        k0 = (k0 + W0) & MASK
        k1 = (k1 + W1) & MASK
    return np.stack([c0, c1, c2, c3], axis=-1).astype(np.uint32)


def site_normals(seed: int, tid: int, step: int, stream: int, n: int, f32_flavour: bool = False):
    """Complex normals for sites 0..n-1 (site pairing: half = ceil(n/2))."""
    half = (n + 1) // 2
    p = np.arange(n)
    c0 = np.where(p < half, p, p - half).astype(np.uint32)
    lane = np.where(p < half, 0, 2)
    if stream == 0:   # Wiener: fixed key, ctr = (site pair, step, tid, seed)
        ctr = np.stack([c0, np.full(n, step, np.uint32), np.full(n, tid, np.uint32), np.full(n, seed, np.uint32)], -1)
        key = np.broadcast_to(np.array(WIENER_KEY, dtype=np.uint32), (n, 2))
    else:             # ctr = (site pair, step, stream, 0), key = (seed, tid)
        ctr = np.stack([c0, np.full(n, step, np.uint32), np.full(n, stream, np.uint32), np.zeros(n, np.uint32)], -1)
        key = np.broadcast_to(np.array([seed, tid], dtype=np.uint32), (n, 2))
    w = philox4x32_10(ctr, key)
    a = w[p, lane].astype(np.float64)
    b = w[p, lane + 1].astype(np.float64)
    if f32_flavour:
        # float(a) rounds to nearest; fma(x, 2^-32, 2^-33) is exact up to one
        # float rounding, reproduced here by rounding the exact double value.
        u1 = (a.astype(np.float32).astype(np.float64) * 2.0**-32 + 2.0**-33).astype(np.float32).astype(np.float64)
        # th = fma(float(b), float(2 pi 2^-32), float(2 pi 2^-33 - pi)) in FP32
        c1 = np.float64(np.float32(2 * np.pi * 2.0**-32))
        c2 = np.float64(np.float32(2 * np.pi * 2.0**-33 - np.pi))
        th = (b.astype(np.float32).astype(np.float64) * c1 + c2).astype(np.float32).astype(np.float64)
        r = np.sqrt(np.maximum(0.0, -2.0 * np.log(u1)))
    else:
        u1 = (a + 0.5) * 2.0**-32
        u2 = (b + 0.5) * 2.0**-32
        th = 2.0 * np.pi * u2 - np.pi
        r = np.sqrt(-2.0 * np.log(u1))
    return r * np.cos(th) + 1j * r * np.sin(th)


def kstep_table(nx: int, ny: int, J: float) -> np.ndarray:
    """k_step_linear of TWMCBaseSolver::Setup (TWMCBaseSolver.cpp:78-88), row-major nx x ny."""
    fx = 0.0 if nx == 1 else 1.0
    fy = 0.0 if ny == 1 else 1.0
    i = np.arange(nx)[:, None]
    j = np.arange(ny)[None, :]
    return -1j * 2.0 * J * (fx * np.cos(2 * np.pi / nx * i) + fy * np.cos(2 * np.pi / ny * j))


def base_run(nx, ny, J, gamma, dt, t_start, t_end, frame_steps, n_frames, store_initial, omega, U, F, beta0,
             xi=None, seed=0, tid=0, noise="buffer", integrator="euler"):
    """One trajectory of the 1-D/2-D solver; returns (frames, beta_final, t_final, steps).
    integrator "split": the engine's optional exponential split step, beta' =
    ifft2(exp(k_step dt) fft2(beta)), then the local step on beta'."""
    n = nx * ny
    beta = np.array(beta0, dtype=np.complex128).reshape(nx, ny)
    rsl = (-1j * np.broadcast_to(np.asarray(omega), (n,)).reshape(nx, ny) - gamma / 2.0)
    U = np.broadcast_to(np.asarray(U), (n,)).reshape(nx, ny)
    F = np.broadcast_to(np.asarray(F), (n,)).reshape(nx, ny)
    ks = kstep_table(nx, ny, J)
    dt4 = np.sqrt(gamma * dt / 4.0)
    frames = []
    i_step = 0
    i_frame = 0
    if store_initial and n_frames > 0:
        frames.append(beta.copy())
        i_frame = 1
    t = t_start
    while t <= t_end:
        if integrator == "split":
            beta = np.fft.ifft2(np.exp(ks * dt) * np.fft.fft2(beta))
            hop = 0.0
        else:
            hop = np.fft.ifft2(ks * np.fft.fft2(beta))  # ifft2 includes the 1/N
        a = ((rsl + 1j * U * (np.abs(beta) ** 2 - 1.0)) * beta + hop + 1j * F) * dt
        if noise == "buffer":
            z = np.asarray(xi[i_step]).reshape(nx, ny)
        else:
            z = site_normals(seed, tid, i_step, 0, n, noise == "philox32").reshape(nx, ny)
        beta = beta + a + dt4 * z
        t += dt
        i_step += 1
        if i_step % frame_steps == 0 and i_frame < n_frames:
            frames.append(beta.copy())
            i_frame += 1
            if i_frame == n_frames:
                break
    return np.array(frames).reshape(len(frames), n), beta.reshape(n), t, i_step


def lieb_coupling(ncell: int, pbc: bool, J_AB: float, J_BC: float) -> np.ndarray:
    """Dense 3N x 3N coupling of TWMCLiebSolver::Setup (TWMCLiebSolver.cpp:52-85), duplicates summed."""
    n = 3 * ncell
    C = np.zeros((n, n))
    for i in range(ncell):
        C[3 * i, 3 * i + 1] += J_AB
        C[3 * i + 1, 3 * i] += J_AB
        C[3 * i + 1, 3 * i + 2] += J_BC
        C[3 * i + 2, 3 * i + 1] += J_BC
        if i == ncell - 1:
            if pbc:
                C[3 * i + 2, 1] += J_BC
                C[1, 3 * i + 2] += J_BC
            break
        C[3 * i + 2, 3 * (i + 1) + 1] += J_BC
        C[3 * (i + 1) + 1, 3 * i + 2] += J_BC
    return C


def lieb_run(ncell, pbc, J_AB, J_BC, detuning, gamma, dt, t_start, t_end, frame_steps, n_frames, store_initial,
             E, U, F, beta0, xi=None, seed=0, tid=0, noise="buffer", F_of_t=None):
    """One Lieb trajectory; F_of_t(t) -> per-site F overrides F when given."""
    n = 3 * ncell
    C = lieb_coupling(ncell, pbc, J_AB, J_BC)
    rsl = -1j * (-np.asarray(E) + detuning) - gamma / 2.0
    U = np.asarray(U)
    Fc = np.asarray(F, dtype=np.complex128)
    beta = np.array(beta0, dtype=np.complex128)
    dt4 = np.sqrt(gamma * dt / 4.0)
    frames = []
    i_step = 0
    i_frame = 0
    if store_initial and n_frames > 0:
        frames.append(beta.copy())
        i_frame = 1
    t = t_start
    while t <= t_end:
        if F_of_t is not None:
            Fc = F_of_t(t)
        a = ((rsl + 1j * U * (np.abs(beta) ** 2 - 1.0)) * beta - 1j * (beta @ C) + 1j * Fc) * dt
        if noise == "buffer":
            z = np.asarray(xi[i_step])
        else:
            z = site_normals(seed, tid, i_step, 0, n, noise == "philox32")
        beta = beta + a + dt4 * z
        t += dt
        i_step += 1
        if i_step % frame_steps == 0 and i_frame < n_frames:
            frames.append(beta.copy())
            i_frame += 1
            if i_frame == n_frames:
                break
    return np.array(frames), beta, t, i_step


def ensemble_observables(frames: np.ndarray, nx: int, ny: int):
    """n_i, <a^+2 a^2>_i, g2_i and n_k from Wigner samples.

    frames: (T, F, N) complex. Returns dict of (F, N) arrays (FP64). The
    Wigner moments: <|a|^2>_W = <a^+a> + 1/2,
    <|a|^4>_W = <a^+2a^2> + 2<a^+a> + 1/2; n_k uses the unitary FFT.
    """
    f = np.asarray(frames, dtype=np.complex128)
    T = f.shape[0]
    ab2 = np.abs(f) ** 2
    m2 = ab2.mean(axis=0)
    m4 = (ab2 ** 2).mean(axis=0)
    n = m2 - 0.5
    a2a2 = m4 - 2.0 * m2 + 0.5
    fk = np.fft.fft2(f.reshape(T, f.shape[1], nx, ny)).reshape(f.shape) / np.sqrt(nx * ny)
    nk = (np.abs(fk) ** 2).mean(axis=0) - 0.5
    with np.errstate(divide="ignore", invalid="ignore"):
        g2 = a2a2 / n ** 2
    return {"n": n, "a2a2": a2a2, "g2": g2, "nk": nk, "m2": m2, "m4": m4}
