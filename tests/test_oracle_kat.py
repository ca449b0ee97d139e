"""Known-answer tests pinning the oracle (CPU only).

The reference cannot be built here and ships no golden outputs, so the
oracle is pinned by closed forms of the discrete Euler recursion and by an
independent numpy restatement (oracle/twmc_oracle.py).
"""
import numpy as np
import pytest

from oracle import twmc_oracle as npo


def test_frame_grid_configs(oracle):
    # C1: dt = 0.005, period 0.5, t_end = 50 -> 100 steps per frame, 100 frames + initial
    g = oracle.frame_grid(0.0, 50.0, 0.005, frames_period=0.5)
    assert g["frame_steps"] == 100 and g["nFramesTot"] == 100 and g["n_frames"] == 101
    g = oracle.frame_grid(0.0, 100.0, 0.002, frames_period=0.5)
    assert g["frame_steps"] == 250 and g["n_frames"] == 201
    g = oracle.frame_grid(0.0, 20.0, 0.01, frames_freq=1.0)  # SampleData/test-sim.ini
    assert g["frame_steps"] == 100 and g["n_frames"] == 21
    g = oracle.frame_grid(0.0, 700.0, 0.0005, frames_freq=0.5)  # SampleData/test-lieb.ini
    assert g["frame_steps"] == 4000 and g["n_frames"] == 351
    g = oracle.frame_grid(0.0, 10.0, 0.01, n_frames=20)  # n_frames back-support
    assert g["frame_steps"] == 50 and g["n_frames"] == 21


def test_single_site_linear_recursion(oracle):
    """N = 1, J = U = 0: beta_{n+1} = (1 + c dt) beta_n + i F dt + sqrt(g dt/4) xi_n, c = -i w - g/2."""
    rng = np.random.default_rng(3)
    w, g, F, dt, S = 0.7, 1.3, 0.4 + 0.2j, 0.01, 300
    xi = rng.normal(size=(S + 1, 1)) + 1j * rng.normal(size=(S + 1, 1))
    b0 = np.array([0.3 - 0.1j])
    r = oracle.base_run(1, 1, 0.0, g, dt, 0.0, S * dt, S, 2, True, w, 0.0, F, b0, xi=xi)
    c = -1j * w - g / 2
    b = b0[0]
    for n in range(r["steps"]):
        b = b + ((c + 0j) * b + 0.0 + 1j * F) * dt + np.sqrt(g * dt / 4) * xi[n, 0]
    assert abs(r["final"][0] - b) < 1e-13
    # mean of the noiseless recursion has the closed form
    z = 1 + c * dt
    r0 = oracle.base_run(1, 1, 0.0, g, dt, 0.0, S * dt, S, 2, True, w, 0.0, F, b0, xi=np.zeros_like(xi))
    Sx = r0["steps"]
    closed = z ** Sx * b0[0] + 1j * F * dt * (1 - z ** Sx) / (1 - z)
    assert abs(r0["final"][0] - closed) < 1e-12


@pytest.mark.parametrize("nx,ny,kx,ky", [(1, 64, 0, 5), (16, 16, 3, 7), (8, 32, 5, 1), (1, 12, 0, 2), (6, 10, 2, 3)])
def test_plane_wave_eigenmode(oracle, nx, ny, kx, ky):
    """U = gamma = F = omega = 0, no noise: a plane wave gains (1 - 2iJ (cos kx + cos ky) dt) per step."""
    J, dt, S = 0.8, 0.01, 50
    i, j = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    b0 = np.exp(2j * np.pi * (kx * i / nx + ky * j / ny)).reshape(-1)
    xi = np.zeros((S + 1, nx * ny), dtype=complex)
    r = oracle.base_run(nx, ny, J, 0.0, dt, 0.0, S * dt, S, 2, True, 0.0, 0.0, 0.0, b0, xi=xi)
    fx = 0.0 if nx == 1 else 1.0
    fy = 0.0 if ny == 1 else 1.0
    lam = 1 - 2j * J * (fx * np.cos(2 * np.pi * kx / nx) + fy * np.cos(2 * np.pi * ky / ny)) * dt
    assert np.abs(r["final"] - lam ** r["steps"] * b0).max() < 1e-11


@pytest.mark.parametrize("nx,ny,kx,ky", [(1, 64, 0, 5), (16, 16, 3, 7), (8, 32, 5, 1), (1, 12, 0, 2)])
def test_split_step_plane_wave(oracle, nx, ny, kx, ky):
    """Split-step integrator, U = gamma = F = omega = 0, no noise: a plane wave
    gains exactly exp(-2iJ (cos kx + cos ky) dt) per step (norm conserved)."""
    J, dt, S = 0.8, 0.01, 50
    i, j = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    b0 = np.exp(2j * np.pi * (kx * i / nx + ky * j / ny)).reshape(-1)
    xi = np.zeros((S + 1, nx * ny), dtype=complex)
    r = oracle.base_run(nx, ny, J, 0.0, dt, 0.0, S * dt, S, 2, True, 0.0, 0.0, 0.0, b0, xi=xi, integrator="split")
    fx = 0.0 if nx == 1 else 1.0
    fy = 0.0 if ny == 1 else 1.0
    th = 2 * J * (fx * np.cos(2 * np.pi * kx / nx) + fy * np.cos(2 * np.pi * ky / ny)) * dt
    assert np.abs(r["final"] - np.exp(-1j * th * r["steps"]) * b0).max() < 1e-11
    assert abs(np.abs(r["final"]).max() - 1.0) < 1e-12


@pytest.mark.parametrize("nx,ny", [(1, 64), (8, 8), (4, 16)])
def test_split_step_matches_numpy_restatement(oracle, nx, ny):
    """The C++ oracle's split step against the numpy twin (deterministic noise)."""
    rng = np.random.default_rng(nx * 7 + ny)
    n = nx * ny
    S = 60
    omega = rng.normal(size=n) * 0.3 - 0.5
    U = 0.2 + 0.05j * rng.normal(size=n)
    F = 1.0 + 0.3 * rng.normal(size=n)
    b0 = 0.5 * (rng.normal(size=n) + 1j * rng.normal(size=n))
    xi = rng.normal(size=(S + 1, n)) + 1j * rng.normal(size=(S + 1, n))
    a = oracle.base_run(nx, ny, 0.9, 1.1, 0.01, 0.0, S * 0.01, 20, 4, True, omega, U, F, b0, xi=xi,
                        integrator="split")
    fr, fin, t, steps = npo.base_run(nx, ny, 0.9, 1.1, 0.01, 0.0, S * 0.01, 20, 4, True, omega, U, F, b0, xi=xi,
                                     integrator="split")
    assert steps == a["steps"]
    scale = np.abs(fin).max()
    assert np.abs(a["final"] - fin).max() / scale < 1e-12
    assert np.abs(a["frames"] - fr).max() / scale < 1e-12
    # and it is a different integrator from the reference's Euler step
    e = oracle.base_run(nx, ny, 0.9, 1.1, 0.01, 0.0, S * 0.01, 20, 4, True, omega, U, F, b0, xi=xi)
    assert np.abs(a["final"] - e["final"]).max() / scale > 1e-6


def test_lieb_linear_matrix_power(oracle):
    """Noiseless linear Lieb chain against the explicit 3N x 3N propagator."""
    nc, JAB, JBC, det, g, dt, S = 5, 1.0, 0.7, 0.3, 0.9, 0.005, 120
    rng = np.random.default_rng(4)
    E = rng.normal(size=3 * nc)
    F = 0.5 * rng.normal(size=3 * nc) + 0.1j
    b0 = rng.normal(size=3 * nc) + 1j * rng.normal(size=3 * nc)
    for pbc in (True, False):
        C = npo.lieb_coupling(nc, pbc, JAB, JBC)
        r = oracle.lieb_run(nc, pbc, JAB, JBC, det, g, dt, 0.0, S * dt, S, 2, True, E, 0.0, F, b0,
                            xi=np.zeros((S + 1, 3 * nc)))
        rsl = -1j * (det - E) - g / 2
        Mx = np.eye(3 * nc) + dt * (np.diag(rsl) - 1j * C)  # row-vector propagator: b -> b M
        b = b0.astype(complex)
        for _ in range(r["steps"]):
            b = b @ Mx + 1j * F * dt
        assert np.abs(r["final"] - b).max() < 1e-12


@pytest.mark.parametrize("nx,ny", [(1, 64), (8, 8), (4, 16), (1, 50), (6, 10), (1, 1)])
def test_base_matches_numpy_restatement(oracle, nx, ny):
    rng = np.random.default_rng(nx * 100 + ny)
    n = nx * ny
    S = 60
    omega = rng.normal(size=n) * 0.3 - 0.5
    U = 0.2 + 0.05j * rng.normal(size=n)
    F = 1.0 + 0.3 * rng.normal(size=n)
    b0 = 0.5 * (rng.normal(size=n) + 1j * rng.normal(size=n))
    xi = rng.normal(size=(S + 1, n)) + 1j * rng.normal(size=(S + 1, n))
    a = oracle.base_run(nx, ny, 0.9, 1.1, 0.01, 0.0, S * 0.01, 20, 4, True, omega, U, F, b0, xi=xi)
    fr, fin, t, steps = npo.base_run(nx, ny, 0.9, 1.1, 0.01, 0.0, S * 0.01, 20, 4, True, omega, U, F, b0, xi=xi)
    assert steps == a["steps"]
    assert abs(t - a["t_final"]) == 0.0
    scale = np.abs(fin).max()
    assert np.abs(a["final"] - fin).max() / scale < 1e-12
    assert np.abs(a["frames"] - fr).max() / scale < 1e-12


@pytest.mark.parametrize("noise", ["philox64", "philox32"])
def test_philox_trajectory_matches_numpy(oracle, noise):
    nx, ny, S = 4, 8, 40
    n = nx * ny
    b0 = np.zeros(n, dtype=complex)
    a = oracle.base_run(nx, ny, 1.0, 1.0, 0.01, 0.0, S * 0.01, 10, 5, True, -0.5, 0.2, 1.0, b0, seed=9, tid=4,
                        noise=noise)
    fr, fin, t, steps = npo.base_run(nx, ny, 1.0, 1.0, 0.01, 0.0, S * 0.01, 10, 5, True, -0.5, 0.2, 1.0, b0,
                                     seed=9, tid=4, noise=noise)
    tol = 1e-6 if noise == "philox32" else 1e-12
    assert steps == a["steps"]
    assert np.abs(a["final"] - fin).max() < tol


def test_lieb_matches_numpy_with_time_table(oracle):
    nc, S, dt = 6, 80, 0.01
    n = 3 * nc
    rng = np.random.default_rng(12)
    times = np.array([0.0, 0.2, 0.35, 0.5])
    vals = rng.normal(size=(4, n)) + 0.3j * rng.normal(size=(4, n))
    vals[1, 4] = np.nan  # gap-filled by interpolation
    E = 0.1 * rng.normal(size=n)
    U = 0.3 + 0.01 * rng.normal(size=n)
    b0 = 0.5 * (rng.normal(size=n) + 1j * rng.normal(size=n))
    xi = rng.normal(size=(S + 1, n)) + 1j * rng.normal(size=(S + 1, n))
    a = oracle.lieb_run(nc, True, 1.0, 0.8, 0.2, 1.0, dt, 0.0, S * dt, 20, 5, True, E, U, 0.0, b0, xi=xi,
                        F_t=(times, vals))
    filled = vals.copy()
    filled[1, 4] = vals[0, 4] + (vals[2, 4] - vals[0, 4]) * (0.2 - 0.0) / (0.35 - 0.0)

    def F_of_t(t):
        if t <= times[0]:
            return filled[0]
        idx = np.searchsorted(times, t, side="left") - 1
        if idx >= len(times) - 1:
            return filled[-1]
        slope = (filled[idx + 1] - filled[idx]) / (times[idx + 1] - times[idx])
        return filled[idx] + (t - times[idx]) * slope

    fr, fin, t, steps = npo.lieb_run(nc, True, 1.0, 0.8, 0.2, 1.0, dt, 0.0, S * dt, 20, 5, True, E, U, 0.0, b0,
                                     xi=xi, F_of_t=F_of_t)
    assert steps == a["steps"]
    assert np.abs(a["final"] - fin).max() / np.abs(fin).max() < 1e-12


def test_time_table_semantics(oracle):
    times = [0.0, 1.0, 3.0]
    vals = np.array([[0.0, 1.0], [2.0, np.nan], [4.0, 5.0]], dtype=complex)
    out = oracle.time_table_eval(times, vals, [-1.0, 0.0, 0.5, 1.0, 2.0, 3.0, 10.0])
    # column 1 gap: 1 + (5-1) * (1-0)/(3-0)
    g = 1 + 4.0 / 3.0
    exp = np.array([[0, 1], [0, 1], [1, 1 + 0.5 * (g - 1)], [2, g], [3, g + 0.5 * (5 - g)], [4, 5], [4, 5]])
    assert np.abs(out - exp).max() < 1e-12


def test_thermo_single_site_recursion(oracle):
    """Work / area of a single site (no hopping, U = 0) with a ramp F(t) and
    given noise, against the recursion written out here."""
    dt, gamma, omega = 0.01, 1.0, -0.7
    times = np.array([0.0, 0.3, 0.8])
    vals = np.array([[0.0], [1.2 + 0.1j], [0.5]])
    steps, fs = 100, 10
    t_end = steps * dt - 1e-9
    rng = np.random.default_rng(4)
    xi = rng.normal(size=(steps + 2, 1)) + 1j * rng.normal(size=(steps + 2, 1))
    b0 = np.array([0.3 - 0.2j])
    r = oracle.thermo_run(1, 1, 0.0, gamma, dt, 0.0, t_end, fs, 11, True, omega, 0.0, 0.0, b0,
                          F_t=(times, vals), xi=xi)
    F = lambda t: np.interp(t, times, vals[:, 0].real) + 1j * np.interp(t, times, vals[:, 0].imag)
    b = b0[0]
    dt4 = np.sqrt(gamma * dt / 4)
    t = 0.0
    W = A = 0.0
    work, area, frames = [0.0], [0.0], [b]
    Fprev = F(0.0)
    for k in range(steps):
        Ft = F(t)
        b = b + ((-1j * omega - gamma / 2) * b + 1j * Ft) * dt + dt4 * xi[k, 0]
        fd = (Ft.real - Fprev.real) / dt
        Fprev = Ft
        W += 2 * dt * b.real * fd
        A += dt * fd * (abs(b) ** 2 - 0.5)
        t += dt
        if (k + 1) % fs == 0:
            frames.append(b)
            work.append(W)
            area.append(A)
            W = A = 0.0
    assert r["frames_written"] == 11
    assert np.allclose(r["frames"][:, 0], frames, rtol=0, atol=1e-12)
    assert np.allclose(r["work"][:, 0], work, rtol=0, atol=1e-12)
    assert np.allclose(r["area"][:, 0], area, rtol=0, atol=1e-12)
    assert abs(r["work"][1:, 0]).max() > 1e-3      # the ramp does work


def test_thermo_without_ramp_does_no_work(oracle):
    """A constant F(t) gives dF/dt = 0: no work, no area; the field equals the
    base run with the same constant F."""
    n = 16
    rng = np.random.default_rng(5)
    b0 = 0.3 * (rng.normal(size=n) + 1j * rng.normal(size=n))
    xi = rng.normal(size=(60, n)) + 1j * rng.normal(size=(60, n))
    Fc = 1.3 + 0.2j
    times = np.array([0.0, 1.0])
    vals = np.full((2, n), Fc)
    r = oracle.thermo_run(4, 4, 1.0, 1.0, 0.005, 0.0, 0.25, 10, 6, True, -0.5, 0.2, 0.0, b0, F_t=(times, vals), xi=xi)
    base = oracle.base_run(4, 4, 1.0, 1.0, 0.005, 0.0, 0.25, 10, 6, True, -0.5, 0.2, Fc, b0, xi=xi)
    assert np.array_equal(r["frames"], base["frames"])
    assert np.all(r["work"] == 0) and np.all(r["area"] == 0)
