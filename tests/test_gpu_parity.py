"""GPU parity against the oracle through the C ABI (deterministic-noise mode).

Tolerances: FP32 state/FFT 1e-5 normwise relative, FP64 mode 1e-12, on
short horizons (200 Euler steps), as the deterministic-noise criterion
states.
"""
import numpy as np
import pytest

from pincosimulator_gb300 import twmc

from gpu_util import check, lieb_case, philox_ref, rel_err, square_case

pytestmark = pytest.mark.gpu

FFT_SHAPES = [(1, 32), (1, 64), (1, 128), (1, 256), (1, 512), (1, 1024), (1, 2048), (1, 4096), (16, 16), (32, 32),
              (64, 64)]


@pytest.mark.parametrize("prec", [twmc.PREC_F32, twmc.PREC_F64])
@pytest.mark.parametrize("shape", FFT_SHAPES)
def test_square_fft_parity(built_lib, oracle, shape, prec):
    nx, ny = shape
    ntraj = 2 if nx * ny >= 4096 else 5
    res, refs = square_case(oracle, nx, ny, ntraj=ntraj, prec=prec)
    assert res["kernel"] == "square_fft_kernel"
    check(res, refs, prec)


@pytest.mark.parametrize("prec", [twmc.PREC_F32, twmc.PREC_F64])
@pytest.mark.parametrize("shape", [(1, 1), (1, 2), (2, 2), (1, 50), (6, 10), (4, 8), (64, 64), (1, 64), (3, 128)])
def test_square_stencil_parity(built_lib, oracle, shape, prec):
    nx, ny = shape
    res, refs = square_case(oracle, nx, ny, ntraj=3, prec=prec, hop=twmc.HOP_STENCIL)
    assert res["kernel"].startswith("ell_kernel")
    check(res, refs, prec)


@pytest.mark.parametrize("shape,kernel", [((128, 128), "ell_cluster_pow2_kernel"), ((64, 256), "ell_cluster_pow2_kernel"),
                                          ((256, 64), "ell_cluster_pow2_kernel"), ((4, 4096), "ell_cluster_pow2_kernel"),
                                          ((96, 128), "ell_cluster_kernel"), ((99, 101), "ell_cluster_kernel"),
                                          ((1, 16384), "ell_cluster_kernel")])
def test_cluster_stencil_parity(built_lib, oracle, shape, kernel):
    """Lattices above 8192 sites (FP32) run on a 2-CTA cluster kernel, the
    neighbours of the other CTA's quarters read through distributed shared
    memory; odd N leaves the last pair without its high site. Power-of-two
    lattices with every row inside one quarter (ny <= N / 4) take the
    bit-arithmetic form (one row per quarter at 4 x 4096)."""
    nx, ny = shape
    res, refs = square_case(oracle, nx, ny, ntraj=3, prec=twmc.PREC_F32, hop=twmc.HOP_STENCIL, steps=60,
                            frame_steps=20)
    assert res["kernel"] == kernel
    check(res, refs, twmc.PREC_F32)


@pytest.mark.parametrize("shape,site_omega", [((128, 128), False), ((128, 128), True), ((4, 4096), False),
                                              ((256, 64), True)])
def test_cluster_pow2_philox(built_lib, oracle, shape, site_omega):
    """Philox-mode runs on the fast power-of-two cluster kernel (noise and
    scalar U, F compiled in; omega per site allowed) against the oracle fed
    the device's Philox normals, 1e-5."""
    nx, ny = shape
    n = nx * ny
    ntraj, steps, dt = 2, 100, 0.005
    rng = np.random.default_rng(11)
    beta0 = 0.3 * (rng.normal(size=(ntraj, n)) + 1j * rng.normal(size=(ntraj, n)))
    omega = -0.5 + 0.2 * rng.normal(size=n) if site_omega else -0.5
    sysd = twmc.System(nx=nx, ny=ny, J=1.0, gamma=1.0, dt=dt, frame_steps=50, omega=omega, U=0.2, F=1.5,
                       precision=twmc.PREC_F32, noise=twmc.NOISE_PHILOX, hop=twmc.HOP_STENCIL)
    seeds = [21, 4242]
    tasks = sysd.make_tasks(ntraj, t_start=0.0, t_end=steps * dt, ic=twmc.IC_GIVEN, init_field=beta0, seeds=seeds,
                            id0=9)
    res = sysd.run(tasks, frames=False)
    kernel = sysd.kernel_name
    sysd.close()
    assert kernel == "ell_cluster_pow2_kernel"
    for k in range(ntraj):
        ref = philox_ref(oracle, twmc.PREC_F32, seeds[k], 9 + k, steps, n, nx=nx, ny=ny, J=1.0, gamma=1.0, dt=dt,
                         t_start=0.0, t_end=steps * dt, frame_steps=50, n_frames=3, store_initial=True, omega=omega,
                         U=0.2, F=1.5, beta0=beta0[k])
        assert rel_err(res["final"][k], ref["final"]) < 1e-5


@pytest.mark.parametrize("shape,site_omega", [((64, 64), True), ((64, 64), False), ((1, 4096), True),
                                              ((16, 256), False), ((256, 16), True), ((1024, 4), False)])
def test_rowrun_philox(built_lib, oracle, shape, site_omega):
    """FP32 Philox runs of the real-space stencil on 4096 sites take the
    row-run kernel (four sites along a row per thread; ny = 4 makes a run a
    whole row) and agree with the oracle fed the device's Philox normals."""
    nx, ny = shape
    n = nx * ny
    ntraj, steps, dt = 2, 60, 0.005
    rng = np.random.default_rng(21)
    beta0 = 0.3 * (rng.normal(size=(ntraj, n)) + 1j * rng.normal(size=(ntraj, n)))
    omega = -0.5 + 0.2 * rng.normal(size=n) if site_omega else -0.5
    sysd = twmc.System(nx=nx, ny=ny, J=1.0, gamma=1.0, dt=dt, frame_steps=50, omega=omega, U=0.2, F=1.5,
                       precision=twmc.PREC_F32, noise=twmc.NOISE_PHILOX, hop=twmc.HOP_STENCIL)
    seeds = [5, 77]
    tasks = sysd.make_tasks(ntraj, t_start=0.0, t_end=steps * dt, ic=twmc.IC_GIVEN, init_field=beta0, seeds=seeds,
                            id0=3)
    res = sysd.run(tasks, frames=False)
    kernel = sysd.kernel_name
    sysd.close()
    assert kernel == "rowrun_kernel"
    for k in range(ntraj):
        ref = philox_ref(oracle, twmc.PREC_F32, seeds[k], 3 + k, steps, n, nx=nx, ny=ny, J=1.0, gamma=1.0, dt=dt,
                         t_start=0.0, t_end=steps * dt, frame_steps=50, n_frames=2, store_initial=True, omega=omega,
                         U=0.2, F=1.5, beta0=beta0[k])
        assert rel_err(res["final"][k], ref["final"]) < 1e-5


def test_cluster_per_site_parameters(built_lib, oracle):
    rng = np.random.default_rng(6)
    n = 128 * 128
    omega = -0.5 + 0.2 * rng.normal(size=n)
    F = 1.0 + 0.3 * rng.normal(size=n) + 0.1j
    res, refs = square_case(oracle, 128, 128, ntraj=2, prec=twmc.PREC_F32, hop=twmc.HOP_STENCIL, omega=omega, F=F,
                            steps=40, frame_steps=20)
    assert res["kernel"] == "ell_cluster_pow2_kernel"
    check(res, refs, twmc.PREC_F32)


def test_nonpow2_falls_back_to_real_space(built_lib, oracle):
    res, refs = square_case(oracle, 6, 10, ntraj=2, prec=twmc.PREC_F32, hop=twmc.HOP_FFT)
    assert res["kernel"] == "ell_kernel<stencil>"
    check(res, refs, twmc.PREC_F32)


def test_per_site_parameters(built_lib, oracle):
    rng = np.random.default_rng(5)
    n = 32 * 32
    omega = -0.5 + 0.2 * rng.normal(size=n)
    U = 0.2 + 0.02j * rng.normal(size=n)
    F = 1.0 + 0.3 * rng.normal(size=n) + 0.1j
    for prec in (twmc.PREC_F32, twmc.PREC_F64):
        res, refs = square_case(oracle, 32, 32, ntraj=3, prec=prec, omega=omega, U=U, F=F)
        check(res, refs, prec)


@pytest.mark.parametrize("prec", [twmc.PREC_F32, twmc.PREC_F64])
@pytest.mark.parametrize("ncell,pbc,jab,jbc", [(256, True, 1.0, 1.0), (24, False, 1.0, 1.0), (1, True, 1.0, 1.0),
                                               (7, True, 1.0, 1.0), (2, True, 1.3, 0.7), (2, False, 1.3, 0.7),
                                               (30, True, 0.6, 1.4)])
def test_lieb_parity(built_lib, oracle, ncell, pbc, jab, jbc, prec):
    """An even number of cells runs the cell kernel (whole cells per thread),
    an odd number the neighbour-table kernel; J_AB != J_BC checks that each
    coupling lands on its bond."""
    rng = np.random.default_rng(ncell)
    E = 0.1 * rng.normal(size=3 * ncell)
    U = 0.27 + 0.06 * rng.random(size=3 * ncell)
    res, refs = lieb_case(oracle, ncell, pbc=pbc, prec=prec, E=E, U=U, F=0.3, detuning=0.5, J_AB=jab, J_BC=jbc)
    assert res["kernel"] == ("lieb_cell_kernel" if ncell % 2 == 0 else "ell_kernel<table>")
    check(res, refs, prec)


@pytest.mark.parametrize("prec", [twmc.PREC_F32, twmc.PREC_F64])
def test_lieb_time_dependent_drive(built_lib, oracle, prec):
    """C4-style drive: B sites only, linear ramp tabulated every 0.01, then held."""
    ncell = 256
    n = 3 * ncell
    times = np.round(np.arange(0, 0.25 + 1e-9, 0.01), 10)
    vals = np.zeros((len(times), n), dtype=complex)
    vals[:, 1::3] = (2.5 * times / 0.25)[:, None]
    res, refs = lieb_case(oracle, ncell, prec=prec, steps=200, dt=0.002, F_t=(times, vals))
    check(res, refs, prec)


@pytest.mark.parametrize("prec", [twmc.PREC_F32, twmc.PREC_F64])
@pytest.mark.parametrize("shape", [(8, 8), (1, 48)])
def test_thermo_work_and_area(built_lib, oracle, prec, shape):
    """Square lattice with a ramped F(t) (records every 0.01 s, then held) and
    the drive's work / area datasets, deterministic noise, against the oracle.
    dF/dt is computed from the table slope on the device and as the
    difference of consecutive F(t) in the oracle, so FP64 agrees to the
    conditioning of that difference (1e-9 normwise), FP32 to 1e-4."""
    nx, ny = shape
    n = nx * ny
    steps, dt, fs = 200, 0.002, 25
    t_end = steps * dt
    rng = np.random.default_rng(11 + n)
    times = np.round(np.arange(0, 0.3 + 1e-9, 0.01), 10)
    vals = np.outer(1.8 * times / 0.3, 1.0 + 0.2 * rng.random(n)).astype(complex)
    beta0 = 0.4 * (rng.normal(size=(3, n)) + 1j * rng.normal(size=(3, n)))
    xi = rng.normal(size=(3, steps + 1, n)) + 1j * rng.normal(size=(3, steps + 1, n))
    n_frames = int(round(t_end / (dt * fs))) + 1
    refs = [oracle.thermo_run(nx, ny, 1.0, 1.0, dt, 0.0, t_end, fs, n_frames, True, -0.5, 0.2, 0.0, beta0[k],
                              F_t=(times, vals), xi=xi[k]) for k in range(3)]
    S = refs[0]["steps"]
    sysd = twmc.System(nx=nx, ny=ny, J=1.0, gamma=1.0, dt=dt, frame_steps=fs, omega=-0.5, U=0.2, F=0.0,
                       F_t=(times, vals), precision=prec, noise=twmc.NOISE_BUFFER, thermo=True)
    tasks = sysd.make_tasks(3, t_start=0.0, t_end=t_end, ic=twmc.IC_GIVEN, init_field=beta0)
    sysd.set_noise(xi[:, :S])
    res = sysd.run(tasks, frames=True)
    assert sysd.kernel_name == "ell_kernel<stencil>"
    sysd.close()
    check(res, refs, prec)
    tol = 1e-9 if prec == twmc.PREC_F64 else 1e-4
    for k, ref in enumerate(refs):
        fw = ref["frames_written"]
        assert np.all(res["work"][k, 0] == 0) and np.all(res["area"][k, 0] == 0)
        for key in ("work", "area"):
            e = rel_err(res[key][k, :fw], ref[key])
            assert e < tol, f"traj {k} {key}: rel err {e:.3e} > {tol}"
