"""GPU checks of the engine beyond single-trajectory parity: Philox noise,
initial fields and disorder, ensemble moments, status flags, full-size
properties."""
import numpy as np
import pytest

from oracle import twmc_oracle as npo
from pincosimulator_gb300 import twmc

from gpu_util import philox_ref, rel_err

pytestmark = pytest.mark.gpu


def test_gpu_philox_bit_exact(built_lib, oracle):
    rng = np.random.default_rng(2)
    ctr = rng.integers(0, 2**32, size=(4096, 4), dtype=np.uint64).astype(np.uint32)
    key = [0x9E3779B9, 0x7F4A7C15]
    assert np.array_equal(twmc.debug_philox(ctr, key), npo.philox4x32_10(ctr, np.broadcast_to(np.array(key, np.uint32), (4096, 2))))


@pytest.mark.parametrize("prec,tol", [(twmc.PREC_F64, 1e-12), (twmc.PREC_F32, 1e-5)])
@pytest.mark.parametrize("shape,hop", [((16, 16), twmc.HOP_FFT), ((1, 64), twmc.HOP_FFT), ((6, 10), twmc.HOP_STENCIL)])
def test_philox_noise_trajectories(built_lib, oracle, prec, tol, shape, hop):
    nx, ny = shape
    n = nx * ny
    ntraj, steps, dt = 3, 200, 0.005
    rng = np.random.default_rng(3)
    beta0 = 0.3 * (rng.normal(size=(ntraj, n)) + 1j * rng.normal(size=(ntraj, n)))
    sysd = twmc.System(nx=nx, ny=ny, J=1.0, gamma=1.0, dt=dt, frame_steps=50, omega=-0.5, U=0.2, F=1.5,
                       precision=prec, noise=twmc.NOISE_PHILOX, hop=hop)
    seeds = [17, 99, 12345]
    tasks = sysd.make_tasks(ntraj, t_start=0.0, t_end=steps * dt, ic=twmc.IC_GIVEN, init_field=beta0, seeds=seeds,
                            id0=5)
    res = sysd.run(tasks, frames=False)
    sysd.close()
    for k in range(ntraj):
        ref = philox_ref(oracle, prec, seeds[k], 5 + k, steps, n, nx=nx, ny=ny, J=1.0, gamma=1.0, dt=dt, t_start=0.0,
                         t_end=steps * dt, frame_steps=50, n_frames=5, store_initial=True, omega=-0.5, U=0.2, F=1.5,
                         beta0=beta0[k])
        assert rel_err(res["final"][k], ref["final"]) < tol


@pytest.mark.parametrize("prec,tol", [(twmc.PREC_F64, 1e-14), (twmc.PREC_F32, 1e-5)])
def test_initial_fields_and_disorder(built_lib, oracle, prec, tol):
    """ReadFromSettings initial fields and Gaussian / Uniform disorder draws:
    FP64 runs with the FP64 Box-Muller flavour (to 1e-14), FP32 runs with the
    FP32 one (hardware logarithm and sine / cosine: 1e-5; the initial field
    is then rounded to the FP32 state). Uniform draws are exact in both."""
    nx, ny, ntraj = 8, 8, 4
    n = nx * ny
    rng = np.random.default_rng(8)
    binit = 0.2 + 0.1j * rng.normal(size=n)
    bsig = 0.5 + 0.1 * rng.random(size=n)
    om_amp = 0.2 + 0.05j
    u_amp = 0.06 * np.ones(n)
    f_amp = 1.0 + 0.5j
    sysd = twmc.System(nx=nx, ny=ny, J=1.0, gamma=1.0, dt=0.01, frame_steps=1,
                       omega=twmc.Noisy(-0.5, twmc.DISORDER_GAUSSIAN, om_amp),
                       U=twmc.Noisy(0.27, twmc.DISORDER_UNIFORM, u_amp),
                       F=twmc.Noisy(2.0, twmc.DISORDER_GAUSSIAN, f_amp),
                       beta_init=binit, beta_init_sigma=bsig, precision=prec)
    tasks = sysd.make_tasks(ntraj, t_start=0.0, t_end=0.01, seed0=77, id0=3)
    res = sysd.run(tasks, frames=True, realizations=True)
    sysd.close()
    f32 = prec == twmc.PREC_F32
    for k in range(ntraj):
        seed, tid = 77 + k, 3 + k
        assert rel_err(res["frames"][k, 0], oracle.initial_field(n, binit, bsig, seed, tid, f32=f32)) < tol
        assert rel_err(res["U_realization"][k], oracle.disorder(n, 2, 0.27, u_amp, seed, tid, 2, f32=f32)) < 1e-14
        assert rel_err(res["omega_realization"][k], oracle.disorder(n, 1, -0.5, om_amp, seed, tid, 3, f32=f32)) < tol
        assert rel_err(res["F_realization"][k], oracle.disorder(n, 1, 2.0, f_amp, seed, tid, 4, f32=f32)) < tol
    if f32:  # the FP32 flavour differs from the FP64 one by more than FP64 rounding
        assert rel_err(res["omega_realization"][0], oracle.disorder(n, 1, -0.5, om_amp, 77, 3, 3)) > 1e-12


def test_disordered_trajectories_match_oracle(built_lib, oracle):
    """C2-style omega disorder: the drawn realisation drives the trajectory (FP64, Philox)."""
    nx = ny = 16
    n = nx * ny
    ntraj, steps, dt = 3, 100, 0.002
    sysd = twmc.System(nx=nx, ny=ny, J=1.0, gamma=1.0, dt=dt, frame_steps=50,
                       omega=twmc.Noisy(-0.5, twmc.DISORDER_GAUSSIAN, 0.2), U=0.2, F=2.0, beta_init=0.0,
                       beta_init_sigma=0.5, precision=twmc.PREC_F64)
    tasks = sysd.make_tasks(ntraj, t_start=0.0, t_end=steps * dt, seed0=5, id0=1)
    res = sysd.run(tasks, frames=True, realizations=True)
    sysd.close()
    for k in range(ntraj):
        b0 = res["frames"][k, 0]
        ref = oracle.base_run(nx, ny, 1.0, 1.0, dt, 0.0, steps * dt, 50, 3, True, res["omega_realization"][k], 0.2,
                              2.0, b0, seed=5 + k, tid=1 + k, noise="philox64")
        assert rel_err(res["final"][k], ref["final"]) < 1e-12


def test_moments_match_frames(built_lib, oracle):
    nx = ny = 16
    n = nx * ny
    ntraj, nb = 40, 8
    sysd = twmc.System(nx=nx, ny=ny, J=1.0, gamma=1.0, dt=0.005, frame_steps=20, omega=-0.5, U=0.2, F=1.0,
                       beta_init_sigma=0.5, precision=twmc.PREC_F64, n_moment_blocks=nb)
    tasks = sysd.make_tasks(ntraj, t_start=0.0, t_end=0.2, seed0=1)
    res = sysd.run(tasks, frames=True, moments=True)
    sysd.close()
    fr = res["frames"]  # (T, F, N)
    for f in range(fr.shape[1]):
        for b in range(nb):
            t0, t1 = b * ntraj // nb, (b + 1) * ntraj // nb
            x = fr[t0:t1, f]
            ab2 = np.abs(x) ** 2
            fk = np.fft.fft2(x.reshape(-1, nx, ny)).reshape(-1, n) / np.sqrt(n)
            assert np.allclose(res["moments"][f, b, :, 0], ab2.sum(0), rtol=1e-12, atol=1e-12)
            assert np.allclose(res["moments"][f, b, :, 1], (ab2 ** 2).sum(0), rtol=1e-12, atol=1e-12)
            # n_k is stored at natural k order
            assert np.allclose(res["moments"][f, b, :, 2], (np.abs(fk) ** 2).sum(0), rtol=1e-10, atol=1e-10)


def test_fp32_moments_float_float(built_lib):
    """FP32 states: the float-float block sums equal FP64 sums of the
    downloaded (exactly widened) fields to 1e-12 relative, over amplitudes
    spread across seven decades and with one site whose |a|^2 >= 2^60 takes
    the FP64 branch."""
    nx = ny = 8
    n = nx * ny
    ntraj, nb = 300, 3
    rng = np.random.default_rng(4)
    b0 = (rng.normal(size=(ntraj, n)) + 1j * rng.normal(size=(ntraj, n))) * np.exp(rng.uniform(-8, 8, (ntraj, n)))
    b0[5, 3] = 3e9 + 1e9j
    sysd = twmc.System(nx=nx, ny=ny, J=1.0, gamma=1.0, dt=0.005, frame_steps=1, omega=-0.5, U=0.0, F=0.0,
                       precision=twmc.PREC_F32, n_moment_blocks=nb, hop=twmc.HOP_STENCIL)
    tasks = sysd.make_tasks(ntraj, t_start=0.0, t_end=0.005, ic=twmc.IC_GIVEN, init_field=b0)
    res = sysd.run(tasks, frames=True, moments=True)
    sysd.close()
    x = res["frames"][:, 0]
    assert np.array_equal(x, b0.astype(np.complex64).astype(np.complex128))
    for b in range(nb):
        t0, t1 = b * ntraj // nb, (b + 1) * ntraj // nb
        ab2 = x[t0:t1].real ** 2 + x[t0:t1].imag ** 2
        assert np.allclose(res["moments"][0, b, :, 0], ab2.sum(0), rtol=1e-12, atol=0)
        assert np.allclose(res["moments"][0, b, :, 1], (ab2 ** 2).sum(0), rtol=1e-12, atol=0)


def test_nonfinite_status_flag(built_lib):
    """A NaN injected into one trajectory's host noise is reported in its status only."""
    nx = ny = 16
    n = nx * ny
    ntraj, steps, dt = 3, 20, 0.01
    xi = np.zeros((ntraj, steps, n), dtype=complex)
    xi[1, 7, 5] = np.nan
    sysd = twmc.System(nx=nx, ny=ny, J=1.0, gamma=1.0, dt=dt, frame_steps=10, omega=0.0, U=0.1, F=0.5,
                       noise=twmc.NOISE_BUFFER)
    tasks = sysd.make_tasks(ntraj, t_start=0.0, t_end=steps * dt, ic=twmc.IC_GIVEN,
                            init_field=np.zeros((ntraj, n)))
    sysd.set_noise(xi)
    res = sysd.run(tasks, frames=False)
    sysd.close()
    assert list(res["status"]) == [0, twmc.ERR_NONFINITE, 0]


def test_invalid_arguments_rejected(built_lib):
    with pytest.raises(twmc.TWMCError):
        twmc.System(nx=0, ny=4)
    with pytest.raises(twmc.TWMCError):
        twmc.System(lattice=twmc.LATTICE_LIEB, nx=4, ny=4)
    sysd = twmc.System(nx=4, ny=4, dt=0.01, noise=twmc.NOISE_BUFFER)
    tasks = sysd.make_tasks(2, t_end=0.1, ic=twmc.IC_GIVEN, init_field=np.zeros((2, 16)))
    with pytest.raises(twmc.TWMCError):
        sysd.run(tasks)  # no noise buffer supplied
    sysd.set_noise(np.zeros((2, 3, 16)))
    with pytest.raises(twmc.TWMCError):
        sysd.run(tasks)  # too short
    sysd.close()


def test_full_size_fft_equals_stencil(built_lib):
    """C2 size (16384 trajectories of 64 x 64, FP32, Philox): the k-space
    (FFT) and real-space kernels apply the same operator; after 50 steps the
    fields agree to FP32 rounding, and the FP64 moment blocks sum to the
    downloaded fields' moments."""
    nx = ny = 64
    ntraj = 16384
    kw = dict(nx=nx, ny=ny, J=1.0, gamma=1.0, dt=0.002, frame_steps=250, U=0.2, F=2.0,
              omega=twmc.Noisy(-0.5, twmc.DISORDER_GAUSSIAN, 0.2), beta_init_sigma=0.5, precision=twmc.PREC_F32)
    out = {}
    for hop in (twmc.HOP_FFT, twmc.HOP_STENCIL):
        sysd = twmc.System(hop=hop, **kw)
        tasks = sysd.make_tasks(ntraj, t_start=0.0, t_end=100.0, seed0=2024)
        sysd.batch_init(tasks)
        sysd.advance(50)
        sysd.reduce()
        sysd.sync()
        out[hop] = sysd.download(field=True, moments=True)
        sysd.close()
    fa, ma = out[twmc.HOP_FFT]
    fb, mb = out[twmc.HOP_STENCIL]
    assert np.isfinite(fa).all()
    assert rel_err(fa, fb) < 1e-4
    assert np.allclose(ma[:, :, 0].sum(0), (np.abs(fa) ** 2).sum(0), rtol=1e-9)


def test_run_interleaved_groups_and_pinned_buffers(built_lib):
    """Tasks of two horizons interleaved in one call form two groups whose
    output rows are not consecutive (the copy-through-host path); each group
    equals a call of its tasks alone (consecutive rows: strided asynchronous
    copies), into pageable and into pinned result arrays alike."""
    import torch
    s = twmc.System(nx=16, ny=16, J=1.0, gamma=1.0, dt=0.002, frame_steps=25,
                    omega=twmc.Noisy(-0.5, twmc.DISORDER_GAUSSIAN, 0.2), U=0.2, F=1.5, beta_init_sigma=0.5)
    tasks = s.make_tasks(40, t_end=0.1, seed0=3, store_initial=True)
    for k in range(1, 40, 2):
        tasks[k].t_end = 0.05
    both = s.run(tasks, frames=True, final=True, moments=False)
    for sel, nf in ((slice(0, 40, 2), 3), (slice(1, 40, 2), 2)):
        sub = s.make_tasks(20, t_end=0.1, seed0=3, store_initial=True)
        for j, k in enumerate(range(40)[sel]):
            sub[j].seed, sub[j].id, sub[j].t_end = tasks[k].seed, tasks[k].id, tasks[k].t_end
        alone = s.run(sub, frames=True, final=True)
        assert alone["frames"].shape == (20, nf, 256)
        assert np.array_equal(both["final"][sel], alone["final"])
        assert np.array_equal(both["frames"][sel, :nf], alone["frames"])
        pinned = {"final": torch.empty((20, 256), dtype=torch.complex128, pin_memory=True).numpy(),
                  "frames": torch.empty((20, nf, 256), dtype=torch.complex128, pin_memory=True).numpy()}
        got = s.run(sub, frames=True, final=True, buffers=pinned)
        assert np.array_equal(got["final"], alone["final"])
        assert np.array_equal(got["frames"], alone["frames"])
    s.close()


def test_run_final_field_pipeline(built_lib):
    """Runs of at least 2^20 sites stage saved frames on a second stream and
    send the final field through the pipeline (the last steps in four
    trajectory ranges, each range copied to the host while the next
    computes): equal to the last saved frame, to the same
    trajectories stepped through the batch API, and into pinned arrays; a
    run shorter than half a frame saves no frame and pipelines its trailing
    steps."""
    import torch
    s = twmc.System(nx=32, ny=32, J=1.0, gamma=1.0, dt=0.002, frame_steps=25,
                    omega=twmc.Noisy(-0.5, twmc.DISORDER_GAUSSIAN, 0.2), U=0.2, F=1.5, beta_init_sigma=0.5)
    n = 1030
    tasks = s.make_tasks(n, t_end=0.1, seed0=11, store_initial=False)
    a = s.run(tasks, frames=True, final=True, moments=True)
    assert np.array_equal(a["final"], a["frames"][:, -1])
    pinned = {"final": torch.empty((n, 1024), dtype=torch.complex128, pin_memory=True).numpy(),
              "frames": torch.empty((n, 2, 1024), dtype=torch.complex128, pin_memory=True).numpy()}
    b = s.run(tasks, frames=True, final=True, buffers=pinned)
    assert np.array_equal(b["final"], a["final"]) and np.array_equal(b["frames"], a["frames"])
    # saved frames (staged on the second stream) against the batch API
    s.batch_init(tasks)
    for f in range(2):
        s.advance(25)
        s.sync()
        field, _ = s.download(field=True, moments=False)
        assert np.array_equal(a["frames"][:, f], field), f
    for t_end in (0.1, 0.02):
        t2 = s.make_tasks(n, t_end=t_end, seed0=11, store_initial=False)
        c = s.run(t2, frames=False, final=True)
        steps = int(round(c["t_final"][0] / 0.002))
        assert steps == (50 if t_end == 0.1 else 10)
        s.batch_init(t2)
        s.advance(steps)
        s.sync()
        field, _ = s.download(field=True, moments=False)
        assert np.array_equal(c["final"], field), t_end
    s.close()


def test_run_into_caller_buffers(built_lib):
    """run() writes into caller-provided result arrays (reused across calls,
    e.g. pinned memory) exactly what it returns in arrays of its own; the
    FP32 field arrives widened to complex128 (chunked on the GPU)."""
    s = twmc.System(nx=32, ny=32, J=1.0, gamma=1.0, dt=0.002, frame_steps=25,
                    omega=twmc.Noisy(-0.5, twmc.DISORDER_GAUSSIAN, 0.2), U=0.2, F=1.5, beta_init_sigma=0.5)
    tasks = s.make_tasks(300, t_end=0.1, seed0=9, store_initial=False)
    ref = s.run(tasks, frames=True, final=True, moments=True)
    bufs = {"final": np.full((300, 1024), np.nan + 0j), "moments": np.full(ref["moments"].shape, np.nan),
            "frames": np.full(ref["frames"].shape, np.nan + 0j)}
    for _ in range(2):
        got = s.run(tasks, frames=True, final=True, moments=True, buffers=bufs)
        for k in ("final", "moments", "frames"):
            assert got[k] is bufs[k] and np.array_equal(got[k], ref[k]), k
    assert np.array_equal(ref["final"], ref["frames"][:, -1])
    with pytest.raises(ValueError):
        s.run(tasks, final=True, frames=False, buffers={"final": np.zeros((300, 1024), np.complex64)})
    s.close()
