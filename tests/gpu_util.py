"""Helpers for the GPU parity tests (run the C ABI and the oracle side by side)."""
import numpy as np

from pincosimulator_gb300 import twmc

TOL = {twmc.PREC_F32: 1e-5, twmc.PREC_F64: 1e-12}


def rel_err(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


def square_case(orc, nx, ny, *, ntraj=3, steps=200, dt=0.005, frame_steps=50, J=1.0, gamma=1.0, omega=-0.5,
                U=0.2, F=1.5, prec=twmc.PREC_F32, hop=twmc.HOP_FFT, seed=0, amp=0.4, integrator="euler"):
    """Deterministic-noise run of ntraj trajectories: returns (gpu result, oracle results)."""
    n = nx * ny
    rng = np.random.default_rng(seed + 1000 * nx + ny)
    beta0 = amp * (rng.normal(size=(ntraj, n)) + 1j * rng.normal(size=(ntraj, n)))
    xi = rng.normal(size=(ntraj, steps + 1, n)) + 1j * rng.normal(size=(ntraj, steps + 1, n))
    t_end = steps * dt
    n_frames = int(round(t_end / (dt * frame_steps))) + 1
    refs = [orc.base_run(nx, ny, J, gamma, dt, 0.0, t_end, frame_steps, n_frames, True, omega, U, F, beta0[k],
                         xi=xi[k], integrator=integrator) for k in range(ntraj)]
    S = refs[0]["steps"]
    sysd = twmc.System(nx=nx, ny=ny, J=J, gamma=gamma, dt=dt, frame_steps=frame_steps, omega=omega, U=U, F=F,
                       precision=prec, noise=twmc.NOISE_BUFFER, hop=hop,
                       integrator={"euler": twmc.INTEGRATOR_EULER, "split": twmc.INTEGRATOR_SPLIT}[integrator])
    tasks = sysd.make_tasks(ntraj, t_start=0.0, t_end=t_end, ic=twmc.IC_GIVEN, init_field=beta0)
    sysd.set_noise(xi[:, :S])
    res = sysd.run(tasks, frames=True)
    res["kernel"] = sysd.kernel_name
    sysd.close()
    return res, refs


def lieb_case(orc, ncell, *, pbc=True, ntraj=3, steps=200, dt=0.002, frame_steps=50, J_AB=1.0, J_BC=1.0,
              detuning=0.0, gamma=1.0, E=0.0, U=0.27, F=0.0, F_t=None, prec=twmc.PREC_F32, seed=0):
    n = 3 * ncell
    rng = np.random.default_rng(seed + ncell)
    beta0 = 0.5 * (rng.normal(size=(ntraj, n)) + 1j * rng.normal(size=(ntraj, n)))
    xi = rng.normal(size=(ntraj, steps + 1, n)) + 1j * rng.normal(size=(ntraj, steps + 1, n))
    t_end = steps * dt
    n_frames = int(round(t_end / (dt * frame_steps))) + 1
    refs = [orc.lieb_run(ncell, pbc, J_AB, J_BC, detuning, gamma, dt, 0.0, t_end, frame_steps, n_frames, True,
                         E, U, F, beta0[k], xi=xi[k], F_t=F_t) for k in range(ntraj)]
    S = refs[0]["steps"]
    sysd = twmc.System(lattice=twmc.LATTICE_LIEB, nx=1, ny=ncell, pbc=pbc, J_AB=J_AB, J_BC=J_BC, gamma=gamma,
                       detuning=detuning, dt=dt, frame_steps=frame_steps, omega=E, U=U, F=F, F_t=F_t,
                       precision=prec, noise=twmc.NOISE_BUFFER)
    tasks = sysd.make_tasks(ntraj, t_start=0.0, t_end=t_end, ic=twmc.IC_GIVEN, init_field=beta0)
    sysd.set_noise(xi[:, :S])
    res = sysd.run(tasks, frames=True)
    res["kernel"] = sysd.kernel_name
    sysd.close()
    return res, refs


def check(res, refs, prec):
    tol = TOL[prec]
    for k, ref in enumerate(refs):
        assert res["frames_written"][k] == ref["frames_written"]
        assert res["t_final"][k] == ref["t_final"]
        assert res["status"][k] == 0
        e = rel_err(res["final"][k], ref["final"])
        assert e < tol, f"traj {k}: final rel err {e:.3e} > {tol}"
        fw = ref["frames_written"]
        e = rel_err(res["frames"][k, :fw], ref["frames"][:fw])
        assert e < tol, f"traj {k}: frames rel err {e:.3e} > {tol}"


def philox_ref(orc, prec, seed, tid, steps, n, **run):
    """Oracle run of one Philox-mode trajectory: FP64 runs draw the oracle's
    own FP64 Philox stream; FP32 runs replay the device's normals
    (twmc_debug_wiener: the same Philox words through the FP32 Box-Muller with
    hardware log / sin / cos) in deterministic-noise mode, so the comparison
    holds the step arithmetic to the FP32 parity tolerance."""
    if prec == twmc.PREC_F64:
        return orc.base_run(**run, seed=seed, tid=tid, noise="philox64")
    xi = twmc.debug_wiener(twmc.PREC_F32, seed, tid, steps, n)
    return orc.base_run(**run, xi=xi)
