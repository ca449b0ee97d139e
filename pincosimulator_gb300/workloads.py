"""Named workloads of the GPU TWMC engine and a command line that runs one.

* ``square64``  -- 2-D 64x64 PBC, J=1, U=0.2, gamma=1, omega=-0.5 with
  Gaussian disorder of amplitude 0.2, F=2, dt=0.002, frames of 250 steps
  (the headline workload; ``--hop stencil`` for the real-space kernel).
* ``square128`` -- the same parameters on a 128x128 lattice (the 2-CTA
  cluster stencil kernel, power-of-two form).
* ``chain64``   -- the 1-D chain of 64 sites, J=1, U=0.1, gamma=1, omega=-1,
  F=1.5, beta_init_sigma=0.5, dt=0.005, a frame every 100 steps: the
  configuration of the reference's own CPU runs (1000 trajectories to
  t = 50 there). Timed through ``twmc_run`` with every frame saved.
* ``batch256``  -- the 256-point heterogeneous batch (chains of 32..1024
  sites and 16..128 square lattices, 512..4096 trajectories per point,
  autotuned step variants), timed with CUDA events.
* ``lieb768``   -- the 1-D Lieb lattice of 256 cells (768 sites), PBC,
  J_AB=J_BC=1, gamma=1, U=0.27 with uniform disorder of amplitude 0.06, and a
  drive F(t) on the B sites ramping from 0 to 2.5 over t in [0, 40] in
  records every 0.01, then held (the configuration of
  ``TWMCLiebSolver``'s F(t) runs).

``python -m pincosimulator_gb300.workloads lieb768 --ntraj 2048 --frames 1``
runs ``twmc_run`` over the given number of frames (after one untimed call)
and prints the kernel, the wall time and the site-updates per second as one
JSON line; square workloads are stepped through the device-resident batch
API and timed with CUDA events on the library's stream.
"""
import argparse
import json
import time

import numpy as np

from . import twmc

DT = 0.002
FRAME_STEPS = 250


def square(nx, ny, hop=twmc.HOP_FFT, precision=twmc.PREC_F32, n_moment_blocks=32, integrator=twmc.INTEGRATOR_EULER):
    return twmc.System(nx=nx, ny=ny, J=1.0, gamma=1.0, dt=DT, frame_steps=FRAME_STEPS,
                       omega=twmc.Noisy(-0.5, twmc.DISORDER_GAUSSIAN, 0.2), U=0.2, F=2.0, beta_init=0.0,
                       beta_init_sigma=0.5, precision=precision, hop=hop, n_moment_blocks=n_moment_blocks,
                       integrator=integrator)


def lieb(ncell=256):
    n = 3 * ncell
    times = np.round(np.arange(0, 40 + 1e-9, 0.01), 10)
    vals = np.zeros((len(times), n), dtype=complex)
    vals[:, 1::3] = (2.5 * times / 40.0)[:, None]
    return twmc.System(lattice=twmc.LATTICE_LIEB, nx=1, ny=ncell, pbc=True, J_AB=1.0, J_BC=1.0, gamma=1.0,
                       detuning=0.0, dt=DT, frame_steps=FRAME_STEPS, omega=0.0,
                       U=twmc.Noisy(0.27, twmc.DISORDER_UNIFORM, 0.06), F=0.0, F_t=(times, vals),
                       beta_init_sigma=0.5)


def chain64(hop=twmc.HOP_FFT):
    return twmc.System(nx=1, ny=64, J=1.0, gamma=1.0, dt=0.005, frame_steps=100, omega=-1.0, U=0.1, F=1.5,
                       beta_init=0.0, beta_init_sigma=0.5, hop=hop)


def batch_points(seed=3, traj_scale=1.0):
    """The heterogeneous-batch workload: 256 parameter points, each a chain of
    32..1024 sites or an L x L lattice (L = 16..128), U ~ U[0.05, 0.5],
    detuning ~ U[-2, 2], F ~ U[0, 3], J = gamma = 1, 512..4096 trajectories
    (uniform in log; times traj_scale, at least 1), dt = 0.002."""
    rng = np.random.default_rng(seed)
    kinds = [(1, n) for n in (32, 64, 128, 256, 512, 1024)] + [(l, l) for l in (16, 32, 64, 128)]
    pts = []
    for _ in range(256):
        nx, ny = kinds[rng.integers(len(kinds))]
        u, om, f = rng.uniform(0.05, 0.5), rng.uniform(-2, 2), rng.uniform(0, 3)
        nt = int(np.exp(rng.uniform(np.log(512), np.log(4096))))
        pts.append(dict(nx=nx, ny=ny, U=u, omega=om, F=f, dt=DT, n_traj=max(1, int(nt * traj_scale)),
                        seed0=int(rng.integers(1, 2 ** 31)), id0=1))
    return pts


def time_hbatch(points, frames, tune=True):
    """Device time (CUDA events) of `frames` frames of a heterogeneous batch
    after one untimed frame; returns (seconds, total site-trajectories, plans)."""
    hb = twmc.HBatch(points, FRAME_STEPS, tune=tune)
    plans = [hb.plan(i) for i in range(len(points))]
    hb.run(1)
    hb.sync()
    hb.run(frames)
    ms = hb.sync()
    hb.close()
    return ms / 1e3, sum(p["nx"] * p["ny"] * p["n_traj"] for p in points), plans


def time_run(sysd, ntraj, frames, save=False):
    """Wall time of one twmc_run call of `frames` frames (after an untimed
    call); with `save`, every frame and the final field are returned."""
    tasks = sysd.make_tasks(ntraj, t_end=frames * sysd.desc.frame_steps * sysd.desc.dt, store_initial=save)
    sysd.run(tasks, frames=save, final=save)
    t0 = time.perf_counter()
    res = sysd.run(tasks, frames=save, final=save)
    return time.perf_counter() - t0, bool(np.all(res["status"] == 0))


def time_batch(sysd, ntraj, frames):
    """CUDA-event time of `frames` frames stepped through the batch API (after one untimed frame)."""
    import torch

    sysd.batch_init(sysd.make_tasks(ntraj, t_end=100.0))
    sysd.advance(FRAME_STEPS)
    sysd.sync()
    ext = torch.cuda.ExternalStream(sysd.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(ext)
    for _ in range(frames):
        sysd.advance(FRAME_STEPS)
    e1.record(ext)
    sysd.sync()
    return e0.elapsed_time(e1) / 1e3


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("workload", choices=["square64", "square128", "lieb768", "chain64", "batch256"])
    ap.add_argument("--traj-scale", type=float, default=1.0, help="batch256: trajectories per point x this")
    ap.add_argument("--ntraj", type=int, default=2048)
    ap.add_argument("--frames", type=int, default=1)
    ap.add_argument("--hop", choices=["fft", "stencil"], default="stencil")
    ap.add_argument("--integrator", choices=["euler", "split"], default="euler",
                    help="square64 / square128 with --hop fft: the step's integrator")
    args = ap.parse_args(argv)
    if args.workload == "batch256":
        el, sites, plans = time_hbatch(batch_points(traj_scale=args.traj_scale), args.frames)
        print(json.dumps({"workload": "batch256", "traj_scale": args.traj_scale, "frames": args.frames,
                          "seconds": el, "site_updates_per_s": sites * FRAME_STEPS * args.frames / el,
                          "variants": sorted(set(p.split("<")[1].split(" ")[0] for p in plans))}), flush=True)
        return
    if args.workload == "lieb768":
        sysd = lieb()
        el, finite = time_run(sysd, args.ntraj, args.frames)
    elif args.workload == "chain64":
        sysd = chain64(hop=twmc.HOP_STENCIL if args.hop == "stencil" else twmc.HOP_FFT)
        el, finite = time_run(sysd, args.ntraj, args.frames, save=True)
    else:
        L = 64 if args.workload == "square64" else 128
        sysd = square(L, L, hop=twmc.HOP_STENCIL if args.hop == "stencil" else twmc.HOP_FFT,
                      integrator=twmc.INTEGRATOR_SPLIT if args.integrator == "split" else twmc.INTEGRATOR_EULER)
        el, finite = time_batch(sysd, args.ntraj, args.frames), True
    line = {"workload": args.workload, "ntraj": args.ntraj, "frames": args.frames, "kernel": sysd.kernel_name,
            "seconds": el, "site_updates_per_s": sysd.n_sites * args.ntraj * args.frames * sysd.desc.frame_steps / el,
            "finite": finite}
    sysd.close()
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
