#!/usr/bin/env python3
"""Benchmark of the TWMC trajectory engine on the 2-D 64 x 64 workload.

Workload (the headline configuration): 2-D square lattice 64 x 64, PBC,
J = 1, U = 0.2, gamma = 1, omega_i = -0.5 + N(0, 0.2^2) site disorder drawn
per trajectory, F = 2.0, vacuum Wigner start (beta_init = 0, sigma = 0.5),
dt = 0.002, frames every 0.5 (250 steps), 16384 trajectories, complex64
state and FFT, FP64 ensemble moments. Synthetic inputs, seeded.

One bench step = one frame of the whole batch: 250 Euler-Maruyama steps of
all 16384 trajectories (on-chip FFT hopping) plus the FP64 reduction of the
frame's moments. The state (512 MB) is larger than L2, so every launch
streams it from HBM.

Metric: site-updates/s (sites x steps x trajectories per second), and, as
the second half of the headline metric, time to steady state with and
without the learned warm start on a reduced 32 x 32 parameter sweep
(`time_to_steady_state`; skip with --no-warm).

  python bench.py [--gpus N --steps K --warmup W]          this engine
  python bench.py --impl reference [...]                   the CPU arm
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NX = NY = 64
NTRAJ = 16384
DT = 0.002
FRAME_STEPS = 250
T_END = 100.0
FLOPS_PER_SITE_UPDATE = 10 * 12 + 26  # 10 log2(N) + 26 for N = 4096
BYTES_PER_SITE_UPDATE_HBM = 16.0 / FRAME_STEPS  # state read + written once per launch (complex64)
METRIC = "site-updates/s"
CONFIG = {
    "workload": "2D 64x64 PBC, 16384 trajectories, J=1 U=0.2 gamma=1 omega=-0.5+N(0,0.04) F=2 dt=0.002, "
                "frame = 250 steps (+FP64 moments), complex64 state/FFT",
    "lattice": [NX, NY], "trajectories": NTRAJ, "dt": DT, "steps_per_bench_step": FRAME_STEPS,
    "l2": "state 512 MB > L2, re-read from HBM every launch",
}


def env_rank():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def clock_sampler_start(path):
    q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    try:
        f = open(path, "w")
        return subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits", "-lms", "200"],
                                stdout=f, stderr=subprocess.DEVNULL), f
    except Exception:
        return None, None


def clock_sampler_stop(proc, f, path, gpu_index):
    if proc is None:
        return None
    proc.terminate()
    try:
        proc.wait(timeout=5)
    except Exception:
        proc.kill()
    f.close()
    sm, smax, reasons = [], 0.0, set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    for line in open(path):
        parts = [p.strip() for p in line.split(",")]
        if len(parts) < 9 or not parts[0].isdigit() or int(parts[0]) != gpu_index:
            continue
        try:
            sm.append(float(parts[1]))
            smax = max(smax, float(parts[2]))
        except ValueError:
            continue
        for nm, v in zip(names, parts[5:9]):
            if v.lower().startswith("active"):
                reasons.add(nm)
    if not sm:
        return None
    return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


def _profile_figure(key, profile="square_fft_kernel_64x64.md"):
    """A figure `key: <number>` from a committed ncu summary of a step kernel
    (default: the FFT kernel on the headline workload), or None."""
    import re
    try:
        txt = open(os.path.join(ROOT, "profiles", profile)).read()
    except OSError:
        return None
    m = re.search(re.escape(key) + r":\s*([0-9.eE+]+)", txt)
    return float(m.group(1)) if m else None


def ncu_traffic():
    """DRAM bytes per step-kernel launch at the full workload (ncu, scaled from the small capture)."""
    return _profile_figure("dram_bytes_per_launch_full_size")


def measure_warm_start():
    """Time to steady state with and without the learned warm start on a
    reduced version of the 32 x 32 sweep (F ~ U[0,3], detuning ~ U[-2,2],
    U ~ U[0.05,0.5], J = gamma = 1, dt = 0.002): plain runs of 1024 points
    generate the training rows, the MLP is trained on the GPU, then 64
    held-out points run warm-started and plain (the plain run is the reference
    each warm-started point is checked against)."""
    from pincosimulator_gb300 import warmstart as wsm

    return wsm.evaluate(32, n_train=1024, traj_train=256, t_train=20.0, n_test=64, traj_test=512, t_test=20.0)


def make_system(twmc, hop=None, precision=None):
    return twmc.System(nx=NX, ny=NY, J=1.0, gamma=1.0, dt=DT, frame_steps=FRAME_STEPS,
                       omega=twmc.Noisy(-0.5, twmc.DISORDER_GAUSSIAN, 0.2), U=0.2, F=2.0, beta_init=0.0,
                       beta_init_sigma=0.5, precision=twmc.PREC_F32 if precision is None else precision,
                       hop=twmc.HOP_FFT if hop is None else hop, n_moment_blocks=32)


def measure_other_paths(twmc, torch, sm_mhz=None):
    """Throughput of the other configurations, one timed unit each: the
    headline workload on the real-space stencil kernel (the same hopping
    operator applied without the FFT), the 256-point heterogeneous batch
    (chains of 32..1024 sites and 16..128 square lattices, 512..4096
    trajectories per point, one frame of 250 steps in one graph launch), and
    the 1-D Lieb lattice (256 cells, U disorder, F(t) ramp, 8192 trajectories,
    1000 steps through twmc_run)."""
    import numpy as np
    out = {}
    sysd = make_system(twmc, hop=twmc.HOP_STENCIL)
    sysd.batch_init(sysd.make_tasks(NTRAJ, t_start=0.0, t_end=T_END, seed0=5, id0=1))
    sysd.advance(FRAME_STEPS)
    sysd.sync()
    ext = torch.cuda.ExternalStream(sysd.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(ext)
    for _ in range(2):
        sysd.advance(FRAME_STEPS)
    e1.record(ext)
    sysd.sync()
    ms = e0.elapsed_time(e1) / 2
    out["headline_real_space"] = {"value": FRAME_STEPS * NTRAJ * NX * NY / (ms / 1e3), "unit": METRIC,
                                  "kernel": sysd.kernel_name, "ms_per_frame": ms}
    kname = out["headline_real_space"]["kernel"]
    prof = "rowrun_kernel_64x64.md" if kname == "rowrun_kernel" else "ell_kernel_64x64_stencil.md"
    ipsu = _profile_figure("inst_per_site_update", prof)
    if ipsu and sm_mhz:
        sms = torch.cuda.get_device_properties(0).multi_processor_count
        ach = out["headline_real_space"]["value"] * ipsu / 32.0
        out["headline_real_space"]["issue"] = {
            "inst_per_site_update": ipsu, "frac": ach / (sms * 4 * sm_mhz * 1e6),
            "source": f"ncu instruction count (profiles/{prof}) x measured rate; "
                      "peak = SMs x 4 schedulers x median SM clock of the headline run"}
    sysd.close()
    rng = np.random.default_rng(3)
    kinds = [(1, n) for n in (32, 64, 128, 256, 512, 1024)] + [(l, l) for l in (16, 32, 64, 128)]
    pts = []
    for _ in range(256):
        nx, ny = kinds[rng.integers(len(kinds))]
        pts.append(dict(nx=nx, ny=ny, U=rng.uniform(0.05, 0.5), omega=rng.uniform(-2, 2), F=rng.uniform(0, 3),
                        dt=DT, n_traj=int(np.exp(rng.uniform(np.log(512), np.log(4096)))),
                        seed0=int(rng.integers(1, 2 ** 31)), id0=1))
    sites = sum(p["nx"] * p["ny"] * p["n_traj"] for p in pts)
    hb = twmc.HBatch(pts, FRAME_STEPS, tune=True)
    hb.run(1)
    hb.sync()
    hb.run(1)
    ms = hb.sync()
    out["heterogeneous_batch"] = {"value": FRAME_STEPS * sites / (ms / 1e3), "unit": METRIC, "points": len(pts),
                                  "ms_per_frame": ms, "autotuned": True}
    hb.close()
    from pincosimulator_gb300 import workloads
    sysd = workloads.lieb()
    el, _ = workloads.time_run(sysd, 8192, 4)
    out["lieb"] = {"value": sysd.n_sites * 8192 * 1000 / el, "unit": METRIC, "kernel": sysd.kernel_name,
                   "timing": "host wall clock around one twmc_run call of 1000 steps (initial draws and frame "
                             "bookkeeping included)"}
    sysd.close()
    return out


def measure_f64(twmc, torch, steps=2):
    """The same workload in the engine's FP64 mode (FP64 state, FFT and noise:
    the plain FP64 GPU split-step), device-timed like the headline."""
    sysd = make_system(twmc, precision=twmc.PREC_F64)
    sysd.batch_init(sysd.make_tasks(NTRAJ, t_start=0.0, t_end=T_END, seed0=3, id0=1))
    sysd.advance(FRAME_STEPS)
    sysd.sync()
    ext = torch.cuda.ExternalStream(sysd.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(ext)
    for _ in range(steps):
        sysd.advance(FRAME_STEPS)
        sysd.reduce()
    e1.record(ext)
    sysd.sync()
    ms = e0.elapsed_time(e1)
    kname = sysd.kernel_name
    sysd.close()
    return {"value": steps * FRAME_STEPS * NTRAJ * NX * NY / (ms / 1e3), "unit": METRIC, "steps": steps,
            "kernel": kname}


def measure_observable_error(twmc, ntraj=256, t_end=T_END):
    """Error of the FP32 engine's observables against the FP64 engine (the
    plain FP64 GPU split-step) on the headline workload over its full
    horizon: the same trajectories (seeds, ids, Philox streams) in both
    precisions, n, g2 and n_k per frame and site compared in units of the
    combined standard error (32 trajectory blocks)."""
    import numpy as np
    from pincosimulator_gb300 import observables as ob

    nframes = int(round(t_end / (DT * FRAME_STEPS)))
    per = {}
    for name, prec in (("f32", twmc.PREC_F32), ("f64", twmc.PREC_F64)):
        sysd = make_system(twmc, precision=prec)
        sysd.batch_init(sysd.make_tasks(ntraj, t_start=0.0, t_end=t_end, seed0=424242, id0=1))
        frames = []
        t0 = time.perf_counter()
        for _ in range(nframes):
            sysd.advance(FRAME_STEPS)
            sysd.reduce()
            _, m = sysd.download(field=False, moments=True)
            o = ob.observables(m, ntraj)
            frames.append({k: o[k] for k in ("n", "n_se", "g2", "g2_se", "nk", "nk_se", "bm2")})
        per[name] = ({k: np.stack([f[k] for f in frames]) for k in frames[0]}, time.perf_counter() - t0)
        sysd.close()
    c = ob.compare(per["f32"][0], per["f64"][0], frames=slice(0, None))
    return {"workload": f"headline workload, {ntraj} trajectories, t_end = {t_end:g} ({nframes} frames of "
                        f"{FRAME_STEPS} steps), same seeds and Philox streams in both precisions",
            "fp32_vs_fp64": c, "f32_s": round(per["f32"][1], 2), "f64_s": round(per["f64"][1], 2),
            "units": "max |z| and mean z^2 over frames x sites, z = (FP32 - FP64) / sqrt(SE32^2 + SE64^2); "
                     "n_site_avg.max_rel_diff = max over frames of |nbar32 - nbar64| / nbar64"}


def cpu_baseline(target_s=12.0, threads=None):
    """Oracle port (FP64 restatement, radix-2 FFT, not FFTW) on the host cores:
    a bounded sample of the same workload (trajectories x 250 steps of 64 x 64)."""
    import numpy as np
    from oracle import loader as orc

    lib = orc.load(fast=True)
    threads = threads or os.cpu_count() or 1
    n = NX * NY
    rng = np.random.default_rng(0)
    omega = np.ascontiguousarray(-0.5 + 0.2 * rng.normal(size=n) + 0j)
    U = np.full(n, 0.2 + 0j)
    F = np.full(n, 2.0 + 0j)
    b0 = np.ascontiguousarray(0.5 * (rng.normal(size=n) + 1j * rng.normal(size=n)))

    def run(ntraj, steps):
        t0 = time.perf_counter()
        done = lib.orc_base_run_batch(NX, NY, 1.0, 1.0, DT, 0.0, (steps - 0.5) * DT, steps, 2, omega.ctypes.data,
                                      U.ctypes.data, F.ctypes.data, b0.ctypes.data, ntraj, 1, threads, None)
        return done, time.perf_counter() - t0

    steps = 25
    _, t1 = run(threads, steps)  # calibration: one trajectory per thread
    per_round = max(t1, 1e-3)
    rounds = max(1, int(target_s / per_round))
    ntraj = threads * rounds
    done, el = run(ntraj, steps)
    su = float(done) * steps * n
    return {"value": su / el, "unit": METRIC, "cores": threads, "kind": "port",
            "sample": f"{done} trajectories x {steps} steps of 64x64 (FP64 oracle restatement, radix-2 FFT, not "
                      f"FFTW), {el:.1f} s"}


def run_reference(args):
    rank, world, _ = env_rank()
    if rank != 0:
        return 0
    steps = args.steps
    vals = []
    for i in range(args.warmup + steps):
        cb = cpu_baseline(target_s=max(2.0, 60.0 / max(1, args.warmup + steps)))
        if i >= args.warmup:
            vals.append(cb)
    v = statistics.median(c["value"] for c in vals)
    ms = 1e3 * (NTRAJ * NX * NY * FRAME_STEPS) / v
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": METRIC, "n_gpus": args.gpus,
            "steps": steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": CONFIG,
            "cpu_baseline": {"value": v, "unit": METRIC, "cores": vals[0]["cores"], "kind": "port",
                             "sample": vals[0]["sample"]},
            "e2e": {"value": v, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "the reference cannot be built here (FFTW3/Eigen3/cpptoml/CLI11/easylogging++ absent); the "
                    "arm runs the oracle's FP64 restatement of TWMCBaseSolver's loop on all host threads; "
                    "ms_per_step extrapolates the per-site rate to one full bench step"}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--hop", default="fft", choices=["fft", "stencil"])
    ap.add_argument("--e2e-steps", type=int, default=4)
    ap.add_argument("--clocks-csv", default=None,
                    help="where nvidia-smi writes its clock samples (default: the temp directory)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-warm", action="store_true", help="skip the learned warm-start time-to-steady-state leg")
    ap.add_argument("--no-f64", action="store_true", help="skip timing the FP64 mode")
    ap.add_argument("--no-other", action="store_true", help="skip the other configurations")
    ap.add_argument("--no-obs-err", action="store_true", help="skip the FP32-vs-FP64 observable-error leg")
    ap.add_argument("--ntraj", type=int, default=NTRAJ, help="profiling cases only; the bench line uses 16384")
    args = ap.parse_args()
    rank, world, local = env_rank()
    if args.impl == "reference":
        return run_reference(args)
    if world > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    import torch

    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(0)
    from pincosimulator_gb300 import build_ext, twmc

    build_ext.build()
    fp32_peak = twmc.measure_fp32_peak()
    sysd = make_system(twmc, twmc.HOP_STENCIL if args.hop == "stencil" else None)
    ntraj = args.ntraj
    tasks = sysd.make_tasks(ntraj, t_start=0.0, t_end=T_END, seed0=1000 + rank * ntraj, id0=1 + rank * ntraj)
    sysd.batch_init(tasks)
    for _ in range(max(args.warmup, 3)):
        sysd.advance(FRAME_STEPS)
        sysd.reduce()
    sysd.sync()
    ext = torch.cuda.ExternalStream(sysd.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clk_path = args.clocks_csv or os.path.join(tempfile.gettempdir(), f"twmc_clocks_rank{rank}.csv")
    if world > 1 and args.clocks_csv:
        clk_path = f"{os.path.splitext(args.clocks_csv)[0]}_rank{rank}.csv"
    if os.path.dirname(clk_path):
        os.makedirs(os.path.dirname(clk_path), exist_ok=True)
    proc, fh = clock_sampler_start(clk_path)
    time.sleep(0.5)
    launches0 = sysd.launch_count
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e0.record(ext)
    for _ in range(args.steps):
        sysd.advance(FRAME_STEPS)
        sysd.reduce()
    e1.record(ext)
    kernel_ms = sysd.sync()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    elapsed_ms = e0.elapsed_time(e1)
    launches = sysd.launch_count - launches0
    clocks = clock_sampler_stop(proc, fh, clk_path, int(os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0])
                                if world > 1 else 0)
    field, _ = sysd.download(field=True, moments=False)
    import numpy as np

    finite = bool(np.isfinite(field).all())
    del field
    info_kernel = sysd.kernel_name
    sysd.close()
    su_rank = float(args.steps) * FRAME_STEPS * ntraj * NX * NY
    t_max = elapsed_ms
    if dist:
        t = torch.tensor([elapsed_ms], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_max = float(t.item())
    value = su_rank * world / (t_max / 1e3)
    # roofline of the dominant kernel (the step kernel; the moments kernel is < 1%)
    achieved = su_rank * FLOPS_PER_SITE_UPDATE / (kernel_ms / 1e3) / 1e12
    # end to end through the C ABI with host buffers (twmc_run)
    e2e = None
    if not args.no_e2e:
        sysd = make_system(twmc, twmc.HOP_STENCIL if args.hop == "stencil" else None)
        tasks = sysd.make_tasks(NTRAJ, t_start=0.0, t_end=args.e2e_steps * FRAME_STEPS * DT, seed0=7,
                                store_initial=False)
        # result buffers in pinned host memory, allocated once and reused by
        # every call as a production caller would; one untimed warm-up call
        bufs = {"final": torch.empty((NTRAJ, NX * NY), dtype=torch.complex128, pin_memory=True).numpy(),
                "moments": torch.empty((args.e2e_steps, 32, NX * NY, 3), dtype=torch.float64,
                                       pin_memory=True).numpy()}
        sysd.run(tasks, frames=False, final=True, moments=True, buffers=bufs)
        reps = 2
        calls = []
        for _ in range(reps):
            t0 = time.perf_counter()
            res = sysd.run(tasks, frames=False, final=True, moments=True, buffers=bufs)
            calls.append(time.perf_counter() - t0)
        el = sum(calls) / reps
        sysd.close()
        n_fr = args.e2e_steps
        h2d = (NTRAJ * (8 + 8) + 5 * 2 * NX * NY * 16) / n_fr
        d2h = (res["final"].size * 8 + n_fr * 32 * NX * NY * 3 * 8 + NTRAJ * (8 + 8 + 4)) / n_fr
        e2e = {"value": n_fr * FRAME_STEPS * NTRAJ * NX * NY / el, "unit": METRIC, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "calls_ms": [round(c * 1e3, 2) for c in calls], "api": "twmc_run (pinned host result buffers reused across calls: "
               "final field widened to complex128 on the GPU, FP64 moment blocks every frame; initial draws and "
               "disorder on the GPU inside the call; mean of 2 calls after 1 warm-up)"}
        del res
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return 0
    peaks = measured_peaks()
    # instruction-issue roofline: ncu's instructions per site-update x the
    # measured rate, against one warp instruction per cycle per scheduler
    ipsu = _profile_figure("inst_per_site_update")
    issue = None
    if ipsu and clocks and clocks.get("sm_mhz"):
        sms = torch.cuda.get_device_properties(0).multi_processor_count
        ach = su_rank / (kernel_ms / 1e3) * ipsu / 32.0
        pk = sms * 4 * clocks["sm_mhz"] * 1e6
        issue = {"inst_per_site_update": ipsu, "achieved_warp_inst_per_s": ach, "peak_warp_inst_per_s": pk,
                 "frac": ach / pk, "source": "ncu instruction count (profiles/square_fft_kernel_64x64.md) x "
                 "measured rate; peak = SMs x 4 schedulers x median SM clock"}
    cpu = None if (args.no_cpu_baseline or world > 1) else cpu_baseline()
    warm = None if (args.no_warm or world > 1) else measure_warm_start()
    f64 = None
    if world == 1 and args.ntraj == NTRAJ and not args.no_f64:
        f64 = measure_f64(twmc, torch)
        f64["fp32_speedup"] = value / f64["value"]
    obs_err = None
    if world == 1 and args.ntraj == NTRAJ and not args.no_obs_err:
        obs_err = measure_observable_error(twmc)
    other = None
    if world == 1 and args.ntraj == NTRAJ and not args.no_other:
        other = measure_other_paths(twmc, torch, clocks.get("sm_mhz") if clocks else None)
    hbm = peaks.get("hbm_gbs")
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded Philox disorder / noise)",
        "config": dict(CONFIG, hop=args.hop, kernel=info_kernel, trajectories=ntraj),
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": achieved / fp32_peak if fp32_peak else None, "traffic": ncu_traffic(),
                     "peak_source": "measured in this run: FP32 FMA chain over all SMs (twmc_measure_fp32_peak)",
                     "flops_per_site_update": FLOPS_PER_SITE_UPDATE,
                     "hbm": {"achieved_gbs": su_rank * BYTES_PER_SITE_UPDATE_HBM / (kernel_ms / 1e3) / 1e9,
                             "peak_gbs": hbm, "source": "MEASURED_PEAKS.json" if hbm else None}},
        "issue": issue, "e2e": e2e, "gpu_launches": launches, "cpu_baseline": cpu, "clocks": clocks,
        "trajectories_per_s": value / (NX * NY * (T_END / DT)), "finite": finite,
        "kernel_ms": kernel_ms, "time_to_steady_state": warm, "fp64_mode": f64, "observable_error": obs_err,
        "other_paths": other,
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
