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


def _profile_source(profile):
    """Where a profile figure came from: the summary file and its `captured:`
    line (date and commit of the capture), so that stale figures show."""
    import re
    try:
        txt = open(os.path.join(ROOT, "profiles", profile)).read()
    except OSError:
        return None
    m = re.search(r"captured:\s*(.+)", txt)
    return {"file": f"profiles/{profile}", "captured": m.group(1).strip() if m else "unrecorded"}


def issue_fraction(rate, profile, sm_mhz, torch):
    """Warp-instruction issue rate of a kernel: site-updates/s x ncu's thread
    instructions per site-update / 32, against one instruction per cycle per
    scheduler (SMs x 4 x the median SM clock of the run)."""
    ipsu = _profile_figure("inst_per_site_update", profile)
    if not ipsu or not sm_mhz:
        return None
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    ach = rate * ipsu / 32.0
    return {"inst_per_site_update": ipsu, "frac": ach / (sms * 4 * sm_mhz * 1e6),
            "profile": _profile_source(profile)}


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


def make_system(twmc, hop=None, precision=None, integrator=0):
    return twmc.System(nx=NX, ny=NY, J=1.0, gamma=1.0, dt=DT, frame_steps=FRAME_STEPS,
                       omega=twmc.Noisy(-0.5, twmc.DISORDER_GAUSSIAN, 0.2), U=0.2, F=2.0, beta_init=0.0,
                       beta_init_sigma=0.5, precision=twmc.PREC_F32 if precision is None else precision,
                       hop=twmc.HOP_FFT if hop is None else hop, n_moment_blocks=32, integrator=integrator)


def measure_batch(twmc, torch, sm_mhz=None, t_end=60.0):
    """The 256-point heterogeneous batch to its full t_end (120 frames of 250
    steps), autotuned step variants, every (point, trajectory group) a work
    item of the persistent queue kernels; device time of the whole run."""
    from collections import Counter
    from pincosimulator_gb300.workloads import batch_points
    pts = batch_points()
    sites = sum(p["nx"] * p["ny"] * p["n_traj"] for p in pts)
    frames = int(round(t_end / (DT * FRAME_STEPS)))
    hb = twmc.HBatch(pts, FRAME_STEPS, tune=True)
    plans = [hb.plan(i) for i in range(len(pts))]
    hb.run(1)  # untimed first frame
    hb.sync()
    hb.run(frames)
    ms = hb.sync()
    bm = hb.block_means()
    import numpy as np
    finite = bool(all(np.isfinite(b).all() for b in bm))
    hb.close()
    rate = frames * FRAME_STEPS * sites / (ms / 1e3)
    out = {"value": rate, "unit": METRIC, "points": len(pts), "t_end": t_end, "frames": frames,
           "device_s": ms / 1e3, "trajectories_per_s": sum(p["n_traj"] for p in pts) / (ms / 1e3),
           "finite": finite, "autotuned": True,
           "kernels": dict(Counter(p.split("<")[0] for p in plans)),
           "variants": dict(sorted(Counter(p.split("<")[1].rstrip(">") for p in plans).items())),
           "timing": "CUDA events around the graph replays of frames 2..121 (t = 0.5..60.5, the 30000 steps of "
                     "a run to t_end = 60); trajectories_per_s = all points' trajectories / that time"}
    iss = issue_fraction(rate, "hbatch_256_points.md", sm_mhz, torch)
    if iss:
        out["issue"] = iss
    return out


def measure_other_paths(twmc, torch, sm_mhz=None):
    """Throughput of the other configurations, device-timed: the headline
    workload on the real-space stencil kernel (the same hopping operator
    applied without the FFT), the 256-point heterogeneous batch to t = 60,
    the 1-D Lieb lattice (256 cells, U disorder, F(t) ramp, 8192
    trajectories) and the 128 x 128 lattice on the 2-CTA cluster kernel
    (4096 trajectories), each with its issue-rate fraction; the Lieb workload
    also through twmc_run (host wall clock, initial draws included)."""
    from pincosimulator_gb300 import workloads
    out = {}
    sysd = make_system(twmc, hop=twmc.HOP_STENCIL)
    s = workloads.time_batch(sysd, NTRAJ, 2)
    r = FRAME_STEPS * NTRAJ * NX * NY * 2 / s
    out["headline_real_space"] = {"value": r, "unit": METRIC, "kernel": sysd.kernel_name, "ms_per_frame": s * 500}
    prof = "rowrun_kernel_64x64.md" if sysd.kernel_name == "rowrun_kernel" else "ell_kernel_64x64_stencil.md"
    out["headline_real_space"]["issue"] = issue_fraction(r, prof, sm_mhz, torch)
    sysd.close()
    out["heterogeneous_batch"] = measure_batch(twmc, torch, sm_mhz)
    sysd = workloads.lieb()
    tasks = sysd.make_tasks(8192, t_end=4 * FRAME_STEPS * DT, store_initial=False)
    sysd.run(tasks, frames=False, final=False)  # untimed; the F(t) table runs through twmc_run
    sysd.sync()
    t0 = time.perf_counter()
    sysd.run(tasks, frames=False, final=False)
    el = time.perf_counter() - t0
    kms = sysd.sync()  # CUDA-event time of the step launches of the timed call
    r = sysd.n_sites * 8192 * 1000 / (kms / 1e3)
    out["lieb"] = {"value": r, "unit": METRIC, "kernel": sysd.kernel_name, "kernel_ms_per_1000_steps": kms,
                   "workload": "1-D Lieb 256 cells x 3, PBC, U = 0.27 + 0.06 U[0,1), F(t) ramp on B sites, "
                               "8192 trajectories, 1000 steps (CUDA events around the step launches)",
                   "issue": issue_fraction(r, "lieb_cell_kernel_lieb768.md", sm_mhz, torch),
                   "twmc_run": {"value": sysd.n_sites * 8192 * 1000 / el, "unit": METRIC,
                                "timing": "host wall clock around the twmc_run call (initial draws and frame "
                                          "bookkeeping included)"}}
    sysd.close()
    sysd = workloads.square(128, 128, hop=twmc.HOP_STENCIL)
    s = workloads.time_batch(sysd, 4096, 1)
    r = 128 * 128 * 4096 * FRAME_STEPS / s
    out["square128"] = {"value": r, "unit": METRIC, "kernel": sysd.kernel_name, "ms_per_frame": s * 1e3,
                        "workload": "128x128 PBC, the headline parameters, 4096 trajectories, one 250-step frame",
                        "issue": issue_fraction(r, "ell_cluster_pow2_kernel_128x128.md", sm_mhz, torch)}
    sysd.close()
    return out


def measure_f64(twmc, torch, steps=2, precision=None, integrator=0):
    """The same workload in the engine's FP64 mode (FP64 state, FFT and noise:
    the plain FP64 GPU step; integrator 1 = the exponential split step),
    device-timed like the headline."""
    sysd = make_system(twmc, precision=twmc.PREC_F64 if precision is None else precision, integrator=integrator)
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


def _cpu_cores():
    """Host CPU description for the baseline record: the model name, or on
    Arm hosts (whose /proc/cpuinfo has none) the implementer and part ids."""
    fields = {}
    try:
        for line in open("/proc/cpuinfo"):
            if ":" in line:
                k, v = line.split(":", 1)
                fields.setdefault(k.strip().lower(), v.strip())
    except OSError:
        pass
    model = fields.get("model name") or fields.get("cpu model") or ""
    if not model and "cpu part" in fields:
        model = f"{platform_machine()} (CPU implementer {fields.get('cpu implementer', '?')}, part {fields['cpu part']})"
    return os.cpu_count() or 1, model


def platform_machine():
    import platform
    return platform.machine()


def cpu_run(ntraj, steps, threads, build, noise):
    """Wall time of ntraj trajectories x `steps` steps of the 64 x 64
    workload through the oracle's threaded batch (one trajectory per task on
    `threads` workers, as the reference's ThreadedTaskProcessor)."""
    import numpy as np
    from oracle import loader as orc

    lib = orc.load(fast=build)
    n = NX * NY
    rng = np.random.default_rng(0)
    omega = np.ascontiguousarray(-0.5 + 0.2 * rng.normal(size=n) + 0j)
    U = np.full(n, 0.2 + 0j)
    F = np.full(n, 2.0 + 0j)
    b0 = np.ascontiguousarray(0.5 * (rng.normal(size=n) + 1j * rng.normal(size=n)))
    t0 = time.perf_counter()
    done = lib.orc_base_run_batch(NX, NY, 1.0, 1.0, DT, 0.0, (steps - 0.5) * DT, steps, 2, omega.ctypes.data,
                                  U.ctypes.data, F.ctypes.data, b0.ctypes.data, ntraj, 1, threads, None,
                                  orc.NOISE[noise])
    return done, time.perf_counter() - t0


def cpu_baseline(target_s=12.0, threads=None):
    """The CPU restatement of the reference's loop (FP64, the oracle's FFT,
    not FFTW) on all host threads, timed on a bounded sample of the same
    workload (trajectories x 25 steps of 64 x 64): the headline figure uses
    the reference's own release flags (-Ofast -march=native) and noise
    generator (std::mt19937 + std::normal_distribution, as randCMat); the
    -O3 build with the GPU solver's Philox stream is reported beside it."""
    from oracle import build_oracle

    cores, model = _cpu_cores()
    threads = threads or cores
    steps = 25
    out = {}
    for key, build, noise, share in (("ref_flags_mt19937", "ref_flags", "mt19937", 0.7),
                                     ("O3_philox", True, "philox64", 0.3)):
        _, t1 = cpu_run(threads, steps, threads, build, noise)  # calibration: one trajectory per thread
        rounds = max(1, int(share * target_s / max(t1, 1e-3)))
        done, el = cpu_run(threads * rounds, steps, threads, build, noise)
        out[key] = {"value": float(done) * steps * NX * NY / el, "seconds": round(el, 2),
                    "sample": f"{done} trajectories x {steps} steps", "flags": build_oracle.build_flags(build),
                    "noise": noise}
    head = out["ref_flags_mt19937"]
    return {"value": head["value"], "unit": METRIC, "cores": threads, "kind": "port", "cpu": model,
            "sample": f"{head['sample']} of 64x64 in {head['seconds']} s; FP64 restatement of "
                      f"TWMCBaseSolver's loop with the reference's flags ({head['flags']}) and noise generator "
                      "(mt19937 + normal_distribution); batched radix-2 FFT, not FFTW",
            "variants": out}


def run_reference(args):
    """The reference arm: the CPU restatement of the reference's loop with the
    reference's flags and noise generator on all host threads, each step a
    bounded sample of the headline workload (trajectories x 25 steps of
    64 x 64) timed on its own; value = the median sample rate."""
    rank, world, _ = env_rank()
    if rank != 0:
        return 0
    from oracle import build_oracle

    build_oracle.build()
    cores, model = _cpu_cores()
    steps = 25
    _, t1 = cpu_run(cores, steps, cores, "ref_flags", "mt19937")
    per_step_s = max(2.0, 45.0 / max(1, args.warmup + args.steps))
    rounds = max(1, int(per_step_s / max(t1, 1e-3)))
    samples = []
    for i in range(args.warmup + args.steps):
        done, el = cpu_run(cores * rounds, steps, cores, "ref_flags", "mt19937")
        if i >= args.warmup:
            samples.append((done, el))
    rates = [d * steps * NX * NY / e for d, e in samples]
    v = statistics.median(rates)
    sample = f"{samples[0][0]} trajectories x {steps} steps of 64x64 per step"
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": METRIC, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * statistics.median(e for _, e in samples), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": CONFIG,
            "sample_site_updates_per_step": samples[0][0] * steps * NX * NY,
            "cpu_baseline": {"value": v, "unit": METRIC, "cores": cores, "kind": "port", "cpu": model,
                             "sample": sample, "flags": build_oracle.build_flags("ref_flags"),
                             "noise": "mt19937 + normal_distribution (randCMat)"},
            "e2e": {"value": v, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "the reference cannot be built here (FFTW3/Eigen3/cpptoml/CLI11/easylogging++ absent); the "
                    "arm runs the oracle's FP64 restatement of TWMCBaseSolver's loop with the reference's release "
                    "flags and noise generator, one trajectory per task on all host threads; each bench step is "
                    "one timed sample (ms_per_step is that sample's wall time, not the full 16384-trajectory "
                    "frame)"}
    print(json.dumps(line), flush=True)
    return 0


def measure_e2e(twmc, torch, args, frames=True):
    """Site-updates/s through twmc_run with host result buffers: one call
    runs e2e_steps frames of all 16384 trajectories (initial draws and
    disorder on the GPU inside the call) and returns, into pinned host arrays
    allocated once and reused as a production caller would, every saved frame
    (complex128, the reference's traj dataset) when `frames`, the final field
    and the FP64 moment blocks of every frame. Mean of two calls after one
    warm-up call."""
    sysd = make_system(twmc, twmc.HOP_STENCIL if args.hop == "stencil" else None)
    n_fr = args.e2e_steps
    tasks = sysd.make_tasks(NTRAJ, t_start=0.0, t_end=n_fr * FRAME_STEPS * DT, seed0=7, store_initial=False)
    bufs = {"final": torch.empty((NTRAJ, NX * NY), dtype=torch.complex128, pin_memory=True).numpy(),
            "moments": torch.empty((n_fr, 32, NX * NY, 3), dtype=torch.float64, pin_memory=True).numpy()}
    if frames:
        bufs["frames"] = torch.empty((NTRAJ, n_fr, NX * NY), dtype=torch.complex128, pin_memory=True).numpy()
    sysd.run(tasks, frames=frames, final=True, moments=True, buffers=bufs)
    calls = []
    for _ in range(2):
        t0 = time.perf_counter()
        res = sysd.run(tasks, frames=frames, final=True, moments=True, buffers=bufs)
        calls.append(time.perf_counter() - t0)
    el = sum(calls) / len(calls)
    sysd.close()
    h2d = (NTRAJ * (8 + 8) + 5 * 2 * NX * NY * 16) / n_fr  # seeds, ids, base / amplitude matrices
    d2h = (sum(b.nbytes for b in bufs.values()) + NTRAJ * (8 + 8 + 4)) / n_fr
    assert res["frames_written"].min() == n_fr
    out = {"value": n_fr * FRAME_STEPS * NTRAJ * NX * NY / el, "unit": METRIC, "h2d_bytes_per_step": int(h2d),
           "d2h_bytes_per_step": int(d2h), "calls_ms": [round(c * 1e3, 2) for c in calls],
           "api": "twmc_run into pinned host result arrays reused across calls: " +
                  ("every frame of every trajectory (complex128, widened on the GPU), " if frames else "") +
                  "the final field, FP64 moment blocks of every frame; initial draws and disorder on the GPU "
                  "inside the call; mean of 2 calls after 1 warm-up"}
    del res, bufs
    return out


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
    field, mom = sysd.download(field=True, moments=True)
    import numpy as np

    finite = bool(np.isfinite(field).all())
    del field
    # replicas: every rank's FP64 moment blocks of its own trajectories,
    # gathered in rank order on the host (gloo) -- the only exchange of the
    # path; the merged blocks are those of one run of all ranks' trajectories
    from pincosimulator_gb300 import observables as obmod, replicas

    if dist:
        gloo = dist.new_group(backend="gloo")
        merged = replicas.gather_blocks(mom, group=gloo)
    else:
        merged = mom
    ens = obmod.observables(merged, ntraj * world)
    ensemble = {"ranks": world, "trajectories": ntraj * world, "blocks": int(merged.shape[0]),
                "n_site_avg": float(np.mean(ens["n"])), "g2_site_avg": float(np.nanmean(ens["g2"])),
                "merge": "moment blocks gathered in rank order (replicas.gather_blocks over gloo)" if dist else
                         "single rank"}
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
    # end to end through the C ABI with host buffers (twmc_run): every saved
    # frame of every trajectory (the reference's "traj" dataset,
    # TWMCBaseSolver.cpp:257-277) plus the moment blocks; the same call
    # without frames beside it
    e2e = None
    if not args.no_e2e:
        e2e = measure_e2e(twmc, torch, args, frames=True)
        e2e["no_frames"] = measure_e2e(twmc, torch, args, frames=False)
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return 0
    peaks = measured_peaks()
    # instruction-issue roofline: ncu's instructions per site-update x the
    # measured rate, against one warp instruction per cycle per scheduler
    issue = issue_fraction(su_rank / (kernel_ms / 1e3), "square_fft_kernel_64x64.md",
                           clocks.get("sm_mhz") if clocks else None, torch)
    cpu = None if (args.no_cpu_baseline or world > 1) else cpu_baseline()
    warm = None if (args.no_warm or world > 1) else measure_warm_start()
    f64 = None
    if world == 1 and args.ntraj == NTRAJ and not args.no_f64:
        f64 = measure_f64(twmc, torch)
        f64["fp32_speedup"] = value / f64["value"]
        # the exponential split step (TWMC_INTEGRATOR_SPLIT) in FP64, the
        # target's plain FP64 GPU split-step, and the same step in FP32
        sp = measure_f64(twmc, torch, integrator=twmc.INTEGRATOR_SPLIT)
        sp["fp32_speedup"] = value / sp["value"]
        sp32 = measure_f64(twmc, torch, precision=twmc.PREC_F32, integrator=twmc.INTEGRATOR_SPLIT)
        sp["fp32_split_step"] = {"value": sp32["value"], "kernel": sp32["kernel"],
                                 "vs_fp64_split": sp32["value"] / sp["value"]}
        f64["split_step"] = sp
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
                     "traffic_profile": _profile_source("square_fft_kernel_64x64.md"),
                     "peak_source": "measured in this run: FP32 FMA chain over all SMs (twmc_measure_fp32_peak)",
                     "flops_per_site_update": FLOPS_PER_SITE_UPDATE,
                     "hbm": {"achieved_gbs": su_rank * BYTES_PER_SITE_UPDATE_HBM / (kernel_ms / 1e3) / 1e9,
                             "peak_gbs": hbm, "source": "MEASURED_PEAKS.json" if hbm else None}},
        "issue": issue, "e2e": e2e, "gpu_launches": launches, "cpu_baseline": cpu, "clocks": clocks,
        "trajectories_per_s": value / (NX * NY * (T_END / DT)), "finite": finite,
        "kernel_ms": kernel_ms, "time_to_steady_state": warm, "fp64_mode": f64, "observable_error": obs_err,
        "other_paths": other, "ensemble": ensemble,
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
