"""Learned warm start for parameter sweeps of the driven-dissipative lattice.

A sweep over parameter points (F, detuning, U at fixed J, gamma) spends the
first part of every plain run relaxing from the vacuum. Here an MLP, trained
on steady states the engine itself produced (plain runs), predicts for a new
point the steady-state k-mode mean field <a_k> and density n; each
trajectory then starts from beta_init = that mean field in real space plus
Gaussian fluctuations of per-quadrature variance (max(n - |beta_init|^2, 0)
+ 1/2) / 2 (the reference's ReadFromSettings initial condition with a
per-site beta_init and beta_init_sigma). The plain vacuum-initialised run
stays the reference: a point whose warm-started steady density or g2 differs
from the plain run's by more than `rerun_se` standard errors is replaced by
its plain result (the rerun rule).

Device work -- plain runs, field moments, MLP rows, training, inference,
initial fields, warm runs -- goes through the C ABI (twmc_hbatch_*,
twmc_mlp_*). torch provides device buffers and shuffles minibatch indices.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Optional, Sequence

import numpy as np

from . import twmc
from .observables import observables, time_to_steady_state

FEATURES = ("F", "omega", "U", "J", "gamma")
# normalisation ranges of the sweep (F in [0, 3], detuning in [-2, 2], U in [0.05, 0.5], J = gamma = 1)
RANGES = {"F": (0.0, 3.0), "omega": (-2.0, 2.0), "U": (0.05, 0.5), "J": (1.0, 1.0), "gamma": (1.0, 1.0)}


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("the learned warm start needs a CUDA device")
    return torch


def features(points: Sequence[dict]) -> np.ndarray:
    """[P][5] float32 network inputs, each parameter mapped to [-1, 1] over RANGES."""
    x = np.zeros((len(points), len(FEATURES)), dtype=np.float32)
    for i, p in enumerate(points):
        for j, k in enumerate(FEATURES):
            lo, hi = RANGES[k]
            v = float(np.real(p.get(k, 1.0 if k in ("J", "gamma") else 0.0)))
            mid, half = 0.5 * (lo + hi), 0.5 * (hi - lo)
            x[i, j] = (v - mid) / half if half > 0 else v - mid
    return x


def sample_points(n: int, seed: int) -> list:
    """Uniform draws over the sweep box: F ~ U[0,3], detuning ~ U[-2,2], U ~ U[0.05,0.5], J = gamma = 1."""
    rng = np.random.default_rng(seed)
    return [{"F": float(rng.uniform(0, 3)), "omega": float(rng.uniform(-2, 2)), "U": float(rng.uniform(0.05, 0.5)),
             "J": 1.0, "gamma": 1.0} for _ in range(n)]


def _point_descs(points, nx, ny, n_traj, dt, seed0):
    out = []
    for i, p in enumerate(points):
        out.append({"nx": nx, "ny": ny, "J": p.get("J", 1.0), "gamma": p.get("gamma", 1.0), "dt": dt,
                    "omega": p["omega"], "U": p["U"], "F": p["F"], "beta_init": 0.0, "beta_init_sigma": 0.5,
                    "n_traj": n_traj, "seed0": seed0 + 7919 * i, "id0": 1 + n_traj * i, "n_moment_blocks": 32})
    return out


def steady_rows(points, nx, ny, n_traj, t_end, dt=0.002, frame_period=0.5, tail_frames=8, seed0=1, tune=False):
    """Plain (vacuum-initialised) runs of every point to t_end; MLP rows
    [P][2N+1] (device float32) from the mean field and <|a|^2> averaged over
    the last tail_frames frames."""
    torch = _torch()
    frame_steps = max(1, int(math.ceil(frame_period / dt - 1e-9)))
    n_frames = max(tail_frames, int(round(t_end / (frame_steps * dt))))
    hb = twmc.HBatch(_point_descs(points, nx, ny, n_traj, dt, seed0), frame_steps, tune=tune)
    try:
        N = nx * ny
        P = len(points)
        mean = torch.zeros(P * N * 2, dtype=torch.float64, device="cuda")
        abs2 = torch.zeros(P * N, dtype=torch.float64, device="cuda")
        rows = torch.zeros(P, 2 * N + 1, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()  # the batch's stream does not order with torch's
        hb.run(n_frames - tail_frames)
        for f in range(tail_frames):
            hb.run(1)
            hb.field_moments(mean.data_ptr(), abs2.data_ptr(), accumulate=f > 0)
        twmc.mlp_targets(mean.data_ptr(), abs2.data_ptr(), P, nx, ny, tail_frames, rows.data_ptr(), 2 * N + 1,
                         hb.stream)
        hb.sync()
        return rows, n_traj * N * frame_steps * n_frames * P
    finally:
        hb.close()


@dataclass
class FitReport:
    losses: list = field(default_factory=list)
    steps: int = 0
    launches: int = 0


class WarmStart:
    """MLP 5 -> hidden... -> 2N+1 for an nx x ny lattice."""

    def __init__(self, nx: int, ny: int, hidden=(256, 256, 256), max_batch: int = 256, seed: int = 1,
                 squash: float = 1.0, max_incoherent: float = 0.25):
        self.nx, self.ny = nx, ny
        self.squash = squash                  # rows are fitted as asinh(v / squash)
        self.max_incoherent = max_incoherent  # cap of the incoherent density in the initial spread
        self.n_out = 2 * nx * ny + 1
        self.widths = [len(FEATURES), *hidden, self.n_out]
        self.net = twmc.MLP(self.widths, max_batch, seed)
        self.max_batch = max_batch
        self.mean = None
        self.std = None

    def fit(self, x: np.ndarray, rows, epochs: int = 400, batch: int = 64, lr: float = 2e-3,
            lr_final: float = 1e-4, floor_frac: float = 0.05, seed: int = 0) -> FitReport:
        """Squashes and standardises the rows (device, [P][2N+1]) and trains
        with Adam on minibatches (learning rate cosine-annealed from lr to
        lr_final), the loss weighted per column by its spread across points."""
        torch = _torch()
        P = rows.shape[0]
        t = rows.clone()
        self.mean = torch.zeros(self.n_out, dtype=torch.float32, device="cuda")
        self.std = torch.zeros(self.n_out, dtype=torch.float32, device="cuda")
        self.weights = torch.zeros(self.n_out, dtype=torch.float32, device="cuda")
        twmc.mlp_standardize(t.data_ptr(), P, self.n_out, floor_frac, self.mean.data_ptr(), self.std.data_ptr(),
                             squash=self.squash, weights_ptr=self.weights.data_ptr())
        xd = torch.as_tensor(np.ascontiguousarray(x, dtype=np.float32)).cuda()
        batch = min(batch, P, self.max_batch)
        g = torch.Generator(device="cuda")
        g.manual_seed(seed)
        rep = FitReport()
        per_epoch = max(1, P // batch)
        total = epochs * per_epoch
        l0 = self.net.launch_count
        for ep in range(epochs):
            perm = torch.randperm(P, device="cuda", generator=g)
            xs = xd.index_select(0, perm).contiguous()
            ts = t.index_select(0, perm).contiguous()
            for j in range(per_epoch):
                step = ep * per_epoch + j
                a = lr_final + 0.5 * (lr - lr_final) * (1 + math.cos(math.pi * step / max(1, total - 1)))
                xb = xs[j * batch:(j + 1) * batch]
                tb = ts[j * batch:(j + 1) * batch]
                self.net.backward(xb.data_ptr(), tb.data_ptr(), batch, self.weights.data_ptr())
                self.net.adam(a)
            if ep % max(1, epochs // 20) == 0 or ep == epochs - 1:
                rep.losses.append((ep, self.net.last_loss()))
        rep.steps = total
        rep.launches = self.net.launch_count - l0
        return rep

    def predict_rows(self, x: np.ndarray):
        """De-standardised, un-squashed MLP rows [P][2N+1] (device float32)."""
        torch = _torch()
        xd = torch.as_tensor(np.ascontiguousarray(x, dtype=np.float32)).cuda()
        y = torch.zeros(xd.shape[0], self.n_out, dtype=torch.float32, device="cuda")
        self.net.forward(xd.data_ptr(), xd.shape[0], y.data_ptr())
        torch.cuda.synchronize()
        v = y * self.std + self.mean
        return self.squash * torch.sinh(v) if self.squash > 0 else v

    def initial_fields(self, x: np.ndarray):
        """(beta_init, beta_sigma): device float64 [P][N][2] each (complex128 layout)."""
        torch = _torch()
        xd = torch.as_tensor(np.ascontiguousarray(x, dtype=np.float32)).cuda()
        P, N = xd.shape[0], self.nx * self.ny
        y = torch.zeros(P, self.n_out, dtype=torch.float32, device="cuda")
        self.net.forward(xd.data_ptr(), P, y.data_ptr())
        bi = torch.zeros(P, N, 2, dtype=torch.float64, device="cuda")
        bs = torch.zeros(P, N, 2, dtype=torch.float64, device="cuda")
        twmc.mlp_fields(y.data_ptr(), self.n_out, P, self.mean.data_ptr(), self.std.data_ptr(), self.nx, self.ny,
                        bi.data_ptr(), bs.data_ptr(), squash=self.squash, max_incoherent=self.max_incoherent)
        torch.cuda.synchronize()
        return bi, bs


@dataclass
class SweepResult:
    times: np.ndarray            # frame times
    n: np.ndarray                # [P][frames] site-averaged density
    n_se: np.ndarray
    g2: np.ndarray
    g2_se: np.ndarray
    ttss: np.ndarray             # [P] time to steady state
    n_inf: np.ndarray            # [P] steady density (tail mean)
    n_inf_se: np.ndarray
    g2_inf: np.ndarray
    g2_inf_se: np.ndarray
    site_updates: int = 0
    device_ms: float = 0.0


def run_sweep(points, nx, ny, n_traj, t_end, dt=0.002, frame_period=0.5, init=None, seed0=1, tail=0.25,
              tune=False):
    """Runs every point from t = 0 to t_end (vacuum start, or `init` =
    (beta_init, beta_sigma) device arrays [P][N][2] from WarmStart) and
    follows the site-averaged n and g2 frame by frame."""
    frame_steps = max(1, int(math.ceil(frame_period / dt - 1e-9)))
    n_frames = int(round(t_end / (frame_steps * dt)))
    hb = twmc.HBatch(_point_descs(points, nx, ny, n_traj, dt, seed0), frame_steps, tune=tune)
    P, N = len(points), nx * ny
    try:
        if init is not None:
            bi, bs = init
            for i in range(P):
                hb.set_init(i, bi[i].data_ptr(), bs[i].data_ptr())
        series = []
        ms = 0.0
        for f in range(n_frames):
            hb.run(1)
            series.append(hb.block_means())
            ms += hb.sync()
    finally:
        hb.close()
    times = (np.arange(n_frames) + 1) * frame_steps * dt
    n = np.zeros((P, n_frames))
    n_se = np.zeros_like(n)
    g2 = np.zeros_like(n)
    g2_se = np.zeros_like(n)
    for f in range(n_frames):
        for i in range(P):
            o = observables(series[f][i][:, None, :], n_traj)
            n[i, f], n_se[i, f], g2[i, f], g2_se[i, f] = o["n"][0], o["n_se"][0], o["g2"][0], o["g2_se"][0]
    ttss = np.zeros(P)
    n_inf = np.zeros(P)
    k0 = int(np.floor((1.0 - tail) * n_frames))
    for i in range(P):
        ttss[i], n_inf[i] = time_to_steady_state(times, n[i], n_se[i], tail)
    tailn = max(1, n_frames - k0)
    # tail averages; frames are correlated, so the SE of the mean uses the
    # per-frame SE (conservative)
    n_inf_se = n_se[:, k0:].mean(axis=1)
    g2_inf = g2[:, k0:].mean(axis=1)
    g2_inf_se = g2_se[:, k0:].mean(axis=1)
    del tailn
    return SweepResult(times, n, n_se, g2, g2_se, ttss, n_inf, n_inf_se, g2_inf, g2_inf_se,
                       site_updates=P * n_traj * N * frame_steps * n_frames, device_ms=ms)


@dataclass
class WarmSweep:
    warm: SweepResult
    plain: SweepResult
    rerun: np.ndarray            # [P] bool: warm result rejected by the rerun rule
    n_final: np.ndarray          # [P] steady density after the rule
    g2_final: np.ndarray
    init_s: float = 0.0          # wall time of the network inference and initial fields
    warm_s: float = 0.0          # wall time of the warm-started runs
    plain_s: float = 0.0         # wall time of the plain (judge) runs


def rerun_mask(warm: SweepResult, plain: SweepResult, rerun_se=1.0) -> np.ndarray:
    """The rerun rule: a warm-started point is replaced by its plain run when
    its steady density n OR its g2 differs from the plain run's by more than
    rerun_se combined standard errors, or when either is not finite."""
    se_n = np.sqrt(warm.n_inf_se ** 2 + plain.n_inf_se ** 2)
    se_g = np.sqrt(warm.g2_inf_se ** 2 + plain.g2_inf_se ** 2)
    ok_n = np.abs(warm.n_inf - plain.n_inf) <= rerun_se * se_n        # False for NaN
    ok_g = np.abs(warm.g2_inf - plain.g2_inf) <= rerun_se * se_g
    return ~(ok_n & ok_g)


def warm_sweep(ws: WarmStart, points, n_traj, t_end, dt=0.002, frame_period=0.5, seed0=1, rerun_se=1.0,
               tune=False):
    """Warm-started sweep checked against plain runs: a point whose warm steady
    n or g2 differs from the plain one by more than rerun_se combined standard
    errors takes the plain result (rerun_mask)."""
    import time
    torch = _torch()
    t0 = time.perf_counter()
    x = features(points)
    init = ws.initial_fields(x)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    warm = run_sweep(points, ws.nx, ws.ny, n_traj, t_end, dt, frame_period, init=init, seed0=seed0, tune=tune)
    t2 = time.perf_counter()
    plain = run_sweep(points, ws.nx, ws.ny, n_traj, t_end, dt, frame_period, init=None, seed0=seed0 + 1000003,
                      tune=tune)
    t3 = time.perf_counter()
    rerun = rerun_mask(warm, plain, rerun_se)
    n_final = np.where(rerun, plain.n_inf, warm.n_inf)
    g2_final = np.where(rerun, plain.g2_inf, warm.g2_inf)
    return WarmSweep(warm, plain, rerun, n_final, g2_final, init_s=t1 - t0, warm_s=t2 - t1, plain_s=t3 - t2)


def evaluate(L=32, n_train=1024, traj_train=256, t_train=20.0, n_test=64, traj_test=512, t_test=20.0,
             epochs=2000, batch=128, lr=3e-3, tune=False) -> dict:
    """Trains the warm start on plain steady states of n_train sampled points
    of an L x L lattice and compares warm-started against plain runs of
    n_test held-out points: median time to steady state, agreement of the
    steady n and g2 within one combined standard error, reruns, timings."""
    import time
    torch = _torch()
    t0 = time.perf_counter()
    train = sample_points(n_train, seed=101)
    rows, su = steady_rows(train, L, L, n_traj=traj_train, t_end=t_train, tune=tune)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    ws = WarmStart(L, L, max_batch=batch, seed=7)
    rep = ws.fit(features(train), rows, epochs=epochs, batch=batch, lr=lr)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    test = sample_points(n_test, seed=202)
    res = warm_sweep(ws, test, n_traj=traj_test, t_end=t_test, tune=tune)
    t3 = time.perf_counter()
    tw, tp = float(np.median(res.warm.ttss)), float(np.median(res.plain.ttss))
    se_n = np.sqrt(res.warm.n_inf_se ** 2 + res.plain.n_inf_se ** 2)
    se_g = np.sqrt(res.warm.g2_inf_se ** 2 + res.plain.g2_inf_se ** 2)
    ok = np.isfinite(se_g) & np.isfinite(res.warm.g2_inf)
    # wall clock: the sweep's device time per unit of simulated time and
    # point turns each point's time to steady state into seconds; a sweep
    # that stops every point at its steady state costs the sum over points
    per_point_s = res.plain.device_ms * 1e-3 / (len(test) * t_test)
    wall_to_steady_plain = float(np.sum(res.plain.ttss) * per_point_s)
    wall_to_steady_warm = float(np.sum(res.warm.ttss) * per_point_s) + res.init_s
    return {
        "workload": f"{L}x{L} PBC sweep, train {n_train} points x {traj_train} trajectories to t={t_train:g}, "
                    f"test {n_test} held-out points x {traj_test} trajectories to t={t_test:g}, dt=0.002, "
                    f"frames every 0.5; MLP 5-256-256-256-{2 * L * L + 1} BF16, {epochs} epochs",
        "ttss_plain_median": tp, "ttss_warm_median": tw, "speedup_median": tp / max(tw, 0.5),
        "ttss_plain_mean": float(np.mean(res.plain.ttss)), "ttss_warm_mean": float(np.mean(res.warm.ttss)),
        "n_within_1se_frac": float(np.mean(np.abs(res.warm.n_inf - res.plain.n_inf) <= se_n)),
        "g2_within_1se_frac": float(np.mean(np.abs(res.warm.g2_inf - res.plain.g2_inf)[ok] <= se_g[ok]))
        if ok.any() else None,
        "reruns": int(res.rerun.sum()), "test_points": n_test,
        "rerun_rule": "warm point replaced by its plain run when n or g2 differs by > 1 combined SE",
        "final_within_1se": "all points by construction (warm where it agrees, plain otherwise)",
        "wall_s": {
            "to_steady_state_plain": wall_to_steady_plain,
            "to_steady_state_warm": wall_to_steady_warm,
            "to_steady_state_speedup": wall_to_steady_plain / max(wall_to_steady_warm, 1e-9),
            "definition": "sweep that stops each point at its time to steady state: sum over points of "
                          "ttss x the sweep's measured device seconds per point and simulated time unit; warm "
                          "adds the network inference and initial-field draws",
            "training_data": t1 - t0, "fit": t2 - t1, "inference_and_init": res.init_s,
            "warm_runs": res.warm_s, "plain_judge_runs": res.plain_s,
            "warm_total_with_judge": (t1 - t0) + (t2 - t1) + res.init_s + res.warm_s + res.plain_s,
            "plain_only": res.plain_s,
            "note": "every warm point is judged by a full plain run here, so this sweep costs more than plain "
                    "runs alone; the gain is the time to steady state of each point"},
        "train_s": t1 - t0, "train_site_updates_per_s": su / (t1 - t0), "fit_s": t2 - t1,
        "fit_steps": rep.steps, "mlp_launches": rep.launches, "final_loss": rep.losses[-1][1], "sweep_s": t3 - t2,
        "ttss_definition": "first save time with |n - n_inf| <= max(1 SE, 1e-3 n_inf), staying within 2x for "
                           "2 more frames; n_inf = mean of the last quarter of frames",
    }


def main(argv=None):
    import argparse
    import json
    ap = argparse.ArgumentParser(description="Learned warm-start sweep: train on plain steady states, then "
                                             "compare warm-started and plain runs of held-out points.")
    ap.add_argument("--L", type=int, default=32, help="lattice side")
    ap.add_argument("--train", type=int, default=1024, help="training points")
    ap.add_argument("--train-traj", type=int, default=256)
    ap.add_argument("--train-t", type=float, default=20.0)
    ap.add_argument("--test", type=int, default=64, help="held-out sweep points")
    ap.add_argument("--test-traj", type=int, default=512)
    ap.add_argument("--test-t", type=float, default=20.0)
    ap.add_argument("--epochs", type=int, default=2000)
    ap.add_argument("--tune", action="store_true", help="let the batch autotuner pick FFT or real-space kernels")
    a = ap.parse_args(argv)
    r = evaluate(a.L, a.train, a.train_traj, a.train_t, a.test, a.test_traj, a.test_t, epochs=a.epochs, tune=a.tune)
    print(json.dumps(r), flush=True)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
