"""Heterogeneous batch (persistent work-queue kernels, one CUDA graph per
frame): every point must equal the same point run alone through the handle
API (same seeds and counters), including the FP64 moment blocks, in every
step variant its lattice admits. Real-space variants apply the standalone
real-space kernels' per-site arithmetic and agree bit for bit; FFT points
run the shared step body in a different CTA instantiation (256 threads in
the batch, the shape's own size alone), where the compiler may fuse
multiplies and adds into FMAs differently, so they agree to the FP32 parity
tolerance (1e-5 relative to the largest value of each quantity)."""
import json
import os

import numpy as np
import pytest

from pincosimulator_gb300 import twmc

pytestmark = pytest.mark.gpu

POINTS = [
    dict(nx=1, ny=32, U=0.3, omega=-1.0, F=1.2, n_traj=300, seed0=10, id0=1),
    dict(nx=1, ny=256, U=0.1, omega=0.5, F=2.0, n_traj=70, seed0=20, id0=1000),
    dict(nx=16, ny=16, U=0.2, omega=-0.5, F=1.0, n_traj=37, seed0=30, id0=5000),
    dict(nx=64, ny=64, U=0.2, omega=-0.5, F=2.0, n_traj=9, seed0=40, id0=9000),
    dict(nx=32, ny=32, U=0.45, omega=1.5, F=0.3, n_traj=21, seed0=50, id0=1),
    dict(nx=6, ny=10, U=0.2, omega=0.0, F=1.0, n_traj=13, seed0=60, id0=1),   # no FFT plan: real space
    dict(nx=1, ny=50, U=0.2, omega=0.0, F=1.0, n_traj=11, seed0=70, id0=1),   # no FFT plan: real space
    dict(nx=128, ny=128, U=0.2, omega=-0.5, F=1.5, n_traj=5, seed0=80, id0=1),  # 2-CTA cluster kernel
]
DT, FS = 0.002, 50


def single(p, frames, hop=twmc.HOP_FFT):
    s = twmc.System(nx=p["nx"], ny=p["ny"], J=1.0, gamma=1.0, dt=DT, frame_steps=FS, omega=p["omega"], U=p["U"],
                    F=p["F"], beta_init=0.0, beta_init_sigma=0.5, precision=twmc.PREC_F32, hop=hop,
                    n_moment_blocks=32)
    s.batch_init(s.make_tasks(p["n_traj"], t_end=1.0, seed0=p["seed0"], id0=p["id0"]))
    for _ in range(frames):
        s.advance(FS)
    s.reduce()
    s.sync()
    f, m = s.download(field=True, moments=True)
    kname = s.kernel_name
    s.close()
    return f, m[: min(32, p["n_traj"])], kname


def make(points, tune=False, variants=None):
    pts = [dict(p, dt=DT) for p in points]
    return twmc.HBatch(pts, FS, tune=tune, variants=variants)


def check_point(hb, i, p, frames):
    """Point i of the batch against the point run alone: FFT variants at the
    FP32 tolerance, real-space variants bit for bit (the standalone real-space
    kernel applies the same per-site arithmetic)."""
    plan = hb.plan(i)
    fft = "<fft " in plan
    f, m, kname = single(p, frames, twmc.HOP_FFT if fft else twmc.HOP_STENCIL)
    st = hb.state(i)
    hm = hb.moments(i)
    if fft:
        assert kname.startswith("square_fft_kernel"), (plan, kname)
        e = np.abs(st - f).max() / np.abs(f).max()
        assert e < 1e-5, f"point {i} ({plan}): rel diff {e:.2e}"
        for c in range(3):  # |a|^2, |a|^4, |a_k|^2 block sums, each relative to its largest
            ec = np.abs(hm[..., c] - m[..., c]).max() / np.abs(m[..., c]).max()
            assert ec < 1e-5, f"point {i} moment {c}: rel diff {ec:.2e}"
    else:  # no k-space populations from the real-space variants
        variant = plan.split("<")[1].split(" ")[0]
        family = {"cluster_pow2": "ell_cluster_pow2_kernel", "cluster": "ell_cluster_kernel",
                  "rowrun": "rowrun_kernel"}.get(variant, "ell_kernel")
        if kname.startswith(family):  # the same step body: bit for bit
            assert np.array_equal(st, f), f"point {i} ({plan}): max diff {np.abs(st - f).max()}"
            assert np.array_equal(hm[..., :2], m[..., :2])
        else:  # another body of the same stencil (the compiler may fuse differently): FP32 tolerance
            e = np.abs(st - f).max() / np.abs(f).max()
            assert e < 1e-5, f"point {i} ({plan} vs {kname}): rel diff {e:.2e}"


def test_hbatch_matches_single_point_runs(built_lib):
    hb = make(POINTS)
    hb.run(3)
    hb.sync()
    for i, p in enumerate(POINTS):
        assert hb.plan(i).startswith("hbatch_"), hb.plan(i)  # every point is a work item of a queue kernel
        check_point(hb, i, p, 3)
    assert hb.launch_count >= 3
    hb.close()


VARIANT_POINTS = POINTS + [
    dict(nx=80, ny=80, U=0.2, omega=0.3, F=1.0, n_traj=6, seed0=90, id0=1),     # 6400 sites: general cluster form
    dict(nx=96, ny=128, U=0.2, omega=0.3, F=1.0, n_traj=4, seed0=95, id0=1),    # 12288 sites: general cluster form
    dict(nx=8, ny=64, U=0.25, omega=-1.0, F=0.8, n_traj=40, seed0=99, id0=1),   # 512 sites, every real-space form
]


@pytest.mark.parametrize("variant", twmc.HBatch.VARIANTS)
def test_hbatch_every_variant(built_lib, variant):
    """Each step variant, forced on every point whose lattice admits it,
    inside one batch (its queue kernel alone), against the points run alone."""
    ok = []
    for p in VARIANT_POINTS:
        try:
            make([p], variants=[variant]).close()
            ok.append(p)
        except twmc.TWMCError as e:
            assert e.code == twmc.ERR_INVALID
    if not ok:
        pytest.skip(f"no test lattice admits {variant}")
    hb = make(ok, variants=[variant] * len(ok))
    hb.run(2)
    hb.sync()
    for i, p in enumerate(ok):
        assert f"<{variant} " in hb.plan(i), hb.plan(i)
        check_point(hb, i, p, 2)
    hb.close()


def test_hbatch_autotuner_cache(built_lib, tmp_path, monkeypatch):
    cache = tmp_path / "tune.json"
    monkeypatch.setenv("TWMC_TUNE_CACHE", str(cache))
    hb = make(POINTS[:5], tune=True)
    hb.run(1)
    hb.sync()
    entries = json.loads(cache.read_text())
    assert len(entries) == 5 and set(entries.values()) <= set(twmc.HBatch.VARIANTS)
    for i, p in enumerate(POINTS[:5]):
        key = [k for k in entries if k.endswith(f"|{p['nx']}x{p['ny']}")][0]
        assert f"<{entries[key]} " in hb.plan(i)
        assert np.isfinite(hb.state(i)).all()
    hb.close()
    # a second batch reads the cache instead of timing again
    mtime = os.path.getmtime(cache)
    hb2 = make(POINTS[:5], tune=True)
    hb2.close()
    assert os.path.getmtime(cache) == mtime
