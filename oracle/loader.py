"""ctypes loader of the C++ oracle (test infrastructure only: used by tests/,
the smoke check and bench.py's CPU-baseline leg, never by the product path)."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build_oracle

_libs = {}

D = C.POINTER(C.c_double)


def _setup(lib):
    lib.orc_philox4x32_10.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    lib.orc_site_normals.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_int64, C.c_int, C.c_void_p]
    lib.orc_fft2d.argtypes = [C.c_void_p, C.c_int64, C.c_int64, C.c_int]
    lib.orc_frame_grid.argtypes = [C.c_double] * 6 + [C.c_int, C.c_void_p]
    lib.orc_base_run.argtypes = [C.c_int64, C.c_int64, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                                 C.c_int64, C.c_int64, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                 C.c_int, C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p]
    lib.orc_split_run.argtypes = lib.orc_base_run.argtypes
    lib.orc_lieb_run.argtypes = [C.c_int64, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                                 C.c_double, C.c_double, C.c_int64, C.c_int64, C.c_int, C.c_void_p, C.c_void_p,
                                 C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                                 C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p]
    lib.orc_thermo_run.argtypes = [C.c_int64, C.c_int64, C.c_double, C.c_double, C.c_double, C.c_double,
                                   C.c_double, C.c_int64, C.c_int64, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                   C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_uint32,
                                   C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.orc_time_table_eval.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, C.c_void_p, C.c_int64,
                                        C.c_void_p]
    lib.orc_initial_field.argtypes = [C.c_int64, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_int]
    lib.orc_disorder.argtypes = [C.c_int64, C.c_int, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32,
                                 C.c_void_p, C.c_int]
    lib.orc_base_run_batch.argtypes = [C.c_int64, C.c_int64, C.c_double, C.c_double, C.c_double, C.c_double,
                                       C.c_double, C.c_int64, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.c_int64, C.c_uint32, C.c_int, C.c_void_p, C.c_int]
    lib.orc_base_run_batch.restype = C.c_int64
    return lib


def load(fast: bool = False):
    if fast in _libs:
        return _libs[fast]
    path = build_oracle.lib_path(fast)
    if not os.path.exists(path):
        build_oracle.build()
    lib = _setup(C.CDLL(path))
    _libs[fast] = lib
    return lib


def _c(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.complex128))


def philox(ctr, key):
    lib = load()
    ctr = np.ascontiguousarray(np.asarray(ctr, dtype=np.uint32).reshape(-1, 4))
    key = np.ascontiguousarray(np.asarray(key, dtype=np.uint32).reshape(2))
    out = np.zeros_like(ctr)
    for i in range(ctr.shape[0]):
        lib.orc_philox4x32_10(ctr[i].ctypes.data, key.ctypes.data, out[i].ctypes.data)
    return out


def site_normals(seed, tid, step, stream, n, f32=False):
    out = np.zeros(n, dtype=np.complex128)
    load().orc_site_normals(seed, tid, step, stream, n, int(f32), out.ctypes.data)
    return out


def frame_grid(t_start, t_end, timestep, frames_freq=0.0, frames_period=0.0, n_frames=0.0, store_initial=True):
    out = np.zeros(5)
    load().orc_frame_grid(t_start, t_end, timestep, frames_freq, frames_period, n_frames, int(store_initial),
                          out.ctypes.data)
    return {"frame_steps": int(out[0]), "dt_obs": out[1], "nFramesTot": int(out[2]), "t_end": out[3],
            "n_frames": int(out[4])}


NOISE = {"buffer": 0, "philox64": 1, "philox32": 2, "mt19937": 3}


def base_run(nx, ny, J, gamma, dt, t_start, t_end, frame_steps, n_frames, store_initial, omega, U, F, beta0,
             xi=None, seed=0, tid=0, noise="buffer", fast=False, integrator="euler"):
    n = nx * ny
    om, u, f = (_c(np.broadcast_to(v, (n,))) for v in (omega, U, F))
    beta = _c(beta0).copy()
    frames = np.zeros((max(n_frames, 1), n), dtype=np.complex128)
    meta = np.zeros(3)
    xi_c = _c(xi) if xi is not None else None
    lib = load(fast)
    run = {"euler": lib.orc_base_run, "split": lib.orc_split_run}[integrator]
    run(nx, ny, J, gamma, dt, t_start, t_end, frame_steps, n_frames, int(store_initial),
        om.ctypes.data, u.ctypes.data, f.ctypes.data, beta.ctypes.data, NOISE[noise],
        None if xi_c is None else xi_c.ctypes.data, seed, tid, frames.ctypes.data, meta.ctypes.data)
    return {"frames": frames[: int(meta[0])], "final": beta, "frames_written": int(meta[0]), "t_final": meta[1],
            "steps": int(meta[2])}


def thermo_run(nx, ny, J, gamma, dt, t_start, t_end, frame_steps, n_frames, store_initial, omega, U, F, beta0,
               F_t=None, xi=None, seed=0, tid=0, noise="buffer"):
    """Square lattice with an F(t) table and the drive's work / area datasets."""
    n = nx * ny
    om, u, f = (_c(np.broadcast_to(v, (n,))) for v in (omega, U, F))
    beta = _c(beta0).copy()
    nf = max(n_frames, 1)
    frames = np.zeros((nf, n), dtype=np.complex128)
    work = np.zeros((nf, n))
    area = np.zeros((nf, n))
    meta = np.zeros(3)
    xi_c = _c(xi) if xi is not None else None
    if F_t is not None:
        ft_t = np.ascontiguousarray(np.asarray(F_t[0], dtype=np.float64))
        ft_v = _c(F_t[1])
        nrec = len(ft_t)
    else:
        ft_t = ft_v = None
        nrec = 0
    load().orc_thermo_run(nx, ny, J, gamma, dt, t_start, t_end, frame_steps, n_frames, int(store_initial),
                          om.ctypes.data, u.ctypes.data, f.ctypes.data, nrec,
                          None if ft_t is None else ft_t.ctypes.data, None if ft_v is None else ft_v.ctypes.data,
                          beta.ctypes.data, NOISE[noise], None if xi_c is None else xi_c.ctypes.data, seed, tid,
                          frames.ctypes.data, work.ctypes.data, area.ctypes.data, meta.ctypes.data)
    k = int(meta[0])
    return {"frames": frames[:k], "work": work[:k], "area": area[:k], "final": beta, "frames_written": k,
            "t_final": meta[1], "steps": int(meta[2])}


def lieb_run(ncell, pbc, J_AB, J_BC, detuning, gamma, dt, t_start, t_end, frame_steps, n_frames, store_initial,
             E, U, F, beta0, xi=None, seed=0, tid=0, noise="buffer", F_t=None):
    n = 3 * ncell
    e, u, f = (_c(np.broadcast_to(v, (n,))) for v in (E, U, F))
    beta = _c(beta0).copy()
    frames = np.zeros((max(n_frames, 1), n), dtype=np.complex128)
    meta = np.zeros(3)
    xi_c = _c(xi) if xi is not None else None
    if F_t is not None:
        ft_t = np.ascontiguousarray(np.asarray(F_t[0], dtype=np.float64))
        ft_v = _c(F_t[1])
        nrec = len(ft_t)
    else:
        ft_t = ft_v = None
        nrec = 0
    load().orc_lieb_run(ncell, int(pbc), J_AB, J_BC, detuning, gamma, dt, t_start, t_end, frame_steps, n_frames,
                        int(store_initial), e.ctypes.data, u.ctypes.data, f.ctypes.data, nrec,
                        None if ft_t is None else ft_t.ctypes.data, None if ft_v is None else ft_v.ctypes.data,
                        beta.ctypes.data, NOISE[noise], None if xi_c is None else xi_c.ctypes.data, seed, tid,
                        frames.ctypes.data, meta.ctypes.data)
    return {"frames": frames[: int(meta[0])], "final": beta, "frames_written": int(meta[0]), "t_final": meta[1],
            "steps": int(meta[2])}


def time_table_eval(times, vals, ts):
    times = np.ascontiguousarray(np.asarray(times, dtype=np.float64))
    vals = _c(vals)
    nrec, nsite = vals.shape
    ts = np.ascontiguousarray(np.asarray(ts, dtype=np.float64))
    out = np.zeros((len(ts), nsite), dtype=np.complex128)
    load().orc_time_table_eval(times.ctypes.data, vals.ctypes.data, nrec, nsite, ts.ctypes.data, len(ts),
                               out.ctypes.data)
    return out


def initial_field(n, binit, bsigma, seed, tid, f32=False):
    bi, bs = _c(np.broadcast_to(binit, (n,))), _c(np.broadcast_to(bsigma, (n,)))
    out = np.zeros(n, dtype=np.complex128)
    load().orc_initial_field(n, bi.ctypes.data, bs.ctypes.data, seed, tid, out.ctypes.data, int(f32))
    return out


def disorder(n, kind, base, amp, seed, tid, stream, f32=False):
    b, a = _c(np.broadcast_to(base, (n,))), _c(np.broadcast_to(amp, (n,)))
    out = np.zeros(n, dtype=np.complex128)
    load().orc_disorder(n, kind, b.ctypes.data, a.ctypes.data, seed, tid, stream, out.ctypes.data, int(f32))
    return out
