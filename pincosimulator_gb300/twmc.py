"""ctypes binding of libtwmc_cuda.so (include/twmc.h).

This is the Python-side caller of the C ABI, the same boundary a C++
Solver plugin or any FFI binds. There is no CPU fallback: constructing a
`System` without the compiled library, or without a CUDA device, raises.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass
from typing import Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libtwmc_cuda.so")

# enums (twmc.h)
OK, ERR_INVALID, ERR_CUDA, ERR_TIMEOUT, ERR_NONFINITE, ERR_NOMEM, ERR_NOT_BUILT = 0, -1, -2, -3, -4, -5, -6
LATTICE_SQUARE, LATTICE_LIEB = 0, 1
PREC_F32, PREC_F64 = 0, 1
NOISE_PHILOX, NOISE_BUFFER = 0, 1
HOP_FFT, HOP_STENCIL = 0, 1
INTEGRATOR_EULER, INTEGRATOR_SPLIT = 0, 1
IC_SETTINGS, IC_FIXED, IC_GIVEN = 0, 1, 2
DISORDER_NONE, DISORDER_GAUSSIAN, DISORDER_UNIFORM = 0, 1, 2

EXPORTED = [
    "twmc_version", "twmc_create", "twmc_run", "twmc_set_noise_buffer", "twmc_progress", "twmc_last_error",
    "twmc_destroy", "twmc_batch_init", "twmc_batch_advance", "twmc_batch_reduce", "twmc_sync",
    "twmc_batch_download", "twmc_launch_count", "twmc_kernel_name", "twmc_stream", "twmc_measure_fp32_peak",
    "twmc_kspace_moments_noalloc", "twmc_debug_philox", "twmc_debug_wiener",
    "twmc_hbatch_create", "twmc_hbatch_create_variants", "twmc_hbatch_run", "twmc_hbatch_sync", "twmc_hbatch_moments", "twmc_hbatch_state",
    "twmc_hbatch_plan", "twmc_hbatch_last_error", "twmc_hbatch_launch_count", "twmc_hbatch_destroy",
    "twmc_hbatch_set_init", "twmc_hbatch_field_moments", "twmc_hbatch_total_sites", "twmc_hbatch_stream",
    "twmc_hbatch_block_means",
    "twmc_mlp_create", "twmc_mlp_param_count", "twmc_mlp_set_params", "twmc_mlp_get_params", "twmc_mlp_get_grads",
    "twmc_mlp_forward", "twmc_mlp_backward", "twmc_mlp_adam", "twmc_mlp_last_loss", "twmc_mlp_last_error",
    "twmc_mlp_launch_count", "twmc_mlp_destroy", "twmc_mlp_standardize", "twmc_mlp_targets", "twmc_mlp_fields",
]


class Matrix(C.Structure):
    _fields_ = [("base", C.c_void_p), ("noise_kind", C.c_int32), ("noise_amp", C.c_void_p)]


class SystemDesc(C.Structure):
    _fields_ = [
        ("lattice", C.c_int32), ("nx", C.c_int64), ("ny", C.c_int64), ("pbc", C.c_int32),
        ("J", C.c_double), ("J_AB", C.c_double), ("J_BC", C.c_double), ("gamma", C.c_double),
        ("detuning", C.c_double), ("dt", C.c_double), ("frame_steps", C.c_int64),
        ("omega", Matrix), ("U", Matrix), ("F", Matrix), ("beta_init", Matrix), ("beta_init_sigma", Matrix),
        ("ft_nrec", C.c_int64), ("ft_times", C.c_void_p), ("ft_values", C.c_void_p),
        ("precision", C.c_int32), ("noise_mode", C.c_int32), ("hop_mode", C.c_int32), ("n_moment_blocks", C.c_int32),
        ("thermo", C.c_int32), ("integrator", C.c_int32),
    ]


class TaskDesc(C.Structure):
    _fields_ = [
        ("id", C.c_uint64), ("seed", C.c_uint32), ("ic_kind", C.c_int32), ("t_start", C.c_double),
        ("t_end", C.c_double), ("store_initial", C.c_int32), ("init_field", C.c_void_p),
        ("U_realization", C.c_void_p), ("omega_realization", C.c_void_p), ("F_realization", C.c_void_p),
    ]


class PointDesc(C.Structure):
    _fields_ = [
        ("nx", C.c_int64), ("ny", C.c_int64), ("J", C.c_double), ("gamma", C.c_double), ("dt", C.c_double),
        ("omega", C.c_double * 2), ("U", C.c_double * 2), ("F", C.c_double * 2), ("beta_init", C.c_double * 2),
        ("beta_init_sigma", C.c_double * 2), ("n_traj", C.c_int64), ("seed0", C.c_uint32), ("id0", C.c_uint64),
        ("n_moment_blocks", C.c_int32),
    ]


class Outputs(C.Structure):
    _fields_ = [
        ("frames", C.c_void_p), ("final_field", C.c_void_p), ("U_realization", C.c_void_p),
        ("omega_realization", C.c_void_p), ("F_realization", C.c_void_p), ("moments", C.c_void_p),
        ("frames_written", C.c_void_p), ("t_final", C.c_void_p), ("status", C.c_void_p),
        ("work", C.c_void_p), ("area", C.c_void_p),
    ]


_lib = None


def load(path: Optional[str] = None):
    """Loads the C-ABI library ($TWMC_LIB if set); raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or os.environ.get("TWMC_LIB") or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(f"libtwmc_cuda.so not built ({path}); run __graft_entry__.build()")
    lib = C.CDLL(path)
    lib.twmc_version.restype = C.c_int
    lib.twmc_create.argtypes = [C.POINTER(SystemDesc), C.POINTER(C.c_void_p)]
    lib.twmc_run.argtypes = [C.c_void_p, C.POINTER(TaskDesc), C.c_size_t, C.POINTER(Outputs)]
    lib.twmc_set_noise_buffer.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t]
    lib.twmc_progress.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
    lib.twmc_last_error.argtypes = [C.c_void_p]
    lib.twmc_last_error.restype = C.c_char_p
    lib.twmc_destroy.argtypes = [C.c_void_p]
    lib.twmc_destroy.restype = None
    lib.twmc_batch_init.argtypes = [C.c_void_p, C.POINTER(TaskDesc), C.c_size_t]
    lib.twmc_batch_advance.argtypes = [C.c_void_p, C.c_int64]
    lib.twmc_batch_reduce.argtypes = [C.c_void_p]
    lib.twmc_sync.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
    lib.twmc_batch_download.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    lib.twmc_launch_count.argtypes = [C.c_void_p]
    lib.twmc_launch_count.restype = C.c_int64
    lib.twmc_kernel_name.argtypes = [C.c_void_p]
    lib.twmc_kernel_name.restype = C.c_char_p
    lib.twmc_debug_philox.argtypes = [C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p]
    lib.twmc_debug_wiener.argtypes = [C.c_int32, C.c_uint32, C.c_uint64, C.c_uint32, C.c_int64, C.c_int64,
                                      C.c_void_p]
    lib.twmc_stream.argtypes = [C.c_void_p]
    lib.twmc_stream.restype = C.c_void_p
    lib.twmc_measure_fp32_peak.argtypes = [C.POINTER(C.c_double)]
    lib.twmc_hbatch_create.argtypes = [C.POINTER(PointDesc), C.c_size_t, C.c_int64, C.c_int32, C.POINTER(C.c_void_p)]
    lib.twmc_hbatch_create_variants.argtypes = [C.POINTER(PointDesc), C.c_size_t, C.c_int64,
                                                C.POINTER(C.c_char_p), C.POINTER(C.c_void_p)]
    lib.twmc_hbatch_run.argtypes = [C.c_void_p, C.c_int64]
    lib.twmc_hbatch_sync.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
    lib.twmc_hbatch_moments.argtypes = [C.c_void_p, C.c_size_t, C.c_void_p]
    lib.twmc_hbatch_state.argtypes = [C.c_void_p, C.c_size_t, C.c_void_p]
    lib.twmc_hbatch_plan.argtypes = [C.c_void_p, C.c_size_t]
    lib.twmc_hbatch_plan.restype = C.c_char_p
    lib.twmc_hbatch_last_error.argtypes = [C.c_void_p]
    lib.twmc_hbatch_last_error.restype = C.c_char_p
    lib.twmc_hbatch_launch_count.argtypes = [C.c_void_p]
    lib.twmc_hbatch_launch_count.restype = C.c_int64
    lib.twmc_hbatch_destroy.argtypes = [C.c_void_p]
    lib.twmc_hbatch_destroy.restype = None
    lib.twmc_kspace_moments_noalloc.argtypes = [C.c_void_p, C.c_int64, C.c_int64, C.c_int64, C.c_int32,
                                                C.c_void_p, C.c_void_p]
    lib.twmc_hbatch_set_init.argtypes = [C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p]
    lib.twmc_hbatch_field_moments.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32]
    lib.twmc_hbatch_total_sites.argtypes = [C.c_void_p]
    lib.twmc_hbatch_total_sites.restype = C.c_int64
    lib.twmc_hbatch_block_means.argtypes = [C.c_void_p, C.c_void_p]
    lib.twmc_hbatch_stream.argtypes = [C.c_void_p]
    lib.twmc_hbatch_stream.restype = C.c_void_p
    lib.twmc_mlp_create.argtypes = [C.c_int32, C.c_void_p, C.c_int64, C.c_uint64, C.POINTER(C.c_void_p)]
    lib.twmc_mlp_param_count.argtypes = [C.c_void_p]
    lib.twmc_mlp_param_count.restype = C.c_int64
    for f in ("twmc_mlp_set_params", "twmc_mlp_get_params", "twmc_mlp_get_grads", "twmc_mlp_last_loss"):
        getattr(lib, f).argtypes = [C.c_void_p, C.c_void_p]
    lib.twmc_mlp_forward.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]
    lib.twmc_mlp_backward.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p,
                                      C.c_void_p]
    lib.twmc_mlp_adam.argtypes = [C.c_void_p, C.c_float, C.c_float, C.c_float, C.c_float, C.c_void_p]
    lib.twmc_mlp_last_error.argtypes = [C.c_void_p]
    lib.twmc_mlp_last_error.restype = C.c_char_p
    lib.twmc_mlp_launch_count.argtypes = [C.c_void_p]
    lib.twmc_mlp_launch_count.restype = C.c_int64
    lib.twmc_mlp_destroy.argtypes = [C.c_void_p]
    lib.twmc_mlp_destroy.restype = None
    lib.twmc_mlp_standardize.argtypes = [C.c_void_p, C.c_int64, C.c_int32, C.c_double, C.c_float, C.c_void_p,
                                         C.c_void_p, C.c_void_p, C.c_void_p]
    lib.twmc_mlp_targets.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, C.c_int64, C.c_int32,
                                     C.c_void_p, C.c_int64, C.c_void_p]
    lib.twmc_mlp_fields.argtypes = [C.c_void_p, C.c_int64, C.c_int64, C.c_void_p, C.c_void_p, C.c_double,
                                    C.c_double, C.c_int64, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]
    _lib = lib
    return lib


class TWMCError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"twmc error {code}: {msg}")
        self.code = code


def _cplx(v, n: int) -> np.ndarray:
    a = np.asarray(v, dtype=np.complex128)
    if a.ndim == 0:
        a = np.full(n, complex(a), dtype=np.complex128)
    a = np.ascontiguousarray(a.reshape(-1))
    if a.size != n:
        raise ValueError(f"expected {n} values, got {a.size}")
    return a


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data


@dataclass
class Noisy:
    """A parameter matrix: base value(s) plus an optional per-trajectory disorder draw."""
    base: object = 0.0
    kind: int = DISORDER_NONE
    amp: object = 0.0


class System:
    """One lattice system (the reference's TWMCSystemData + solver Setup)."""

    def __init__(self, *, lattice=LATTICE_SQUARE, nx=1, ny=1, pbc=True, J=0.0, J_AB=0.0, J_BC=0.0, gamma=1.0,
                 detuning=0.0, dt=0.01, frame_steps=1, omega=0.0, U=0.0, F=0.0, beta_init=0.0, beta_init_sigma=0.0,
                 F_t: Optional[tuple] = None, precision=PREC_F32, noise=NOISE_PHILOX, hop=HOP_FFT, n_moment_blocks=32,
                 thermo=False, integrator=INTEGRATOR_EULER):
        self.lib = load()
        self.n_sites = (3 if lattice == LATTICE_LIEB else 1) * nx * ny
        n = self.n_sites
        self._keep = []
        d = SystemDesc()
        d.lattice, d.nx, d.ny, d.pbc = lattice, nx, ny, int(bool(pbc))
        d.J, d.J_AB, d.J_BC, d.gamma, d.detuning, d.dt = J, J_AB, J_BC, gamma, detuning, dt
        d.frame_steps = frame_steps
        for name, val in (("omega", omega), ("U", U), ("F", F), ("beta_init", beta_init),
                          ("beta_init_sigma", beta_init_sigma)):
            nv = val if isinstance(val, Noisy) else Noisy(base=val)
            base = _cplx(nv.base, n)
            amp = _cplx(nv.amp, n)
            self._keep += [base, amp]
            setattr(d, name, Matrix(base.ctypes.data, nv.kind, amp.ctypes.data if nv.kind else None))
        if F_t is not None:
            times, vals = F_t
            times = np.ascontiguousarray(np.asarray(times, dtype=np.float64))
            vals = np.ascontiguousarray(np.asarray(vals, dtype=np.complex128).reshape(len(times), n))
            self._keep += [times, vals]
            d.ft_nrec, d.ft_times, d.ft_values = len(times), times.ctypes.data, vals.ctypes.data
        d.precision, d.noise_mode, d.hop_mode, d.n_moment_blocks = precision, noise, hop, n_moment_blocks
        d.thermo = int(bool(thermo))
        d.integrator = integrator
        self.thermo = bool(thermo)
        self.desc = d
        self.n_blocks = n_moment_blocks
        self.precision = precision
        h = C.c_void_p()
        rc = self.lib.twmc_create(C.byref(d), C.byref(h))
        self.h = h
        if rc != OK:
            msg = self.last_error()
            self.close()
            raise TWMCError(rc, msg)

    # -- plumbing --------------------------------------------------------
    def last_error(self) -> str:
        if not self.h:
            return ""
        return self.lib.twmc_last_error(self.h).decode()

    def _check(self, rc: int):
        if rc != OK:
            raise TWMCError(rc, self.last_error())

    def close(self):
        if getattr(self, "h", None):
            self.lib.twmc_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def kernel_name(self) -> str:
        return self.lib.twmc_kernel_name(self.h).decode()

    @property
    def stream(self) -> int:
        """cudaStream_t of the handle (an integer address)."""
        return int(self.lib.twmc_stream(self.h) or 0)

    @property
    def launch_count(self) -> int:
        return int(self.lib.twmc_launch_count(self.h))

    # -- tasks -----------------------------------------------------------
    def make_tasks(self, n: int, *, t_start=0.0, t_end=1.0, seed0=1234, id0=1, store_initial=True,
                   ic=IC_SETTINGS, init_field=None, seeds: Optional[Sequence[int]] = None,
                   realizations: Optional[dict] = None):
        """n task descriptors. `realizations` may give the disorder
        realisations per task ({"U" | "omega" | "F": (n, n_sites) complex}),
        as a continuation run passes the stored datasets."""
        tasks = (TaskDesc * n)()
        keep = []
        if init_field is not None:
            f = np.ascontiguousarray(np.asarray(init_field, dtype=np.complex128).reshape(n, self.n_sites))
            keep.append(f)
        given = {}
        for name, arr in (realizations or {}).items():
            given[name] = np.ascontiguousarray(np.asarray(arr, dtype=np.complex128).reshape(n, self.n_sites))
            keep.append(given[name])
        for i in range(n):
            t = tasks[i]
            t.id = id0 + i
            t.seed = (seeds[i] if seeds is not None else seed0 + i) & 0xFFFFFFFF
            t.ic_kind = ic
            t.t_start, t.t_end = t_start, t_end
            t.store_initial = int(bool(store_initial))
            if init_field is not None:
                t.init_field = f[i].ctypes.data
            for name, arr in given.items():
                setattr(t, name + "_realization", arr[i].ctypes.data)
        self._keep.append(keep)
        return tasks

    def set_noise(self, xi: np.ndarray):
        """Deterministic-noise mode: xi[task][step][site] complex normals."""
        xi = np.ascontiguousarray(np.asarray(xi, dtype=np.complex128))
        self._noise = xi
        self._check(self.lib.twmc_set_noise_buffer(self.h, xi.ctypes.data, xi.size))

    def run(self, tasks, *, frames=True, final=True, moments=False, realizations=False, n_frames=None,
            buffers: Optional[dict] = None):
        """twmc_run: returns a dict of numpy arrays. `buffers` may supply
        preallocated C-contiguous arrays for "frames", "final" and "moments"
        (e.g. views of pinned host memory reused across calls); the others are
        allocated here."""
        n = len(tasks)
        N = self.n_sites
        if n_frames is None:
            dt_obs = self.desc.dt * self.desc.frame_steps
            n_frames = max(int(round((t.t_end - t.t_start) / dt_obs)) + int(t.store_initial) for t in tasks)
        buffers = buffers or {}

        def buf(key, shape, dtype):
            b = buffers.get(key)
            if b is None:
                return np.zeros(shape, dtype=dtype)
            if b.shape != shape or b.dtype != dtype or not b.flags["C_CONTIGUOUS"]:
                raise ValueError(f"buffer {key}: need C-contiguous {dtype} of shape {shape}")
            return b

        out = Outputs()
        res = {}
        if frames:
            res["frames"] = buf("frames", (n, n_frames, N), np.complex128)
            out.frames = res["frames"].ctypes.data
        if final:
            res["final"] = buf("final", (n, N), np.complex128)
            out.final_field = res["final"].ctypes.data
        if moments:
            res["moments"] = buf("moments", (n_frames, self.n_blocks, N, 3), np.float64)
            out.moments = res["moments"].ctypes.data
        if realizations:
            for key in ("U_realization", "omega_realization", "F_realization"):
                res[key] = np.zeros((n, N), dtype=np.complex128)
                setattr(out, key, res[key].ctypes.data)
        if self.thermo and frames:
            for key in ("work", "area"):
                res[key] = np.zeros((n, n_frames, N), dtype=np.float64)
                setattr(out, key, res[key].ctypes.data)
        res["frames_written"] = np.zeros(n, dtype=np.int64)
        res["t_final"] = np.zeros(n, dtype=np.float64)
        res["status"] = np.zeros(n, dtype=np.int32)
        out.frames_written = res["frames_written"].ctypes.data
        out.t_final = res["t_final"].ctypes.data
        out.status = res["status"].ctypes.data
        self._check(self.lib.twmc_run(self.h, tasks, n, C.byref(out)))
        return res

    # -- device-resident batch API ---------------------------------------
    def batch_init(self, tasks):
        self._check(self.lib.twmc_batch_init(self.h, tasks, len(tasks)))
        self._batch_n = len(tasks)

    def advance(self, n_steps: int):
        self._check(self.lib.twmc_batch_advance(self.h, int(n_steps)))

    def reduce(self):
        self._check(self.lib.twmc_batch_reduce(self.h))

    def sync(self) -> float:
        ms = C.c_double()
        self._check(self.lib.twmc_sync(self.h, C.byref(ms)))
        return ms.value

    def download(self, field=True, moments=False):
        f = np.zeros((self._batch_n, self.n_sites), dtype=np.complex128) if field else None
        m = np.zeros((self.n_blocks, self.n_sites, 3), dtype=np.float64) if moments else None
        self._check(self.lib.twmc_batch_download(self.h, _ptr(f), _ptr(m)))
        return f, m


def _c2(v):
    v = complex(v)
    return (C.c_double * 2)(v.real, v.imag)


class HBatch:
    """Heterogeneous batch of parameter points (twmc_hbatch_*)."""

    VARIANTS = ("fft", "ell2", "ell4", "ell8", "rowrun", "ell8w", "cluster_pow2", "cluster")

    def __init__(self, points, frame_steps: int, tune: bool = False, variants: Optional[Sequence[str]] = None):
        """variants: a step variant name per point (twmc_hbatch_create_variants);
        None = the default choice, or the autotuner's with tune=True."""
        self.lib = load()
        arr = (PointDesc * len(points))()
        self.n_sites = []
        self.n_traj = []
        self.n_blocks = []
        for i, p in enumerate(points):
            d = arr[i]
            d.nx, d.ny = p.get("nx", 1), p["ny"]
            d.J, d.gamma, d.dt = p.get("J", 1.0), p.get("gamma", 1.0), p["dt"]
            d.omega, d.U, d.F = _c2(p.get("omega", 0)), _c2(p.get("U", 0)), _c2(p.get("F", 0))
            d.beta_init, d.beta_init_sigma = _c2(p.get("beta_init", 0)), _c2(p.get("beta_init_sigma", 0.5))
            d.n_traj, d.seed0, d.id0 = p["n_traj"], p.get("seed0", 1), p.get("id0", 1)
            d.n_moment_blocks = p.get("n_moment_blocks", 32)
            self.n_sites.append(d.nx * d.ny)
            self.n_traj.append(d.n_traj)
            self.n_blocks.append(min(d.n_moment_blocks or 32, d.n_traj))
        h = C.c_void_p()
        if variants is not None:
            names = (C.c_char_p * len(points))(*[v.encode() for v in variants])
            rc = self.lib.twmc_hbatch_create_variants(arr, len(points), frame_steps, names, C.byref(h))
        else:
            rc = self.lib.twmc_hbatch_create(arr, len(points), frame_steps, int(tune), C.byref(h))
        self.h = h
        if rc != OK:
            msg = self.lib.twmc_hbatch_last_error(h).decode() if h else ""
            self.close()
            raise TWMCError(rc, msg)

    def _check(self, rc):
        if rc != OK:
            raise TWMCError(rc, self.lib.twmc_hbatch_last_error(self.h).decode())

    def run(self, n_frames: int):
        self._check(self.lib.twmc_hbatch_run(self.h, n_frames))

    def sync(self) -> float:
        ms = C.c_double()
        self._check(self.lib.twmc_hbatch_sync(self.h, C.byref(ms)))
        return ms.value

    def state(self, i):
        out = np.zeros((self.n_traj[i], self.n_sites[i]), dtype=np.complex128)
        self._check(self.lib.twmc_hbatch_state(self.h, i, out.ctypes.data))
        return out

    def moments(self, i):
        out = np.zeros((self.n_blocks[i], self.n_sites[i], 3))
        self._check(self.lib.twmc_hbatch_moments(self.h, i, out.ctypes.data))
        return out

    def plan(self, i) -> str:
        return self.lib.twmc_hbatch_plan(self.h, i).decode()

    @property
    def stream(self) -> int:
        """cudaStream_t of the batch (for torch.cuda.ExternalStream)."""
        return int(self.lib.twmc_hbatch_stream(self.h) or 0)

    @property
    def total_sites(self) -> int:
        return int(self.lib.twmc_hbatch_total_sites(self.h))

    def set_init(self, i, beta_init_ptr: int, beta_sigma_ptr: int):
        """Redraws point i's initial fields from per-site device arrays
        (complex128, sites each; 0 = the point's uniform value). Before run()."""
        self._check(self.lib.twmc_hbatch_set_init(self.h, i, beta_init_ptr or None, beta_sigma_ptr or None))

    def block_means(self):
        """Per point: (n_blocks, 3) site averages of the last frame's moment blocks."""
        tot = sum(self.n_blocks)
        out = np.zeros((tot, 3))
        self._check(self.lib.twmc_hbatch_block_means(self.h, out.ctypes.data))
        res, o = [], 0
        for nb in self.n_blocks:
            res.append(out[o:o + nb])
            o += nb
        return res

    def field_moments(self, mean_ptr: int, abs2_ptr: int, accumulate: bool = False):
        """Trajectory means <a> (complex128) and <|a|^2> per site of every point
        into device arrays of total_sites entries (asynchronous on `stream`)."""
        self._check(self.lib.twmc_hbatch_field_moments(self.h, mean_ptr, abs2_ptr, int(accumulate)))

    @property
    def launch_count(self) -> int:
        return int(self.lib.twmc_hbatch_launch_count(self.h))

    def close(self):
        if getattr(self, "h", None):
            self.lib.twmc_hbatch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class MLP:
    """BF16 tensor-core MLP of the learned warm start (twmc_mlp_*). Arrays
    passed to forward / backward are device pointers (e.g. torch tensors'
    data_ptr()); parameters and gradients come back as host FP32 arrays."""

    def __init__(self, widths: Sequence[int], max_batch: int, seed: int = 1):
        self.lib = load()
        self.widths = [int(w) for w in widths]
        w = (C.c_int32 * len(self.widths))(*self.widths)
        h = C.c_void_p()
        rc = self.lib.twmc_mlp_create(len(self.widths) - 1, w, int(max_batch), int(seed), C.byref(h))
        self.h = h
        if rc != OK:
            msg = self.lib.twmc_mlp_last_error(h).decode() if h else ""
            self.close()
            raise TWMCError(rc, msg)
        self.max_batch = int(max_batch)
        self.n_params = int(self.lib.twmc_mlp_param_count(self.h))

    def _check(self, rc):
        if rc != OK:
            raise TWMCError(rc, self.lib.twmc_mlp_last_error(self.h).decode())

    def offsets(self):
        """[(w_off, b_off)] per layer into the parameter array."""
        out, off = [], 0
        for k, n in zip(self.widths[:-1], self.widths[1:]):
            out.append((off, off + n * k))
            off += n * k + n
        return out

    def get_params(self) -> np.ndarray:
        out = np.zeros(self.n_params, dtype=np.float32)
        self._check(self.lib.twmc_mlp_get_params(self.h, out.ctypes.data))
        return out

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.n_params
        self._check(self.lib.twmc_mlp_set_params(self.h, p.ctypes.data))

    def get_grads(self) -> np.ndarray:
        out = np.zeros(self.n_params, dtype=np.float32)
        self._check(self.lib.twmc_mlp_get_grads(self.h, out.ctypes.data))
        return out

    def forward(self, x_ptr: int, batch: int, y_ptr: int, stream: int = 0):
        self._check(self.lib.twmc_mlp_forward(self.h, x_ptr, int(batch), y_ptr, stream or None))

    def backward(self, x_ptr: int, t_ptr: int, batch: int, w_ptr: int = 0, stream: int = 0, want_loss=False):
        loss = C.c_float(0.0)
        self._check(self.lib.twmc_mlp_backward(self.h, x_ptr, t_ptr, w_ptr or None, int(batch),
                                               C.byref(loss) if want_loss else None, stream or None))
        return float(loss.value) if want_loss else None

    def adam(self, lr: float, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8, stream: int = 0):
        self._check(self.lib.twmc_mlp_adam(self.h, lr, beta1, beta2, eps, stream or None))

    def last_loss(self) -> float:
        v = C.c_float()
        self._check(self.lib.twmc_mlp_last_loss(self.h, C.byref(v)))
        return float(v.value)

    @property
    def launch_count(self) -> int:
        return int(self.lib.twmc_mlp_launch_count(self.h))

    def close(self):
        if getattr(self, "h", None):
            self.lib.twmc_mlp_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def mlp_standardize(t_ptr: int, rows: int, cols: int, floor_frac: float, mean_ptr: int, std_ptr: int,
                    squash: float = 0.0, weights_ptr: int = 0, stream: int = 0):
    rc = load().twmc_mlp_standardize(t_ptr, int(rows), int(cols), float(squash), float(floor_frac), mean_ptr,
                                     std_ptr, weights_ptr or None, stream or None)
    if rc != OK:
        raise TWMCError(rc, "twmc_mlp_standardize failed")


def mlp_targets(mean_ptr: int, abs2_ptr: int, n_points: int, nx: int, ny: int, frames: int, rows_ptr: int,
                ld: int, stream: int = 0):
    rc = load().twmc_mlp_targets(mean_ptr, abs2_ptr, int(n_points), int(nx), int(ny), int(frames), rows_ptr,
                                 int(ld), stream or None)
    if rc != OK:
        raise TWMCError(rc, "twmc_mlp_targets failed")


def mlp_fields(rows_ptr: int, ld: int, n_points: int, mean_ptr: int, std_ptr: int, nx: int, ny: int,
               binit_ptr: int, bsigma_ptr: int, squash: float = 0.0, max_incoherent: float = 1e30, stream: int = 0):
    rc = load().twmc_mlp_fields(rows_ptr, int(ld), int(n_points), mean_ptr or None, std_ptr or None,
                                float(squash), float(max_incoherent), int(nx), int(ny), binit_ptr, bsigma_ptr,
                                stream or None)
    if rc != OK:
        raise TWMCError(rc, "twmc_mlp_fields failed")


def measure_fp32_peak() -> float:
    """Measured FP32 FMA throughput of the current device (TFLOP/s)."""
    lib = load()
    v = C.c_double()
    rc = lib.twmc_measure_fp32_peak(C.byref(v))
    if rc != OK:
        raise TWMCError(rc, "FP32 peak measurement failed")
    return v.value


def debug_philox(ctr: np.ndarray, key) -> np.ndarray:
    lib = load()
    ctr = np.ascontiguousarray(np.asarray(ctr, dtype=np.uint32).reshape(-1, 4))
    k = np.ascontiguousarray(np.asarray(key, dtype=np.uint32).reshape(2))
    out = np.zeros_like(ctr)
    rc = lib.twmc_debug_philox(ctr.ctypes.data, ctr.shape[0], k.ctypes.data, out.ctypes.data)
    if rc != OK:
        raise TWMCError(rc, "twmc_debug_philox failed")
    return out


def debug_wiener(precision: int, seed: int, tid: int, n_steps: int, n_sites: int, step0: int = 0) -> np.ndarray:
    """Philox-mode Wiener normals of one trajectory as the step kernels draw
    them: (n_steps, n_sites) complex128."""
    lib = load()
    out = np.zeros((n_steps, n_sites), dtype=np.complex128)
    rc = lib.twmc_debug_wiener(precision, seed & 0xFFFFFFFF, tid, step0 & 0xFFFFFFFF, n_steps, n_sites,
                               out.ctypes.data)
    if rc != OK:
        raise TWMCError(rc, "twmc_debug_wiener failed")
    return out
