"""The allocation-free entry point against the library's own path (GPU).

twmc_kspace_moments_noalloc serves callers that cannot allocate device
memory (a host application whose own memory pool already owns the device,
or a loop where cudaMalloc's implicit synchronisation is not acceptable).
This test plays such a caller: the batch state and the output buffer are
its own device buffers (allocated here with torch, outside the entry point),
and the entry point must produce the moment blocks that the library's
twmc_batch_advance + twmc_batch_reduce path produces for the same state,
within the FP32 tolerance of the parity tests, on two calls in a row (the
second call, with fewer trajectories, reuses the scratch array the first
one left filled). The file sorts last so that a run stopping at the first
failure has run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from pincosimulator_gb300 import twmc

pytestmark = pytest.mark.gpu

TOL = 1e-5  # FP32 tolerance of the parity tests


def library_moments(nx, ny, ntraj, seed, nblocks):
    s = twmc.System(nx=nx, ny=ny, J=1.0, gamma=1.0, dt=0.002, frame_steps=250,
                    omega=twmc.Noisy(-0.5, twmc.DISORDER_GAUSSIAN, 0.2), U=0.2, F=2.0, beta_init_sigma=0.5,
                    precision=twmc.PREC_F32, n_moment_blocks=nblocks)
    s.batch_init(s.make_tasks(ntraj, t_end=10.0, seed0=seed))
    s.advance(20)  # also writes |FFT(state)|^2 / N for the reduction
    s.reduce()
    s.sync()
    field, moments = s.download(field=True, moments=True)
    s.close()
    return field, moments


@pytest.mark.parametrize("nx,ny,runs", [
    (64, 64, ((600, 11), (97, 23))),    # one trajectory per CTA
    (32, 32, ((1001, 5), (333, 6))),    # several trajectories per CTA
    (16, 16, ((2049, 7), (37, 8))),     # n_traj not a multiple of the trajectories per CTA
    (1, 256, ((777, 9), (65, 10))),     # 1-D chain plan
])
def test_noalloc_matches_library_path_twice(built_lib, nx, ny, runs):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    lib = twmc.load()
    nb = 16
    for ntraj, seed in runs:
        field, ref = library_moments(nx, ny, ntraj, seed, nb)
        # the caller's own device buffers: complex64 state, FP64 output
        state = torch.from_numpy(field.astype(np.complex64)).cuda()
        out = torch.full((nb, nx * ny, 3), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        rc = lib.twmc_kspace_moments_noalloc(C.c_void_p(state.data_ptr()), ntraj, nx, ny, nb,
                                             C.c_void_p(out.data_ptr()), None)
        assert rc == twmc.OK
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert np.isfinite(got).all()
        err = np.abs(got - ref).max() / np.abs(ref).max()
        assert err < TOL, f"{ntraj} trajectories: relative error {err:.3e}"


def test_noalloc_more_blocks_than_trajectories(built_lib):
    """n_blocks > n_traj: block b holds trajectories [b T / B, (b + 1) T / B),
    so the blocks without a trajectory are exactly zero and the block sums
    equal the library path's (which clamps the block count to T)."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    lib = twmc.load()
    nx = ny = 32
    ntraj, nb = 5, 12
    field, ref = library_moments(nx, ny, ntraj, 31, nb)
    assert np.all(ref[ntraj:] == 0)  # the library path fills min(n_blocks, n_traj) blocks
    ref = ref[:ntraj]
    state = torch.from_numpy(field.astype(np.complex64)).cuda()
    out = torch.full((nb, nx * ny, 3), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rc = lib.twmc_kspace_moments_noalloc(C.c_void_p(state.data_ptr()), ntraj, nx, ny, nb,
                                         C.c_void_p(out.data_ptr()), None)
    assert rc == twmc.OK
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    cnt = np.diff((np.arange(nb + 1) * ntraj) // nb)
    assert np.all(got[cnt == 0] == 0.0)
    full = got[cnt > 0]
    assert full.shape == ref.shape
    err = np.abs(full - ref).max() / np.abs(ref).max()
    assert err < TOL, f"relative error {err:.3e}"


def test_noalloc_rejects_sizes_beyond_the_scratch(built_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    lib = twmc.load()
    state = torch.zeros(2, 4096, dtype=torch.complex64, device="cuda")
    out = torch.zeros(1, 4096, 3, dtype=torch.float64, device="cuda")
    # 1025 x 4096 > 4194304 floats of scratch (the buffers are never touched)
    rc = lib.twmc_kspace_moments_noalloc(C.c_void_p(state.data_ptr()), 1025, 64, 64, 1, C.c_void_p(out.data_ptr()),
                                         None)
    assert rc == twmc.ERR_INVALID
    rc = lib.twmc_kspace_moments_noalloc(C.c_void_p(state.data_ptr()), 2, 48, 64, 1, C.c_void_p(out.data_ptr()),
                                         None)
    assert rc == twmc.ERR_INVALID
    # sides beyond any compiled plan are rejected before any arithmetic on them
    for nx, ny in ((1 << 40, 1 << 40), (-1, 64), (8192, 1), (128, 64)):
        rc = lib.twmc_kspace_moments_noalloc(C.c_void_p(state.data_ptr()), 1, nx, ny, 1, C.c_void_p(out.data_ptr()),
                                             None)
        assert rc == twmc.ERR_INVALID, (nx, ny)
