"""Pins the oracle's Philox4x32-10 (CPU, no GPU)."""
import ctypes
import os

import numpy as np
import pytest

from oracle import twmc_oracle as npo


def test_oracle_matches_numpy_philox(oracle):
    rng = np.random.default_rng(1)
    ctr = rng.integers(0, 2**32, size=(64, 4), dtype=np.uint64).astype(np.uint32)
    key = np.array([0xDEADBEEF, 0x12345678], dtype=np.uint32)
    a = oracle.philox(ctr, key)
    b = npo.philox4x32_10(ctr, np.broadcast_to(key, (64, 2)))
    assert np.array_equal(a, b)


def _curand():
    for path in ("/usr/local/cuda/lib64/libcurand.so", "libcurand.so", "libcurand.so.10"):
        try:
            return ctypes.CDLL(path)
        except OSError:
            continue
    return None


@pytest.mark.parametrize("seed", [0, 0x123456789ABCDEF0, 0xFFFFFFFFFFFFFFFF, 42])
def test_oracle_matches_curand_host_philox(oracle, seed):
    """cuRAND's host Philox4x32-10 generator: block j = Philox(ctr=(0,0,j,0), key=seed)."""
    cr = _curand()
    if cr is None:
        pytest.skip("libcurand not available")
    gen = ctypes.c_void_p()
    if cr.curandCreateGeneratorHost(ctypes.byref(gen), 161) != 0:  # CURAND_RNG_PSEUDO_PHILOX4_32_10
        pytest.skip("cuRAND host generator unavailable")
    try:
        assert cr.curandSetPseudoRandomGeneratorSeed(gen, ctypes.c_ulonglong(seed)) == 0
        out = np.zeros(64, dtype=np.uint32)
        assert cr.curandGenerate(gen, out.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(64)) == 0
    finally:
        cr.curandDestroyGenerator(gen)
    key = [seed & 0xFFFFFFFF, seed >> 32]
    ctr = np.array([[0, 0, j, 0] for j in range(16)], dtype=np.uint32)
    ref = oracle.philox(ctr, key).reshape(-1)
    assert np.array_equal(ref, out)


def test_normals_statistics(oracle):
    z = np.concatenate([oracle.site_normals(7, 3, s, 0, 4096) for s in range(8)])
    for part in (z.real, z.imag):
        assert abs(part.mean()) < 0.03
        assert abs(part.var() - 1.0) < 0.03
    assert abs(np.mean(z.real * z.imag)) < 0.03


def test_site_pairing_matches_numpy(oracle):
    for n in (1, 7, 64, 768):
        a = oracle.site_normals(11, 5, 3, 0, n)
        b = npo.site_normals(11, 5, 3, 0, n)
        assert np.allclose(a, b, rtol=0, atol=1e-13)
        a32 = oracle.site_normals(11, 5, 3, 0, n, f32=True)
        b32 = npo.site_normals(11, 5, 3, 0, n, f32_flavour=True)
        assert np.allclose(a32, b32, rtol=0, atol=1e-6)


def test_wiener_stream_key_layout(oracle):
    """The Wiener stream (stream 0) uses the fixed key with the trajectory in
    the counter, (site pair, step, id, seed); the other streams the key
    (seed, id) with counter (site pair, 0, stream, 0)."""
    seed, tid, step, n = 123456789, 42, 17, 10
    z = oracle.site_normals(seed, tid, step, 0, n)
    ctr = np.array([[p, step, tid, seed] for p in range(5)], dtype=np.uint32)
    w = npo.philox4x32_10(ctr, np.broadcast_to(np.array(npo.WIENER_KEY, np.uint32), (5, 2)))
    a, b = w[0, 0].astype(np.float64), w[0, 1].astype(np.float64)
    u1, u2 = (a + 0.5) * 2.0 ** -32, (b + 0.5) * 2.0 ** -32
    z0 = np.sqrt(-2 * np.log(u1)) * complex(np.cos(2 * np.pi * u2 - np.pi), np.sin(2 * np.pi * u2 - np.pi))
    assert abs(z[0] - z0) < 1e-12
    # an init-stream draw is keyed by (seed, id) instead
    zi = oracle.site_normals(seed, tid, 0, 1, n)
    w1 = npo.philox4x32_10(np.array([[0, 0, 1, 0]], np.uint32), np.array([[seed, tid]], np.uint32))
    u1, u2 = (w1[0, 0] + 0.5) * 2.0 ** -32, (w1[0, 1] + 0.5) * 2.0 ** -32
    assert abs(zi[0] - np.sqrt(-2 * np.log(u1)) * np.exp(1j * (2 * np.pi * u2 - np.pi))) < 1e-12


def test_initial_field_flavours(oracle):
    """Initial fields beta_init + beta_init_sigma * xi from the init stream in
    the FP64 and the FP32 Box-Muller flavour agree with the numpy restatement."""
    n = 37
    rng = np.random.default_rng(2)
    bi = rng.normal(size=n) + 1j * rng.normal(size=n)
    bs = 0.5 + 0.1 * rng.random(size=n)
    for f32, tol in ((False, 1e-13), (True, 1e-6)):
        got = oracle.initial_field(n, bi, bs, 99, 7, f32=f32)
        ref = bi + bs * npo.site_normals(99, 7, 0, 1, n, f32_flavour=f32)
        assert np.allclose(got, ref, rtol=0, atol=tol), f32
