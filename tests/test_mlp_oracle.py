"""CPU checks of the warm-start network's oracle: BF16 rounding, analytic
gradients against finite differences, Adam, and the row <-> field transforms."""
import numpy as np
import pytest

from oracle import mlp_oracle as mo


def test_bf16_rounding_known_values():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -9, -2.5, 0.0, 3.0e38, 1e-40],
                 dtype=np.float32)
    r = mo.bf16(x)
    assert r[0] == 1.0
    assert r[1] == 1.0                     # tie -> even mantissa
    assert r[2] == 1.0 + 4 * 2 ** -8       # tie -> even (rounds up)
    assert r[3] == 1.0                     # below half an ulp
    assert r[4] == -2.5
    assert r[5] == 0.0
    assert np.isfinite(r[6])
    # idempotent and within half an ulp
    y = np.random.default_rng(0).normal(size=1000).astype(np.float32)
    b = mo.bf16(y)
    assert np.all(mo.bf16(b.astype(np.float32)) == b)
    assert np.max(np.abs(b - y) / np.abs(y)) <= 2 ** -8  # half an ulp of an 8-bit significand


def test_gelu_grad_matches_difference():
    z = np.linspace(-5, 5, 101)
    h = 1e-6
    fd = (mo.gelu(z + h) - mo.gelu(z - h)) / (2 * h)
    assert np.allclose(mo.gelu_grad(z), fd, atol=1e-8)


@pytest.mark.parametrize("widths", [[5, 7, 6, 4], [5, 16, 16, 16, 9]])
def test_gradients_match_finite_differences(widths):
    rng = np.random.default_rng(1)
    p = mo.init_params(widths, seed=2).astype(np.float64)
    _, n = mo.offsets(widths)
    p[:] += 0.05 * rng.normal(size=n)          # non-zero biases
    x = rng.normal(size=(11, widths[0]))
    t = rng.normal(size=(11, widths[-1]))
    w = rng.uniform(0.5, 2.0, size=widths[-1])
    loss, g, _ = mo.backward(p, widths, x, t, w, emulate_bf16=False)
    h = 1e-6
    idx = rng.choice(n, size=min(n, 60), replace=False)
    for i in idx:
        q = p.copy()
        q[i] += h
        lp = mo.backward(q, widths, x, t, w, emulate_bf16=False)[0]
        q[i] -= 2 * h
        lm = mo.backward(q, widths, x, t, w, emulate_bf16=False)[0]
        assert abs((lp - lm) / (2 * h) - g[i]) <= 1e-6 * max(1.0, abs(g[i])), i


def test_bf16_emulation_is_close_to_exact():
    widths = [5, 32, 32, 20]
    rng = np.random.default_rng(3)
    p = mo.init_params(widths, seed=4)
    x = rng.normal(size=(16, 5))
    t = rng.normal(size=(16, 20))
    l1, g1, _ = mo.backward(p, widths, x, t)
    l2, g2, _ = mo.backward(p, widths, x, t, emulate_bf16=False)
    assert abs(l1 - l2) < 2e-2 * l2
    assert np.linalg.norm(g1 - g2) < 3e-2 * np.linalg.norm(g2)


def test_adam_first_step_is_signed_lr():
    g = np.array([1e-3, -2.0, 5.0, 0.0])
    p, m, v = mo.adam(np.zeros(4), g, np.zeros(4), np.zeros(4), step=1, lr=0.01, eps=1e-12)
    assert np.allclose(p[:3], -0.01 * np.sign(g[:3]), rtol=1e-6)
    assert p[3] == 0.0


def test_rows_and_fields_round_trip():
    rng = np.random.default_rng(5)
    nx, ny, P = 4, 8, 3
    N = nx * ny
    mean = rng.normal(size=(P, N)) + 1j * rng.normal(size=(P, N))
    abs2 = np.abs(mean) ** 2 + rng.uniform(0.5, 2.0, size=(P, N))
    rows = mo.targets(mean, abs2, nx, ny)
    # Parseval: sum |a_k|^2 = sum |<a>|^2 (unitary transform)
    ak = rows[:, 0:2 * N:2] + 1j * rows[:, 1:2 * N:2]
    assert np.allclose((np.abs(ak) ** 2).sum(1), (np.abs(mean) ** 2).sum(1))
    # explicit DFT at one k
    kx, ky = 1, 3
    ph = np.exp(-2j * np.pi * (kx * np.arange(nx)[:, None] / nx + ky * np.arange(ny)[None, :] / ny)).reshape(-1)
    assert np.allclose(ak[:, kx * ny + ky], (mean * ph).sum(1) / np.sqrt(N))
    b, sg = mo.fields(rows, nx, ny)
    assert np.allclose(b, mean)
    dens = abs2.mean(1) - 0.5
    assert np.allclose(sg.real ** 2 * 2 - 0.5, np.maximum(dens[:, None] - np.abs(mean) ** 2, 0))
    # standardised rows de-standardise exactly
    mu, sd = rows.mean(0), rows.std(0) + 1.0
    b2, _ = mo.fields((rows - mu) / sd, nx, ny, mu, sd)
    assert np.allclose(b2, mean)
