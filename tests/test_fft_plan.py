"""The register FFT plans executed in numpy (CPU): exact math, layout rules, bank model."""
import numpy as np
import pytest

from pincosimulator_gb300 import fft_plan as fp


@pytest.mark.parametrize("shape", fp.SUPPORTED_SHAPES + [(7, 7), (1, 3), (2, 5)])
def test_plan_matches_numpy_fft(shape):
    bx, by = shape
    p = fp.make_plan(bx, by, 4)
    N = 1 << p.nbits
    rng = np.random.default_rng(N)
    x = rng.normal(size=N) + 1j * rng.normal(size=N)
    y = fp.run_forward(p, x)
    kx, ky = fp.freq_of_position(p)
    ref = np.fft.fft2(x.reshape(1 << bx, 1 << by))
    assert np.abs(y - ref[kx, ky]).max() < 1e-10 * np.abs(ref).max()
    assert np.abs(fp.run_inverse(p, y) / N - x).max() < 1e-12


@pytest.mark.parametrize("shape", fp.SUPPORTED_SHAPES)
def test_plan_layout_rules(shape):
    p = fp.make_plan(*shape, 4)
    for ps in p.passes:
        assert sorted(ps.reg + ps.thr) == list(range(p.nbits))
        active = set()
        for st in ps.stages:
            active |= {p.lo[st.dim] + st.t + k for k in range(st.rb)}
        assert active <= set(ps.reg)
    # the top site bit is a register bit of the first pass (Philox site pairing)
    assert p.nbits - 1 in p.passes[0].reg


def test_headline_shape_bank_conflict_free():
    p = fp.make_plan(6, 6, 4)
    for k in range(len(p.passes)):
        assert fp.exchange_wavefronts(p, k, 1, 8, True) == 2.0
