"""Observables from FP64 moment blocks equal the direct estimators (CPU)."""
import numpy as np

from oracle import twmc_oracle as npo
from pincosimulator_gb300 import observables as ob


def blocks_from_frames(frames, nx, ny, nb):
    T, F, N = frames.shape
    out = np.zeros((F, nb, N, 3))
    edges = (np.arange(nb + 1) * T) // nb
    for b in range(nb):
        x = frames[edges[b]:edges[b + 1]]
        ab2 = np.abs(x) ** 2
        fk = np.fft.fft2(x.reshape(-1, F, nx, ny)).reshape(x.shape) / np.sqrt(N)
        out[:, b, :, 0] = ab2.sum(0)
        out[:, b, :, 1] = (ab2**2).sum(0)
        out[:, b, :, 2] = (np.abs(fk) ** 2).sum(0)
    return out


def test_observables_match_direct_estimators():
    rng = np.random.default_rng(0)
    T, F, nx, ny = 203, 3, 4, 4
    frames = (rng.normal(size=(T, F, nx * ny)) + 1j * rng.normal(size=(T, F, nx * ny))) * 0.8 + 0.3
    m = blocks_from_frames(frames, nx, ny, 16)
    o = ob.observables(m, T)
    ref = npo.ensemble_observables(frames, nx, ny)
    for k in ("n", "a2a2", "g2", "nk"):
        assert np.allclose(o[k], ref[k], rtol=1e-12, atol=1e-12), k
    # batch-means SE is close to the naive SE for independent samples
    naive = (np.abs(frames) ** 2).std(axis=0, ddof=1) / np.sqrt(T)
    assert np.all(np.abs(o["n_se"] / naive - 1) < 0.6)
    assert np.all(np.isfinite(o["g2_se"]))


def test_vacuum_has_zero_occupation():
    """Vacuum Wigner samples (variance 1/2 per quadrature... i.e. sigma 0.5 per
    quadrature as the reference's beta_init_sigma) give n = 0 within SE."""
    rng = np.random.default_rng(1)
    T, N = 20000, 8
    a = 0.5 * (rng.normal(size=(T, 1, N)) + 1j * rng.normal(size=(T, 1, N)))
    m = blocks_from_frames(a, 1, N, 32)
    o = ob.observables(m, T)
    assert np.all(np.abs(o["n"]) < 5 * o["n_se"])


def test_time_to_steady_state():
    t = np.arange(0, 50.5, 0.5)
    nbar = 2.0 * (1 - np.exp(-t / 3.0))
    se = np.full_like(t, 0.01)
    ts, ninf = ob.time_to_steady_state(t, nbar, se)
    assert abs(ninf - 2.0) < 1e-3
    # 2 e^{-t/3} <= 0.01 from t = 3 ln 200 = 15.9 on
    assert 15.5 <= ts <= 16.5


def test_compare_reports_bias_in_standard_errors():
    """compare(): two samples of one distribution give z ~ N(0, 1); a bias of
    five standard errors planted in one ensemble's fields shows up as |z| of
    about five in n and in the site-averaged density."""
    rng = np.random.default_rng(4)
    T, F, N = 1024, 6, 32
    a = 0.7 * (rng.normal(size=(T, F, N)) + 1j * rng.normal(size=(T, F, N)))
    b = 0.7 * (rng.normal(size=(T, F, N)) + 1j * rng.normal(size=(T, F, N)))
    oa, ob_ = ob.frame_observables(a), ob.frame_observables(b)
    c = ob.compare(oa, ob_, keys=("n", "g2"))
    assert 0.5 < c["n"]["mean_z2"] < 1.6 and c["n"]["max_abs_z"] < 4.5
    assert 0.5 < c["g2"]["mean_z2"] < 1.6
    se = float(np.median(oa["n_se"]))
    biased = ob.frame_observables(np.sqrt(1.0 + 5.0 * se / (np.abs(b) ** 2).mean()) * b)
    c2 = ob.compare(oa, biased, keys=("n",))
    assert c2["n"]["mean_z2"] > 10.0
    assert c2["n_site_avg"]["max_abs_z"] > 20.0
