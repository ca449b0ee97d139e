"""Learned warm start on the GPU: the BF16 tensor-core MLP (forward,
backward, Adam) against the FP64 oracle with BF16 emulation, the row <-> field
transforms, the batch's field-moment / initial-field / block-mean entry
points, and a reduced warm-start sweep that must beat the plain vacuum start
on time to steady state.

Tolerances: the device accumulates in FP32 where the oracle uses FP64, and a
value near a BF16 rounding boundary can round the other way, so outputs and
gradients are compared norm-wise at 2e-3 relative (forward) and 1e-2
(gradients), far below the 2^-8 relative step of one BF16 rounding."""
import numpy as np
import pytest

from oracle import mlp_oracle as mo
from pincosimulator_gb300 import twmc

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

SMALL = [5, 64, 48, 37]
FULL = [5, 256, 256, 256, 2049]


def nrel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-30))


def setup_net(widths, batch, seed):
    rng = np.random.default_rng(seed)
    p = mo.init_params(widths, seed=seed)
    _, n = mo.offsets(widths)
    offs, _ = mo.offsets(widths)
    for (wo, bo), m in zip(offs, widths[1:]):
        p[bo:bo + m] = 0.1 * rng.normal(size=m)
    net = twmc.MLP(widths, max_batch=batch, seed=seed)
    net.set_params(p)
    x = rng.uniform(-1, 1, size=(batch, widths[0])).astype(np.float32)
    t = rng.normal(size=(batch, widths[-1])).astype(np.float32)
    return net, p, x, t


@pytest.mark.parametrize("widths,batch", [(SMALL, 70), (FULL, 128)])
def test_forward_matches_oracle(built_lib, widths, batch):
    net, p, x, _ = setup_net(widths, batch, 1)
    xd = torch.as_tensor(x).cuda()
    y = torch.zeros(batch, widths[-1], dtype=torch.float32, device="cuda")
    net.forward(xd.data_ptr(), batch, y.data_ptr())
    torch.cuda.synchronize()
    ref, _ = mo.forward(p, widths, x)
    assert nrel(y.cpu().numpy(), ref) < 2e-3
    assert np.array_equal(net.get_params(), p)   # forward leaves parameters alone


@pytest.mark.parametrize("widths,batch", [(SMALL, 70), (FULL, 128)])
def test_backward_matches_oracle(built_lib, widths, batch):
    net, p, x, t = setup_net(widths, batch, 2)
    w = np.random.default_rng(3).uniform(0.5, 1.5, size=widths[-1]).astype(np.float32)
    xd, td, wd = (torch.as_tensor(a).cuda() for a in (x, t, w))
    loss = net.backward(xd.data_ptr(), td.data_ptr(), batch, wd.data_ptr(), want_loss=True)
    g = net.get_grads()
    lref, gref, _ = mo.backward(p, widths, x, t, w)
    assert abs(loss - lref) < 2e-3 * lref
    offs, _ = mo.offsets(widths)
    for l, ((wo, bo), k, m) in enumerate(zip(offs, widths[:-1], widths[1:])):
        assert nrel(g[wo:wo + m * k], gref[wo:wo + m * k]) < 1e-2, f"dW layer {l}"
        assert nrel(g[bo:bo + m], gref[bo:bo + m]) < 1e-2, f"db layer {l}"


def test_adam_matches_oracle(built_lib):
    widths = SMALL
    net, p, x, t = setup_net(widths, 40, 4)
    xd, td = torch.as_tensor(x).cuda(), torch.as_tensor(t).cuda()
    pm = p.astype(np.float64)
    m = np.zeros_like(pm)
    v = np.zeros_like(pm)
    for step in range(1, 4):
        net.backward(xd.data_ptr(), td.data_ptr(), 40)
        g = net.get_grads().astype(np.float64)   # the device's own gradients, so only Adam is compared
        net.adam(1e-3, 0.9, 0.999, 1e-8)
        pm, m, v = mo.adam(pm, g, m, v, step, 1e-3, 0.9, 0.999, 1e-8)
        got = net.get_params()
        assert np.max(np.abs(got - pm)) < 1e-6 + 1e-5 * np.max(np.abs(pm))


def test_training_reduces_loss_like_oracle(built_lib):
    """A few Adam steps on a smooth regression target: device and oracle
    losses agree step by step and fall."""
    widths = [5, 32, 32, 9]
    rng = np.random.default_rng(5)
    x = rng.uniform(-1, 1, size=(64, 5)).astype(np.float32)
    t = np.stack([np.sin(2 * x[:, 0]) * x[:, 1] + 0.3 * k * x[:, 2] ** 2 for k in range(9)], 1).astype(np.float32)
    p = mo.init_params(widths, seed=6)
    net = twmc.MLP(widths, 64, 1)
    net.set_params(p)
    xd, td = torch.as_tensor(x).cuda(), torch.as_tensor(t).cuda()
    pm, m, v = p.astype(np.float64), np.zeros(p.size), np.zeros(p.size)
    dl, ol = [], []
    for step in range(1, 41):
        dl.append(net.backward(xd.data_ptr(), td.data_ptr(), 64, want_loss=True))
        net.adam(5e-3)
        lo, g, _ = mo.backward(pm, widths, x, t)
        ol.append(lo)
        pm, m, v = mo.adam(pm, g, m, v, step, 5e-3)
    assert dl[-1] < 0.5 * dl[0]
    assert np.allclose(dl, ol, rtol=2e-2)


def test_targets_and_fields_kernels_match_oracle(built_lib):
    rng = np.random.default_rng(7)
    nx, ny, P, frames = 32, 32, 5, 3
    N = nx * ny
    mean = rng.normal(size=(P, N)) + 1j * rng.normal(size=(P, N))
    abs2 = np.abs(mean) ** 2 + rng.uniform(0.5, 2, size=(P, N))
    md = torch.as_tensor(np.stack([mean.real, mean.imag], -1).reshape(-1) * frames).cuda()
    ad = torch.as_tensor(abs2.reshape(-1) * frames).cuda()
    rows = torch.zeros(P, 2 * N + 1, dtype=torch.float32, device="cuda")
    twmc.mlp_targets(md.data_ptr(), ad.data_ptr(), P, nx, ny, frames, rows.data_ptr(), 2 * N + 1)
    torch.cuda.synchronize()
    ref = mo.targets(mean, abs2, nx, ny)
    assert np.max(np.abs(rows.cpu().numpy() - ref)) < 1e-5 * np.max(np.abs(ref))
    # squash + standardise + weights, then fields back, against the oracle
    sq = 0.5
    tr = rows.clone()
    mu = torch.zeros(2 * N + 1, dtype=torch.float32, device="cuda")
    sd = torch.zeros_like(mu)
    wt = torch.zeros_like(mu)
    twmc.mlp_standardize(tr.data_ptr(), P, 2 * N + 1, 0.05, mu.data_ptr(), sd.data_ptr(), squash=sq,
                         weights_ptr=wt.data_ptr())
    torch.cuda.synchronize()
    rt, rmu, rsd, rw = mo.standardize(rows.cpu().numpy(), squash=sq, floor_frac=0.05)
    assert np.max(np.abs(tr.cpu().numpy() - rt)) < 1e-4 * max(1.0, np.max(np.abs(rt)))
    assert np.allclose(sd.cpu().numpy(), rsd, rtol=1e-5) and np.allclose(wt.cpu().numpy(), rw, rtol=1e-4)
    bi = torch.zeros(P, N, 2, dtype=torch.float64, device="cuda")
    bs = torch.zeros(P, N, 2, dtype=torch.float64, device="cuda")
    twmc.mlp_fields(tr.data_ptr(), 2 * N + 1, P, mu.data_ptr(), sd.data_ptr(), nx, ny, bi.data_ptr(), bs.data_ptr(),
                    squash=sq, max_incoherent=0.3)
    torch.cuda.synchronize()
    fb, fs = mo.fields(tr.cpu().numpy().astype(np.float64), nx, ny, mu.cpu().numpy(), sd.cpu().numpy(), squash=sq,
                       max_incoherent=0.3)
    b = bi.cpu().numpy()
    assert np.max(np.abs(b[..., 0] + 1j * b[..., 1] - fb)) < 1e-9 * np.max(np.abs(fb)) + 1e-12
    s = bs.cpu().numpy()
    assert np.max(np.abs(s[..., 0] - fs.real)) < 1e-9 and np.all(s[..., 1] == 0)
    assert np.max(s[..., 0]) <= np.sqrt((0.3 + 0.5) * 0.5) + 1e-12
    # the round trip returns the mean field to FP32 accuracy
    assert np.max(np.abs(b[..., 0] + 1j * b[..., 1] - mean)) < 1e-4 * np.max(np.abs(mean))


def test_hbatch_field_moments_init_and_block_means(built_lib):
    pts = [dict(nx=32, ny=32, dt=0.002, omega=-0.5, U=0.2, F=1.0, n_traj=40, seed0=3, id0=1),
           dict(nx=1, ny=64, dt=0.002, omega=0.5, U=0.1, F=2.0, n_traj=33, seed0=4, id0=100)]
    hb = twmc.HBatch(pts, 20)
    # per-site initial field with zero spread: every trajectory starts at it
    rng = np.random.default_rng(8)
    N0 = 1024
    b0 = rng.normal(size=(N0, 2))
    bi = torch.as_tensor(b0).cuda()
    bs = torch.zeros(N0, 2, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    hb.set_init(0, bi.data_ptr(), bs.data_ptr())
    st = hb.state(0)
    assert np.array_equal(st, np.broadcast_to((b0[:, 0] + 1j * b0[:, 1]).astype(np.complex64), st.shape))
    hb.run(2)
    hb.sync()
    T = hb.total_sites
    assert T == 1024 + 64
    mean = torch.zeros(T, 2, dtype=torch.float64, device="cuda")
    abs2 = torch.zeros(T, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    hb.field_moments(mean.data_ptr(), abs2.data_ptr())
    hb.sync()
    m, a2 = mean.cpu().numpy(), abs2.cpu().numpy()
    o = 0
    for i, p in enumerate(pts):
        s = hb.state(i)
        n = s.shape[1]
        assert np.allclose(m[o:o + n, 0] + 1j * m[o:o + n, 1], s.mean(0), rtol=0, atol=1e-12)
        assert np.allclose(a2[o:o + n], (np.abs(s) ** 2).mean(0), rtol=1e-12)
        o += n
    bm = hb.block_means()
    for i in range(len(pts)):
        assert np.allclose(bm[i], hb.moments(i).mean(axis=1), rtol=1e-12)
    with pytest.raises(twmc.TWMCError):
        hb.set_init(0, bi.data_ptr(), bs.data_ptr())   # only before the first run
    hb.close()


def test_warm_start_cuts_time_to_steady_state(built_lib):
    """Reduced learned-warm-start sweep on 32 x 32 (512 training points of 128
    trajectories to t = 16; 24 held-out points of 256 trajectories to t = 12):
    the median time to steady state must drop at least 2.5x against the plain
    vacuum start, no warm run may diverge, and warm and plain steady
    densities must agree within 3 combined standard errors for >= 80% of the
    points, and the rerun rule replaces every point whose n or g2 is off by
    more than one combined standard error by its plain result."""
    from pincosimulator_gb300 import warmstart as wsm

    train = wsm.sample_points(512, seed=11)
    rows, _ = wsm.steady_rows(train, 32, 32, n_traj=128, t_end=16.0)
    ws = wsm.WarmStart(32, 32, max_batch=64, seed=3)
    rep = ws.fit(wsm.features(train), rows, epochs=800, batch=64)
    assert rep.losses[-1][1] < 0.1 * rep.losses[0][1]
    test = wsm.sample_points(24, seed=12)
    res = wsm.warm_sweep(ws, test, n_traj=256, t_end=12.0)
    tw, tp = np.median(res.warm.ttss), np.median(res.plain.ttss)
    print(f"median time to steady state: warm {tw:.2f}, plain {tp:.2f}; reruns {int(res.rerun.sum())}/24")
    assert np.all(np.isfinite(res.warm.n_inf))
    assert tw * 2.5 <= tp
    se = np.sqrt(res.warm.n_inf_se ** 2 + res.plain.n_inf_se ** 2)
    assert np.mean(np.abs(res.warm.n_inf - res.plain.n_inf) <= 3 * se) >= 0.8
    assert np.array_equal(res.n_final[res.rerun], res.plain.n_inf[res.rerun])
    # the rule judges n and g2: every kept warm point agrees with its plain run in both
    keep = ~res.rerun
    se_g = np.sqrt(res.warm.g2_inf_se ** 2 + res.plain.g2_inf_se ** 2)
    assert np.all(np.abs(res.warm.n_inf - res.plain.n_inf)[keep] <= se[keep])
    assert np.all(np.abs(res.warm.g2_inf - res.plain.g2_inf)[keep] <= se_g[keep])
    assert np.array_equal(res.g2_final[res.rerun], res.plain.g2_inf[res.rerun])
    assert np.array_equal(res.rerun, wsm.rerun_mask(res.warm, res.plain))
