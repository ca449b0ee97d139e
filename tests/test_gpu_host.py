"""End to end through the C++ host layer on the GPU: twmc_sim reads an .ini,
runs the TWMCCuda solver plugin, writes the Pinco archive; the archive is
read back by an independent reader and checked against the same run through
the C ABI; a second invocation resumes every trajectory (continuations)."""
import os
import subprocess

import numpy as np
import pytest

from pincosimulator_gb300 import twmc

import pinco_reader as pr

pytestmark = pytest.mark.gpu


def mt19937(seed, n):
    """std::mt19937(seed) outputs (Matsumoto & Nishimura; seeding by the standard's recurrence)."""
    mt = [0] * 624
    mt[0] = seed & 0xFFFFFFFF
    for i in range(1, 624):
        mt[i] = (1812433253 * (mt[i - 1] ^ (mt[i - 1] >> 30)) + i) & 0xFFFFFFFF
    idx = 624
    out = []
    for _ in range(n):
        if idx >= 624:
            for i in range(624):
                y = (mt[i] & 0x80000000) | (mt[(i + 1) % 624] & 0x7FFFFFFF)
                mt[i] = mt[(i + 397) % 624] ^ (y >> 1) ^ (0x9908B0DF if y & 1 else 0)
            idx = 0
        y = mt[idx]
        idx += 1
        y ^= y >> 11
        y ^= (y << 7) & 0x9D2C5680
        y ^= (y << 15) & 0xEFC60000
        y ^= y >> 18
        out.append(y)
    return out


INI = """
Manager = "TWMC"
nx = 8
ny = 8
PBC = true
J = 1
U = 0.2
gamma = 1
omega = -0.5
"omega.Noise_Type" = "Gaussian"
"omega.Noise_Val_0" = 0.2
F = 1.5
beta_init = 0
beta_init_sigma = 0.5
timestep = 0.01
t_start = 0
t_end = 2
frames_period = 0.5
n_traj = 6
SEED = 77
"""


@pytest.fixture(scope="module")
def sim(built_lib):
    from pincosimulator_gb300 import build_ext

    return build_ext.build_host()


def run_sim(sim, ini, out, *kv):
    r = subprocess.run([sim, "-i", str(ini), "-o", str(out), *map(str, kv)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return r


def test_sim_archive_matches_c_abi(sim, tmp_path):
    ini = tmp_path / "run.ini"
    ini.write_text(INI)
    out = tmp_path / "out"
    run_sim(sim, ini, out)
    data = out / "data"
    reg = pr.read_register(data)
    assert reg["names"] == ["Omega_Realization", "traj"]
    assert reg["dims"] == [[8, 8], [8, 8]] and reg["formats"] == [22, 22]
    assert [e["id"] for e in reg["entries"]] == [1, 2, 3, 4, 5, 6]
    assert all(e["chunk"] == 1 and e["cont"] == 0 for e in reg["entries"])
    times = pr.read_times(data / "_t.dat")
    assert np.allclose(times, [0, 0.5, 1.0, 1.5, 2.0])
    # the same run through the C ABI with the manager's seeds
    seeds = mt19937(77, 6)
    s = twmc.System(nx=8, ny=8, J=1.0, gamma=1.0, dt=0.01, frame_steps=50,
                    omega=twmc.Noisy(-0.5, twmc.DISORDER_GAUSSIAN, 0.2), U=0.2, F=1.5, beta_init_sigma=0.5)
    tasks = s.make_tasks(6, t_start=0.0, t_end=2.0, seeds=seeds, id0=1)
    res = s.run(tasks, frames=True, realizations=True)
    s.close()
    for k in range(6):
        fr, real, ents = pr.read_trajectory(data, k + 1)
        assert fr.shape == (5, 64)
        assert np.array_equal(fr, res["frames"][k])
        assert np.array_equal(real["Omega_Realization"], res["omega_realization"][k])
        assert ents[0]["t_start"] == 0.0 and ents[0]["t_end"] == res["t_final"][k]


def test_sim_split_step_integrator(sim, tmp_path):
    """The ini key integrator = "split" selects the exponential split step:
    the archive equals the same run through the C ABI with
    TWMC_INTEGRATOR_SPLIT and differs from the default (Euler) run."""
    ini = tmp_path / "run.ini"
    # 16 x 16: the split step needs a lattice the FFT kernel has a plan for
    ini.write_text(INI.replace("nx = 8", "nx = 16").replace("ny = 8", "ny = 16") + 'integrator = "split"\n')
    out = tmp_path / "out"
    run_sim(sim, ini, out)
    seeds = mt19937(77, 6)
    res = {}
    for integ in (twmc.INTEGRATOR_SPLIT, twmc.INTEGRATOR_EULER):
        s = twmc.System(nx=16, ny=16, J=1.0, gamma=1.0, dt=0.01, frame_steps=50,
                        omega=twmc.Noisy(-0.5, twmc.DISORDER_GAUSSIAN, 0.2), U=0.2, F=1.5, beta_init_sigma=0.5,
                        integrator=integ)
        res[integ] = s.run(s.make_tasks(6, t_start=0.0, t_end=2.0, seeds=seeds, id0=1), frames=True)
        s.close()
    for k in range(6):
        fr, _, _ = pr.read_trajectory(out / "data", k + 1)
        assert np.array_equal(fr, res[twmc.INTEGRATOR_SPLIT]["frames"][k])
        assert not np.allclose(fr[-1], res[twmc.INTEGRATOR_EULER]["frames"][k][-1], rtol=1e-6, atol=0)


def test_sim_resume_appends_continuations(sim, tmp_path):
    ini = tmp_path / "run.ini"
    ini.write_text(INI)
    out = tmp_path / "out"
    run_sim(sim, ini, out)
    reg1 = pr.read_register(out / "data")
    first = {k: pr.read_trajectory(out / "data", k)[0] for k in range(1, 7)}
    run_sim(sim, ini, out, "t_end", "3")
    reg = pr.read_register(out / "data")
    ents = reg["entries"]
    assert len(ents) == 12 and [e["id"] for e in ents[6:]] == [1, 2, 3, 4, 5, 6]
    assert all(e["chunk"] == 2 for e in ents[6:])
    for k in range(6):
        old, new = ents[k], ents[6 + k]
        assert old["cont"] == new["pos"] and new["cont"] == 0
        assert new["t_start"] == old["t_end"]
        fr, real, _ = pr.read_trajectory(out / "data", k + 1)
        # 5 frames of the first run + 2 frames of the continuation (no initial state)
        assert fr.shape == (7, 64)
        assert np.array_equal(fr[:5], first[k + 1])
        assert np.isfinite(fr).all()
    assert len(reg1["entries"]) == 6


def test_lieb_ini_runs(sim, tmp_path):
    src = os.path.join(os.path.dirname(__file__), "golden", "sampledata")
    for name in ("_E.dat", "_F.dat", "_U.dat"):
        (tmp_path / name).write_bytes(open(os.path.join(src, name), "rb").read())
    text = open(os.path.join(src, "test-lieb.ini")).read()
    ini = tmp_path / "lieb.ini"
    ini.write_text(text)
    out = tmp_path / "out"
    run_sim(sim, ini, out, "t_end", "1", "n_traj", "3", "timestep", "0.005", "frames_freq", "2")
    reg = pr.read_register(out / "data")
    assert reg["names"] == ["Omega_Realization", "traj"] and reg["dims"][1] == [1, 24, 3]
    fr, real, _ = pr.read_trajectory(out / "data", 1)
    assert fr.shape == (3, 72) and np.isfinite(fr).all()


def test_time_dependent_drive_writes_work_and_area(sim, tmp_path):
    """A periodic lattice with F(t) runs in thermo mode (the reference's
    manager picks its Thermo solver there): the archive gains the float64
    datasets work and area after traj, equal to the same run through the C
    ABI (the time table read at float precision, as the reader does)."""
    times = [0.0, 0.5, 1.0]
    amp = [0.0, 2.0, 2.0]
    lines = []
    for t, a in zip(times, amp):
        lines.append(f"{t}")
        for r in range(4):
            lines.append("  ".join(f"{a * (1 + 0.1 * (r * 4 + c)):.6f}" for c in range(4)))
        lines.append("")
    (tmp_path / "F_t.dat").write_text("\n".join(lines) + "\n")
    ini = tmp_path / "thermo.ini"
    ini.write_text("""
Manager = "TWMC"
nx = 4
ny = 4
PBC = true
J = 1
U = 0.2
gamma = 1
omega = -0.5
F_t = "F_t.dat"
beta_init = 0
beta_init_sigma = 0.5
timestep = 0.01
t_start = 0
t_end = 1.5
frames_period = 0.5
n_traj = 3
SEED = 9
""")
    out = tmp_path / "out"
    run_sim(sim, ini, out)
    data = out / "data"
    reg = pr.read_register(data)
    assert reg["names"] == ["traj", "work", "area"] and reg["formats"] == [22, 11, 11]
    seeds = mt19937(9, 3)
    vals = np.array([[np.float32(a * (1 + 0.1 * k)) for k in range(16)] for a in amp], dtype=np.float64)
    s = twmc.System(nx=4, ny=4, J=1.0, gamma=1.0, dt=0.01, frame_steps=50, omega=-0.5, U=0.2, F=0.0,
                    beta_init_sigma=0.5, F_t=(np.array(times), vals.astype(complex)), thermo=True)
    tasks = s.make_tasks(3, t_start=0.0, t_end=1.5, seeds=seeds, id0=1)
    res = s.run(tasks, frames=True)
    s.close()
    for k in range(3):
        fr, real, _ = pr.read_trajectory(data, k + 1)
        assert fr.shape == (4, 16) and np.array_equal(fr, res["frames"][k])
        assert real["work"].shape == (4, 16) and np.array_equal(real["work"], res["work"][k])
        assert np.array_equal(real["area"], res["area"][k])
        assert np.all(real["work"][0] == 0) and np.abs(real["work"][1]).max() > 0
