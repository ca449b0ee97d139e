"""The C++ host layer's input reading (CPU): `twmc_sim --describe` on the
reference's SampleData inputs and on synthetic inputs exercising every
matrix-resolution rule of Settings::GetMatrix (Settings.cpp:357-497)."""
import json
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
SAMPLE = os.path.join(HERE, "golden", "sampledata")


@pytest.fixture(scope="module")
def sim(built_lib):
    from pincosimulator_gb300 import build_ext

    return build_ext.build_host()


def describe(sim, ini, *overrides):
    r = subprocess.run([sim, "--describe", "-i", str(ini), *map(str, overrides)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return json.loads(r.stdout)


def cvec(m):
    return np.array([complex(a, b) for a, b in m])


def test_sample_sim_ini(sim):
    d = describe(sim, os.path.join(SAMPLE, "test-sim.ini"))
    assert (d["nx"], d["ny"], d["dimension"], d["PBC"]) == (4, 4, 2, True)
    assert d["J"] == 0.45 and d["gamma"] == 1.0 and d["n_traj"] == 100
    assert np.allclose(cvec(d["U"]["base"]), 0.1) and np.allclose(cvec(d["omega"]["base"]), 1.0)
    # F = 3 with the quoted back-support keys "F_Noise_Type" / "F_Noise_Val_0"
    assert np.allclose(cvec(d["F"]["base"]), 3.0)
    assert d["F"]["noise"] == 2 and np.allclose(cvec(d["F"]["amp"]), 1.0)
    assert np.allclose(cvec(d["beta_init_sigma"]["base"]), 0.5)
    # frames_freq = 1, dt = 0.01: 100 steps per frame, 20 frames + initial
    assert d["frame_steps"] == 100 and d["nFramesTot"] == 20 and d["t_end"] == 20.0
    assert len(d["stored_times"]) == 21 and abs(d["stored_times"][-1] - 20.0) < 1e-9


def test_sample_lieb_ini(sim):
    d = describe(sim, os.path.join(SAMPLE, "test-lieb.ini"))
    # 1-D swap: nx = 24, ny = 1 -> nx = 1, ny = 24; 3 sites per cell
    assert (d["nx"], d["ny"], d["cellSz"], d["lattice"], d["PBC"]) == (1, 24, 3, "lieb", False)
    assert d["J_AB"] == 4 and d["J_BC"] == 4 and d["detuning"] == 2
    E = np.loadtxt(os.path.join(SAMPLE, "_E.dat"))
    assert np.allclose(cvec(d["E"]["base"]), E)  # a 1 x 72 matrix: column-major == memory order
    assert d["E"]["noise"] == 2 and np.allclose(cvec(d["E"]["amp"]), 0.2)
    # frames_freq = 0.5, dt = 5e-4 -> 4000 steps per frame; t_end 700 -> 350 frames
    assert d["frame_steps"] == 4000 and d["nFramesTot"] == 350


def test_temporal_table_file(sim, tmp_path):
    """SampleData/F_t.dat: records at t = 0, 400, 410, 810, 811 of 72 real or 144
    interleaved values (values read at float precision, as the reference does)."""
    src = open(os.path.join(SAMPLE, "test-lieb.ini")).read().replace('F = "_F.dat"', 'F_t = "F_t.dat"')
    for name in ("F_t.dat", "_E.dat", "_U.dat"):
        (tmp_path / name).write_bytes(open(os.path.join(SAMPLE, name), "rb").read())
    ini = tmp_path / "run.ini"
    ini.write_text(src)
    d = describe(sim, ini)
    F = d["F"]
    assert F["times"] == [0.0, 400.0, 410.0, 810.0, 811.0]
    tv = cvec(F["time_values"]).reshape(5, 72)
    assert np.all(tv[0] == 0) and np.all(tv[3] == 0)
    rec = open(os.path.join(SAMPLE, "F_t.dat")).read().split("\n\n")[1].split()
    vals = np.array([float(np.float32(x)) for x in rec[1:]])
    assert np.allclose(tv[1], vals[0::2] + 1j * vals[1::2], rtol=0, atol=0)


def write(tmp_path, text, **files):
    for k, v in files.items():
        (tmp_path / k).write_text(v)
    p = tmp_path / "run.ini"
    p.write_text(text)
    return p


BASE = """
nx = 2
ny = 3
J = 1
gamma = 1
timestep = 0.01
t_end = 1.0
frames_period = 0.5
beta_init = 0
beta_init_sigma = 0.5
omega = 0
F = 0
"""


def test_matrix_resolution_rules(sim, tmp_path):
    # column-major file: values[j * nx + i] -> (i, j)
    vals = np.arange(6) + 1.0
    ini = write(tmp_path, BASE + 'U = "u.dat"\n"F.Noise_Type" = "Uniform"\n"F.Noise_Val_0" = 0.06\n'
                "omega.data = [1, 2, 3, 4, 5, 6]\n"
                "beta_init.real = 0.25\nbeta_init.imag = -0.5\n", **{"u.dat": " ".join(map(str, vals))})
    d = describe(sim, ini)
    U = cvec(d["U"]["base"]).reshape(2, 3)
    assert np.allclose(U, vals.reshape(3, 2).T)
    assert np.allclose(cvec(d["omega"]["base"]).reshape(2, 3), vals.reshape(3, 2).T)
    assert np.allclose(cvec(d["beta_init"]["base"]), 0.25 - 0.5j)
    assert d["F"]["noise"] == 1 and np.allclose(cvec(d["F"]["amp"]), 0.06)


def test_complex_file_and_overrides(sim, tmp_path):
    vals = np.arange(12) * 0.5  # 6 complex values, interleaved, column-major
    ini = write(tmp_path, BASE + 'U.file = "uc.dat"\nSEED = 11\n', **{"uc.dat": " ".join(map(str, vals))})
    d = describe(sim, ini, "J", "2.5", "nx", "1", "ny", "6")
    assert d["J"] == 2.5 and d["seed"] == 11
    assert (d["nx"], d["ny"], d["dimension"]) == (1, 6, 1)
    c = vals[0::2] + 1j * vals[1::2]
    assert np.allclose(cvec(d["U"]["base"]), c)


def test_missing_matrix_file_is_an_error(sim, tmp_path):
    ini = write(tmp_path, BASE + 'U = "does_not_exist.dat"\n')
    r = subprocess.run([sim, "--describe", "-i", str(ini)], capture_output=True, text=True)
    assert r.returncode != 0 and "not found" in r.stderr


def test_bad_override_count(sim, tmp_path):
    ini = write(tmp_path, BASE + "U = 0.1\n")
    r = subprocess.run([sim, "--describe", "-i", str(ini), "J"], capture_output=True, text=True)
    assert r.returncode != 0


def test_folder_input_reads_sim_ini(sim, tmp_path):
    (tmp_path / "_sim.ini").write_text(BASE + "U = 0.3\n")
    r = subprocess.run([sim, "--describe", "-i", str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    d = json.loads(r.stdout)
    assert d["output"] == str(tmp_path) and np.allclose(cvec(d["U"]["base"]), 0.3)


def test_engine_options(sim, tmp_path):
    """The engine's own keys (absent from the reference's inputs): precision,
    hop and integrator, from the .ini and as command-line overrides; an
    unknown value is an error."""
    d = describe(sim, write(tmp_path, BASE))
    assert (d["precision"], d["hop"], d["integrator"]) == ("f32", "fft", "euler")
    ini = write(tmp_path, BASE + 'integrator = "split"\nprecision = "f64"\n')
    d = describe(sim, ini)
    assert (d["precision"], d["hop"], d["integrator"]) == ("f64", "fft", "split")
    d = describe(sim, ini, "hop", '"stencil"', "integrator", '"euler"')  # overrides are TOML values
    assert (d["hop"], d["integrator"]) == ("stencil", "euler")
    for key, val in (("integrator", '"rk4"'), ("hop", '"dense"'), ("precision", '"f16"')):
        r = subprocess.run([sim, "--describe", "-i", str(ini), key, val], capture_output=True, text=True)
        assert r.returncode != 0 and key in r.stderr, (key, r.stderr)
