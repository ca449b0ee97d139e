"""The merge manager of twmc_sim (MergeManager.cpp:54-102) on the CPU:
archives written by an independent test writer are merged and read back."""
import os
import subprocess

import numpy as np
import pytest

import pinco_reader as pr
import pinco_writer as pw

NAMES = ["Omega_Realization", "traj", "work"]
DIMS = [[2, 2], [2, 2], [2, 2]]
FORMATS = [22, 22, 11]


def entry(rng, tid, ts, te, frames):
    return (tid, ts, te, {"Omega_Realization": rng.normal(size=(1, 4)) + 1j * rng.normal(size=(1, 4)),
                          "traj": rng.normal(size=(frames, 4)) + 1j * rng.normal(size=(frames, 4)),
                          "work": rng.normal(size=(frames, 4))})


@pytest.fixture(scope="module")
def sim():
    from pincosimulator_gb300 import build_ext

    return build_ext.build_host()


def test_merge_two_archives(sim, tmp_path):
    rng = np.random.default_rng(1)
    a = [entry(rng, 1, 0.0, 1.0, 3), entry(rng, 2, 0.0, 1.0, 3), entry(rng, 1, 1.0, 2.0, 2)]  # id 1 continued
    b = [entry(rng, 7, 0.0, 1.0, 3), entry(rng, 2, 0.0, 1.0, 3)]                             # id 2 in both
    pw.write_archive(tmp_path / "A" / "data", NAMES, DIMS, FORMATS, a)
    pw.write_archive(tmp_path / "B" / "data", NAMES, DIMS, FORMATS, b)
    (tmp_path / "A" / "data" / "_t.dat").write_text("%\tformat:real\n0\n0.5\n")
    # the writer's archives read back as written
    fr, real, ents = pr.read_trajectory(tmp_path / "A" / "data", 1)
    assert np.array_equal(fr, np.concatenate([a[0][3]["traj"], a[2][3]["traj"]])) and len(ents) == 2
    ini = tmp_path / "merge.ini"
    ini.write_text(f'Manager = "merge"\noldArchive1 = "{tmp_path / "A"}"\noldArchive2 = "{tmp_path / "B"}"\n')
    out = tmp_path / "M"
    r = subprocess.run([sim, "-i", str(ini), "-o", str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    data = out / "data"
    reg = pr.read_register(data)
    assert reg["names"] == NAMES and reg["dims"] == DIMS and reg["formats"] == FORMATS
    # archive 1 in id order (continuations joined into one entry), then archive 2
    assert [e["id"] for e in reg["entries"]] == [1, 2, 2, 7]
    fr1, real1, e1 = pr.read_trajectory(data, 1)
    assert len(e1) == 1 and e1[0]["t_start"] == 0.0 and e1[0]["t_end"] == 2.0
    assert np.array_equal(fr1, np.concatenate([a[0][3]["traj"], a[2][3]["traj"]]))
    assert np.array_equal(real1["work"], np.concatenate([a[0][3]["work"], a[2][3]["work"]]))
    assert np.array_equal(real1["Omega_Realization"], a[2][3]["Omega_Realization"][0])
    fr2, real2, e2 = pr.read_trajectory(data, 2)   # stored twice: the second is a continuation
    assert len(e2) == 2 and e2[0]["cont"] == e2[1]["pos"]
    assert np.array_equal(fr2, np.concatenate([a[1][3]["traj"], b[1][3]["traj"]]))
    fr7, _, _ = pr.read_trajectory(data, 7)
    assert np.array_equal(fr7, b[0][3]["traj"])
    assert (data / "_t.dat").read_text() == "%\tformat:real\n0\n0.5\n"


def test_merge_requires_both_archives(sim, tmp_path):
    ini = tmp_path / "merge.ini"
    ini.write_text(f'Manager = "merge"\noldArchive1 = "{tmp_path / "nope"}"\noldArchive2 = "{tmp_path / "nope"}"\n')
    r = subprocess.run([sim, "-i", str(ini), "-o", str(tmp_path / "M")], capture_output=True, text=True)
    assert r.returncode != 0 and "no archive" in (r.stdout + r.stderr)
