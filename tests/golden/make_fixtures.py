"""Copies the reference's SampleData input fixtures into tests/golden/sampledata.

Source: SampleData/test-sim.ini, SampleData/test-lieb.ini and
SampleData/F_t.dat of the PincoSimulator project (the only fixtures it ships;
they pin input parsing, not results). test-lieb.ini names matrix files
_E.dat, _F.dat and _U.dat that the project does not ship; this script writes
small synthetic ones (24 cells x 3 sites, column-major values) so the file
resolves. Run once where the reference is mounted, with its root as the
argument or in $PINCO_REFERENCE_ROOT:

    python tests/golden/make_fixtures.py /path/to/PincoSimulator
"""
import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
DST = os.path.join(HERE, "sampledata")


def main(ref_root):
    os.makedirs(DST, exist_ok=True)
    for name in ("test-sim.ini", "test-lieb.ini", "F_t.dat"):
        shutil.copyfile(os.path.join(ref_root, "SampleData", name), os.path.join(DST, name))
    rng = np.random.default_rng(20171127)
    n = 24 * 3
    np.savetxt(os.path.join(DST, "_E.dat"), rng.normal(size=n), fmt="%.6f", newline=" ")
    np.savetxt(os.path.join(DST, "_U.dat"), 0.3 + 0.01 * rng.normal(size=n), fmt="%.6f", newline=" ")
    F = np.zeros(n)
    F[1::3] = 2.5
    np.savetxt(os.path.join(DST, "_F.dat"), F, fmt="%.6f", newline=" ")


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PINCO_REFERENCE_ROOT")
    if not root:
        sys.exit("usage: make_fixtures.py <PincoSimulator root> (or set PINCO_REFERENCE_ROOT)")
    main(root)
