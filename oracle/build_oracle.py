"""Build recipe for the oracle (test infrastructure, not product code).

Compiles oracle/twmc_oracle.cpp into oracle/_build/libtwmc_oracle.so with
g++ -O2 and no fast-math or FP contraction, so the FP64 restatement rounds
like textbook IEEE arithmetic. A second, optimised copy
(libtwmc_oracle_fast.so, -O3, no -march=native so it runs on both x86 and
Arm hosts) is what bench.py times as the CPU baseline.

The reference itself is not built: its hot path needs Eigen3, FFTW3, cpptoml,
CLI11 and easylogging++, none of which exists in this image.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
SRC = os.path.join(HERE, "twmc_oracle.cpp")

VARIANTS = {
    "libtwmc_oracle.so": ["-O2", "-fno-fast-math", "-ffp-contract=off"],
    "libtwmc_oracle_fast.so": ["-O3", "-ffp-contract=fast"],
}


def build(force: bool = False) -> dict:
    os.makedirs(BUILD, exist_ok=True)
    out = {}
    for name, flags in VARIANTS.items():
        dst = os.path.join(BUILD, name)
        out[name] = dst
        if not force and os.path.exists(dst) and os.path.getmtime(dst) >= os.path.getmtime(SRC):
            continue
        cmd = ["g++", "-std=c++17", "-fPIC", "-shared", "-pthread", *flags, SRC, "-o", dst + ".tmp"]
        subprocess.run(cmd, check=True)
        os.replace(dst + ".tmp", dst)
    return out


def lib_path(fast: bool = False) -> str:
    return os.path.join(BUILD, "libtwmc_oracle_fast.so" if fast else "libtwmc_oracle.so")


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
