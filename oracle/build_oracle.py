"""Build recipe for the oracle (test infrastructure, not product code).

Compiles oracle/twmc_oracle.cpp into oracle/_build/libtwmc_oracle.so with
g++ -O2 and no fast-math or FP contraction, so the FP64 restatement rounds
like textbook IEEE arithmetic. Two optimised copies are timing builds for
bench.py's CPU baseline: libtwmc_oracle_fast.so (-O3) and
libtwmc_oracle_ref_flags.so with the reference's own release flags (-Ofast
-march=native, CMakeLists.txt:15; built on the host that runs it, so the
native target is that host's).

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
    # the reference's own release flags (CMakeLists.txt:15); a CPU-baseline
    # timing build only, never the checker
    "libtwmc_oracle_ref_flags.so": ["-Ofast", "-march=native"],
}
# if the compiler rejects -march=native on a host, the timing build drops it
FALLBACK = {"-march=native": None}


def build(force: bool = False) -> dict:
    os.makedirs(BUILD, exist_ok=True)
    out = {}
    for name, flags in VARIANTS.items():
        dst = os.path.join(BUILD, name)
        out[name] = dst
        if not force and os.path.exists(dst) and os.path.getmtime(dst) >= os.path.getmtime(SRC):
            continue
        cmd = ["g++", "-std=c++17", "-fPIC", "-shared", "-pthread", *flags, SRC, "-o", dst + ".tmp"]
        if subprocess.run(cmd).returncode != 0:
            cmd = [c for c in cmd if c not in FALLBACK]
            subprocess.run(cmd, check=True)
        os.replace(dst + ".tmp", dst)
        with open(dst + ".flags", "w") as f:
            f.write(" ".join(c for c in cmd if c.startswith("-O") or c.startswith("-m") or c.startswith("-ff")))
    return out


def lib_path(fast=False) -> str:
    """fast: False = the checker, True = the -O3 timing build, "ref_flags" =
    the timing build with the reference's -Ofast -march=native."""
    if fast == "ref_flags":
        return os.path.join(BUILD, "libtwmc_oracle_ref_flags.so")
    return os.path.join(BUILD, "libtwmc_oracle_fast.so" if fast else "libtwmc_oracle.so")


def build_flags(fast=False) -> str:
    """Optimisation flags the given build was compiled with."""
    try:
        return open(lib_path(fast) + ".flags").read()
    except OSError:
        return ""


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
