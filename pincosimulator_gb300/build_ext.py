"""Builds libtwmc_cuda.so (the C-ABI CUDA library) in-tree for sm_103a.

Steps: emit csrc/fft_plans.inc from fft_plan.py, compile every csrc/*.cu
with nvcc (one -gencode, translation units in parallel), link a shared
library into pincosimulator_gb300/_build/. No cmake; runs the same on the
x86 build container and the Arm GPU host.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libtwmc_cuda.so")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
         "-Xcompiler", "-fvisibility=hidden", "-DNDEBUG", "-I", os.path.join(HERE, "..", "include")]
SOURCES = ["twmc_api.cu", "twmc_square_f32.cu", "twmc_square_f64.cu", "twmc_ell.cu", "twmc_misc.cu",
           "twmc_noalloc.cu", "twmc_hbatch.cu",
           "twmc_mlp.cu", "twmc_ell_fast.cu"]


def _write_plans() -> None:
    sys.path.insert(0, os.path.dirname(HERE))
    from pincosimulator_gb300 import fft_plan

    text = fft_plan.emit_header()
    dst = os.path.join(CSRC, "fft_plans.inc")
    if not os.path.exists(dst) or open(dst).read() != text:
        with open(dst, "w") as f:
            f.write(text)


def _deps_hash() -> str:
    h = hashlib.sha256()
    for name in sorted(os.listdir(CSRC)):
        if name.endswith((".cu", ".cuh", ".h", ".inc")):
            with open(os.path.join(CSRC, name), "rb") as f:
                h.update(name.encode() + f.read())
    with open(os.path.join(HERE, "..", "include", "twmc.h"), "rb") as f:
        h.update(f.read())
    h.update(" ".join(ARCH + FLAGS).encode())
    return h.hexdigest()


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(BUILD, src.replace(".cu", ".o"))
    cmd = [NVCC, *ARCH, *FLAGS, "-c", os.path.join(CSRC, src), "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
    if verbose and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


HOST = os.path.join(HERE, "host")
HOST_LIB = os.path.join(BUILD, "libtwmc_host.so")
SIM = os.path.join(BUILD, "twmc_sim")
HOST_SOURCES = ["Settings.cpp", "NoisyMatrix.cpp", "TWMC.cpp", "PincoFormat.cpp"]
CXX = os.environ.get("CXX", "g++")


def _host_hash() -> str:
    h = hashlib.sha256()
    for name in sorted(os.listdir(HOST)):
        with open(os.path.join(HOST, name), "rb") as f:
            h.update(name.encode() + f.read())
    with open(os.path.join(HERE, "..", "include", "twmc.h"), "rb") as f:
        h.update(f.read())
    return h.hexdigest()


def build_host(force: bool = False) -> str:
    """libtwmc_host.so (Solver plugin layer, settings, archive) and twmc_sim."""
    stamp = os.path.join(BUILD, "host_stamp.txt")
    digest = _host_hash()
    if not force and os.path.exists(SIM) and os.path.exists(stamp) and open(stamp).read() == digest:
        return SIM
    flags = ["-std=c++17", "-O2", "-fPIC", "-Wall", "-Wno-sign-compare", "-I" + os.path.join(HERE, "..", "include")]
    link = ["-L" + BUILD, "-Wl,-rpath,$ORIGIN"]
    srcs = [os.path.join(HOST, s) for s in HOST_SOURCES]
    subprocess.run([CXX, *flags, "-shared", *srcs, "-o", HOST_LIB + ".tmp", *link, "-ltwmc_cuda"], check=True)
    os.replace(HOST_LIB + ".tmp", HOST_LIB)
    subprocess.run([CXX, *flags, os.path.join(HOST, "twmc_sim.cpp"), "-o", SIM + ".tmp", *link,
                    "-Wl,--no-as-needed", "-ltwmc_host", "-ltwmc_cuda"], check=True)
    os.replace(SIM + ".tmp", SIM)
    with open(stamp, "w") as f:
        f.write(digest)
    return SIM


def build(force: bool = False, verbose: bool = False) -> str:
    lib = build_cuda(force=force, verbose=verbose)
    build_host(force=force)
    return lib


def build_cuda(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    _write_plans()
    stamp = os.path.join(BUILD, "stamp.txt")
    digest = _deps_hash()
    if not force and os.path.exists(LIB) and os.path.exists(stamp) and open(stamp).read() == digest:
        return LIB
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    tmp = LIB + ".tmp"
    subprocess.run([NVCC, *ARCH, "-shared", "-o", tmp, *objs], check=True)
    os.replace(tmp, LIB)
    with open(stamp, "w") as f:
        f.write(digest)
    # the host library links against this one
    hs = os.path.join(BUILD, "host_stamp.txt")
    if os.path.exists(hs):
        os.remove(hs)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
