"""GB300-native Truncated Wigner Monte Carlo trajectory engine.

The compute path is libtwmc_cuda.so (pincosimulator_gb300/csrc, C ABI in
include/twmc.h); `pincosimulator_gb300.twmc` is its ctypes binding.
"""
from . import fft_plan  # noqa: F401

__all__ = ["fft_plan", "twmc", "build"]


def build(force: bool = False, verbose: bool = False) -> str:
    from . import build_ext

    return build_ext.build(force=force, verbose=verbose)
