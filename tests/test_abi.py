"""The C-ABI library builds, loads and exports every declared symbol (CPU, no GPU calls)."""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "twmc.h")).read()
    return sorted(set(re.findall(r"TWMC_API\s+[\w\s\*]+?\b(twmc_\w+)\s*\(", text)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("twmc_version", "twmc_create", "twmc_run", "twmc_set_noise_buffer", "twmc_progress",
              "twmc_last_error", "twmc_destroy"):
        assert s in syms


def test_library_exports_all_declared(built_lib):
    for s in declared_symbols():
        assert hasattr(built_lib, s), s
    assert built_lib.twmc_version() == 3


def test_binding_lists_every_export():
    from pincosimulator_gb300 import twmc

    assert sorted(twmc.EXPORTED) == declared_symbols()
