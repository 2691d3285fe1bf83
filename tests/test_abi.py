"""The C ABI library loads here (no GPU needed) and exports every entry point
include/te_gpu.h declares; the Python binding covers the same set."""
import os
import re

from conftest import ROOT


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "te_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(te_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "te_domain_create" in syms and "te_bicgstab_solve" in syms
    assert len(syms) >= 40


def test_library_exports_all_declared_symbols(te):
    import ctypes

    from thunderegg_gb300 import capi

    lib = ctypes.CDLL(capi.LIB_PATH)
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_python_binding_matches_header():
    from thunderegg_gb300 import capi

    assert sorted(capi.exported_symbols()) == declared_symbols()


def test_library_loads_without_gpu(te):
    from thunderegg_gb300 import capi

    assert capi.lib().te_kernel_launch_count() >= 0
