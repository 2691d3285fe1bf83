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


def test_slot_entry_points_reject_bad_arguments_without_gpu(te):
    """The slot-mode batch entry points check their arguments before any device work, so
    a null handle is an error status and a message, not a crash."""
    import ctypes

    from thunderegg_gb300 import capi

    L = capi.lib()
    fin, sl = (ctypes.c_int * 1)(), (ctypes.c_int * 1)(0)
    assert L.te_bicgstab_batch_reset(None, 0) == capi.TE_ERR_INVALID
    assert b"null" in L.te_last_error_message()
    assert L.te_bicgstab_batch_finish_slots(None, 1, sl, fin) == capi.TE_ERR_INVALID
    assert L.te_bicgstab_batch_step(None, 1, ctypes.byref(ctypes.c_int())) == capi.TE_ERR_INVALID
