"""The C++ adapters (include/thunderegg_gb300/adapters.hpp) against ThunderEgg's headers.

Where the reference sources are present: the header compiles with every adapter
instantiated, and flattening a Domain<D> that ThunderEgg built from our level
tables reproduces the tables exactly (the host logic the GPU path relies on).
"""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle as orc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _need_reference():
    if not orc.ref_sources_present():
        pytest.skip("reference sources not present")


def test_adapters_compile_against_reference_headers():
    _need_reference()
    orc.build(ref=True)
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    inc = [os.path.join(ROOT, "oracle", "_ref", "gen"), os.path.join(ROOT, "oracle", "ref", "mpishim"),
           os.path.dirname(orc.REF_SRC), os.path.join(ROOT, "include"), "/usr/local/cuda/include"]
    cmd = [cxx, "-std=c++17", "-fsyntax-only"] + [f"-I{p}" for p in inc] + [os.path.join(ROOT, "tests",
                                                                                      "adapters_check.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-4000:]


def _meshes():
    from thunderegg_gb300 import mesh as M

    return [M.uniform_mesh(2, 2, 8), M.circle_mesh(n=8, lo=2, hi=5), M.random_mesh(3, n=6, lo=1, hi=4),
            M.random_mesh(5, n=4, dim=3, lo=1, hi=3), M.uniform_mesh(3, 1, 4)]


@pytest.mark.parametrize("idx", range(5))
def test_flatten_roundtrip(idx):
    _need_reference()
    orc.build(ref=True)
    lib = ctypes.CDLL(orc.REF_LIB)
    for lv in _meshes()[idx]:
        d = lv.to_desc()
        outs = {}
        args = []
        for name, dt in (("id", np.int32), ("refine_level", np.int32), ("parent_id", np.int32),
                         ("orth_on_parent", np.int32), ("child_ids", np.int32), ("starts", np.float64),
                         ("spacings", np.float64), ("nbr_type", np.int32), ("nbr_ids", np.int32),
                         ("nbr_orth", np.int32)):
            a = np.full(np.shape(getattr(lv, name)), -7, dtype=dt)
            outs[name] = a
            args.append(a.ctypes.data_as(ctypes.c_void_p))
        rc = lib.teref_flatten_roundtrip(ctypes.byref(d), *args)
        assert rc == 0
        for name, a in outs.items():
            want = np.asarray(getattr(lv, name))
            if name == "nbr_orth":
                # only coarse neighbours carry an orthant
                want = np.where(np.asarray(lv.nbr_type) == 1, want, -1)
            if name == "nbr_ids":
                want = np.where((np.asarray(lv.nbr_type) >= 0)[..., None], want, -1)
            assert np.array_equal(a, want.astype(a.dtype)), name


def _adapt_lib():
    _need_reference()
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "adapt", f"REF_ROOT={orc.REF_ROOT}"],
                   check=True)
    lib = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libteadapt.so"))
    lib.teadapt_last_error.restype = ctypes.c_char_p
    return lib


@pytest.mark.parametrize("case", ["2d_circle_dft", "2d_uniform_bicgstab", "3d_random_dft"])
@pytest.mark.parametrize("path", [0, 1, 2])
def test_adapters_run_inside_reference_solvers(oracle, case, path):
    """The C++ adapters linked and run inside ThunderEgg's own classes (CPU; the ABI is a host
    stand-in forwarding to the oracle): (0) GMG::CycleBuilder handed the GPU parts, ThunderEgg's
    VCycle as Mr of ThunderEgg's Iterative::BiCGStab; (1) that builder's level chain as a GpuCycle
    (a GMG::Cycle subclass) under GpuBiCGStab; (2) GpuCycleBuilder's GpuCycle under ThunderEgg's
    BiCGStab.  The solution and iteration count equal the oracle's GMG-BiCGStab solve exactly."""
    from oracle import gmg_config
    from thunderegg_gb300 import capi
    from thunderegg_gb300 import mesh as M

    levels, scheme, smoother = {
        "2d_circle_dft": (M.circle_mesh(n=8, lo=2, hi=4), 1, 0),
        "2d_uniform_bicgstab": (M.uniform_mesh(2, 2, 8), 0, 1),
        "3d_random_dft": (M.random_mesh(5, n=4, dim=3, lo=1, hi=3), 2, 0),
    }[case]
    lib = _adapt_lib()
    f = np.random.default_rng(70).standard_normal(levels[0].padded_shape(1))
    arr = (capi.TeLevelDesc * len(levels))(*[lv.to_desc() for lv in levels])
    u = np.zeros_like(f)
    its = ctypes.c_int(0)
    dp = ctypes.POINTER(ctypes.c_double)
    rc = lib.teadapt_solve(arr, len(levels), scheme, smoother, path, ctypes.c_double(1e-10),
                           f.ctypes.data_as(dp), u.ctypes.data_as(dp), ctypes.byref(its))
    assert rc == 0, lib.teadapt_last_error()
    cfg = gmg_config(scheme=scheme, smoother=smoother, tol=1e-10, inner_continue_on_breakdown=1)
    u_o, its_o, _, rc_o = oracle.solve(levels, f, cfg)
    assert rc_o == 0
    assert its.value == its_o
    g = levels[0].num_ghost
    inner = (Ellipsis,) + tuple(slice(g, -g) for _ in range(levels[0].dim))
    assert np.array_equal(u[inner], u_o[inner])


def test_adapters_translate_errors():
    """A failing ABI call throws ThunderEgg::RuntimeError; a breakdown Iterative::BreakdownError."""
    assert _adapt_lib().teadapt_error_paths() == 3
