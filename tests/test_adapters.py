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
