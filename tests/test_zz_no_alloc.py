"""te_level_dot_noalloc: the dot product for callers that cannot allocate.

Such callers (hosts whose device memory is owned by another allocator, or
code that must not cause the device-wide synchronisation an allocation can)
get a reduction whose scratch is a fixed device array instead of a cudaMalloc.  Its result must equal the
existing te_vec_dot (same interior dot product) within FP64 reduction-order
tolerance, on consecutive calls (the shared scratch keeps the previous
call's contents), and oversized levels must be rejected before any GPU work.
This file is collected last so a failure here leaves every other test run.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-13  # relative; reduction order differs from te_vec_dot


def _noalloc_dot(te, lv, ncomp, dtype, x, y):
    ns = (ctypes.c_int * 3)(*(list(lv.ns) + [1] * (3 - len(lv.ns))))
    out = ctypes.c_double(np.nan)
    rc = te.capi.lib().te_level_dot_noalloc(lv.dim, ns, lv.num_ghost, lv.num_patches, ncomp, dtype, x.ptr, y.ptr,
                                            ctypes.byref(out), None)
    return rc, out.value


def test_noalloc_dot_matches_vec_dot_twice(te):
    import torch

    from thunderegg_gb300 import mesh as M

    for lv, ncomp in ((M.circle_mesh(n=8, lo=2, hi=5)[0], 1), (M.uniform_mesh(3, 1, 4)[0], 2)):
        dom = te.Domain(lv)
        rng = np.random.default_rng(7)
        for call in range(2):  # two calls in a row: the scratch must not leak state
            for dtype in (te.TE_F64, te.TE_F32):
                a = te.Vector.from_numpy(dom, rng.standard_normal(lv.padded_shape(ncomp)), dtype=dtype)
                b = te.Vector.from_numpy(dom, rng.standard_normal(lv.padded_shape(ncomp)), dtype=dtype)
                want = a.dot(b)
                torch.cuda.synchronize()
                rc, got = _noalloc_dot(te, lv, ncomp, dtype, a, b)
                assert rc == 0, te.capi.lib().te_last_error_message()
                scale = float(np.sum(np.abs(a.numpy() * b.numpy())))
                assert abs(got - want) <= TOL * scale, (call, dtype, got, want)


def test_noalloc_dot_rejects_oversized_level(te):
    from thunderegg_gb300 import mesh as M

    lv = M.uniform_mesh(2, 1, 4)[0]
    dom = te.Domain(lv)
    a = te.Vector(dom)
    ns = (ctypes.c_int * 3)(4, 4, 1)
    out = ctypes.c_double(0)
    too_many = te.capi.TE_NOALLOC_MAX_PARTIALS + 1 if hasattr(te.capi, "TE_NOALLOC_MAX_PARTIALS") else 65537
    rc = te.capi.lib().te_level_dot_noalloc(2, ns, 1, too_many, 1, te.TE_F64, a.ptr, a.ptr, ctypes.byref(out), None)
    assert rc == te.capi.TE_ERR_UNSUPPORTED
    assert b"exceeds the limit" in te.capi.lib().te_last_error_message()
