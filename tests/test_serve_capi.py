"""The C ABI's serving entry points (te_serve_*) on the host side: argument
checks, budget rejection, unknown ids and the counters.  None of these calls
touches the GPU (requests are only queued; no scheduling round runs)."""
import ctypes

import numpy as np
import pytest


@pytest.fixture(scope="module")
def lib():
    from thunderegg_gb300 import build, capi

    build.build()
    return capi


def _mesh():
    from thunderegg_gb300 import mesh as M

    return M.uniform_mesh(2, 2, 16)


def test_native_server_rejects_oversize_and_unknown_ids(lib):
    from thunderegg_gb300 import capi
    from thunderegg_gb300.gmg import GmgOptions
    from thunderegg_gb300.serve import NativeServer

    levels = _mesh()
    f = np.zeros(levels[0].padded_shape(1))
    srv = NativeServer(budget_bytes=1e5)  # smaller than any request
    with pytest.raises(capi.TeError) as e:
        srv.submit(levels, f, GmgOptions(scheme=1))
    assert e.value.code == capi.TE_ERR_BUDGET
    srv2 = NativeServer(budget_bytes=1e9)
    rid = srv2.submit(levels, f, GmgOptions(scheme=1))
    assert srv2.poll(rid) is None  # queued, no round has run
    assert lib.lib().te_serve_poll(srv2.h, 12345, None, None) == capi.TE_ERR_INVALID
    st, st2 = srv.stats(), srv2.stats()
    assert st["rejected"] == 1 and st["submitted"] == 0
    assert st2["submitted"] == 1 and st2["queued"] == 1 and st2["completed"] == 0
    srv.close()
    srv2.close()


def test_native_server_argument_checks(lib):
    from thunderegg_gb300 import capi
    from thunderegg_gb300.gmg import GmgOptions
    from thunderegg_gb300.serve import NativeServer

    L = lib.lib()
    o = capi.TeServeOpts(0.0, 1, 1)
    h = ctypes.c_void_p()
    assert L.te_serve_create(ctypes.byref(o), ctypes.byref(h)) == capi.TE_ERR_INVALID
    o = capi.TeServeOpts(1e9, 1, 0)
    assert L.te_serve_create(ctypes.byref(o), ctypes.byref(h)) == capi.TE_ERR_INVALID
    with pytest.raises(ValueError):
        NativeServer.solve_opts(GmgOptions(cycle_type="W"))
    with pytest.raises(ValueError):
        NativeServer.solve_opts(GmgOptions(krylov="cg"))
    srv = NativeServer(budget_bytes=1e9)
    levels = _mesh()
    rid = ctypes.c_longlong()
    so = NativeServer.solve_opts(GmgOptions())
    f = np.zeros(levels[0].padded_shape(1))
    descs = (capi.TeLevelDesc * 1)(levels[0].to_desc())
    # no levels, bad cycle precision, missing right-hand side
    assert L.te_serve_submit(srv.h, descs, 0, ctypes.byref(so), f.ctypes.data_as(capi._dp), ctypes.byref(rid)) \
        == capi.TE_ERR_INVALID
    so.cycle_dtype = 7
    assert L.te_serve_submit(srv.h, descs, 1, ctypes.byref(so), f.ctypes.data_as(capi._dp), ctypes.byref(rid)) \
        == capi.TE_ERR_INVALID
    so.cycle_dtype = capi.TE_F32
    assert L.te_serve_submit(srv.h, descs, 1, ctypes.byref(so), None, ctypes.byref(rid)) == capi.TE_ERR_INVALID
    assert srv.stats()["submitted"] == 0
    srv.close()
