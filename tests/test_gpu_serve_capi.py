"""The C ABI's serving loop (te_serve_*, driven through NativeServer).

Requests of two patch sizes and several depths arrive while others are on the
GPU; each served result is checked against the same request solved alone:
  true FP64 residual ||f - A u|| / ||f|| <= 1e-10 (the solver tolerance)
  relative difference to the solo solution <= 1e-7 (both stop at 1e-10)
"""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


def _requests(te, n, seed):
    from thunderegg_gb300 import mesh as M
    from thunderegg_gb300 import problems as PB
    from thunderegg_gb300.gmg import GmgOptions

    rng = np.random.default_rng(seed)
    meshes = [M.circle_mesh(n=16, lo=2, hi=4), M.uniform_mesh(2, 3, 16), M.uniform_mesh(2, 2, 32)]
    opts = GmgOptions(scheme=1, smoother=0, cycle_dtype=te.TE_F32, bicgstab_flags=1)
    out = []
    for i in range(n):
        levels = meshes[i % 3]
        out.append((levels, PB.sine_modes_rhs(levels[0], rng), opts))
    return out


def _check(te, req, r):
    from thunderegg_gb300.gmg import GmgSolver

    levels, f, opts = req
    assert r.status == 0
    s = GmgSolver(levels, opts)
    fv, uv = te.Vector.from_numpy(s.finest, f), te.Vector(s.finest)
    s.solve(fv, uv)
    served = te.Vector.from_numpy(s.finest, r.u)
    assert s.residual(fv, served) <= 1e-10
    inner = (Ellipsis, slice(1, -1), slice(1, -1))
    assert rel_err(r.u[inner], uv.numpy()[inner]) <= 1e-7


def test_native_server_continuous_batching(te):
    from thunderegg_gb300.serve import NativeServer

    reqs = _requests(te, 6, 50)
    with NativeServer(budget_bytes=64 << 30, steps_per_round=2) as srv:
        ids = [srv.submit(*r) for r in reqs[:3]]
        srv.step()
        srv.step()
        assert srv.stats()["active"] > 0
        ids += [srv.submit(*r) for r in reqs[3:]]  # arrive while the first three iterate
        res = srv.run(ids)
        st = srv.stats()
        assert sorted(res) == sorted(ids)
        assert st["completed"] == 6 and st["active"] == 0 and st["queued"] == 0
        assert st["classes"] == 2  # 16^2 (two depths in one class) and 32^2
        assert st["reforms"] >= 2
        for rid, req in zip(ids, reqs):
            _check(te, req, res[rid])
        # a second wave on the same meshes: served from the cached unions
        reqs2 = _requests(te, 3, 51)
        ids2 = [srv.submit(*r) for r in reqs2]
        res2 = srv.run(ids2)
        assert srv.stats()["union_cache_hits"] >= 1
        for rid, req in zip(ids2, reqs2):
            _check(te, req, res2[rid])


def test_native_server_budget_holds_two(te):
    """With room for two requests at a time every request still finishes."""
    from thunderegg_gb300 import serve as S
    from thunderegg_gb300.serve import NativeServer

    reqs = _requests(te, 12, 52)[::3][:4]  # four requests on the same mesh
    one = S.request_bytes(reqs[0][0], reqs[0][2])
    with NativeServer(budget_bytes=2.5 * one, steps_per_round=2) as srv:
        ids = [srv.submit(*r) for r in reqs]
        srv.step()
        st = srv.stats()
        assert st["active"] <= 2 and st["queued"] >= 2
        res = srv.run(ids)
        for rid, req in zip(ids, reqs):
            _check(te, req, res[rid])
