"""The continuous-batching server (thunderegg_gb300.serve).

Requests arrive while others are on the GPU, are admitted against a memory
budget, share per-level launches with the other active requests of their class,
and leave when they finish.  Each served result is checked against the same
request solved alone:
  true FP64 residual ||f - A u|| / ||f|| <= 1e-10 (the solver tolerance)
  relative difference to the solo solution <= 1e-7 (both stop at 1e-10; the
  difference is bounded by cond(A) x tolerance)
"""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


def _requests(te, n=6):
    from thunderegg_gb300 import mesh as M
    from thunderegg_gb300 import problems as PB
    from thunderegg_gb300.gmg import GmgOptions
    from thunderegg_gb300.serve import Request

    rng = np.random.default_rng(40)
    circ = M.circle_mesh(n=16, lo=2, hi=4)
    uni = M.uniform_mesh(2, 3, 16)
    opts = GmgOptions(scheme=1, smoother=0, cycle_dtype=te.TE_F32, bicgstab_flags=1)
    out = []
    for i in range(n):
        levels = uni if i % 3 == 0 else circ
        out.append(Request(levels, PB.sine_modes_rhs(levels[0], rng), opts))
    return out


def _solo(te, req):
    from thunderegg_gb300.gmg import GmgSolver

    s = GmgSolver(req.levels, req.opts)
    fv, uv = te.Vector.from_numpy(s.finest, req.f), te.Vector(s.finest)
    s.solve(fv, uv)
    return s, fv, uv.numpy()


def _check(te, reqs, results):
    for rid, req in enumerate(reqs):
        r = results[rid]
        assert r.status == 0
        s, fv, solo = _solo(te, req)
        served = te.Vector.from_numpy(s.finest, r.u)
        assert s.residual(fv, served) <= 1e-10, rid
        inner = (Ellipsis, slice(1, -1), slice(1, -1))
        assert rel_err(r.u[inner], solo[inner]) <= 1e-7, rid


def test_serving_continuous_admission(te):
    """Requests submitted while earlier ones iterate join the running batches."""
    from thunderegg_gb300.serve import Server

    reqs = _requests(te)
    srv = Server(budget_bytes=64 << 30, steps_per_round=2)
    for r in reqs[:3]:
        srv.submit(r)
    srv.step()
    srv.step()
    assert not srv.idle()
    for r in reqs[3:]:
        srv.submit(r)  # arrive while the first three are on the GPU
    results = srv.run()
    assert sorted(results) == list(range(len(reqs)))
    assert srv.stats["max_batch"] >= 2          # requests shared launches
    assert any(res.restarts > 0 for res in results.values())  # a running batch was re-formed to admit
    _check(te, reqs, results)


def test_serving_memory_budget(te):
    """With room for two requests, at most two are active at a time and all finish."""
    from thunderegg_gb300.serve import Server, request_bytes

    reqs = _requests(te, 4)
    per = max(request_bytes(r.levels, r.opts) for r in reqs)
    srv = Server(budget_bytes=2 * per, steps_per_round=3)
    for r in reqs:
        srv.submit(r)
    results = srv.run()
    assert srv.stats["max_active_bytes"] <= 2 * per
    assert sorted(results) == list(range(len(reqs)))
    _check(te, reqs, results)


def test_serving_rejects_oversize(te):
    from thunderegg_gb300.capi import TE_ERR_BUDGET, TeError
    from thunderegg_gb300.serve import Server

    req = _requests(te, 1)[0]
    srv = Server(budget_bytes=1 << 20)
    with pytest.raises(TeError) as e:
        srv.submit(req)
    assert e.value.code == TE_ERR_BUDGET


def test_serving_union_cache(te):
    """A second wave of requests on the same meshes reuses the cached union
    hierarchies (and their captured graphs); results are unchanged."""
    from thunderegg_gb300.serve import Server

    reqs = _requests(te, 4)
    srv = Server(budget_bytes=64 << 30, steps_per_round=2)
    for r in reqs:
        srv.submit(r)
    first = srv.run()
    builds = srv.stats["union_builds"]
    assert builds >= 1
    for r in reqs:
        srv.submit(r)
    results = srv.run()
    assert srv.stats["union_hits"] >= 1
    assert srv.stats["union_builds"] - builds < builds  # most unions of the second wave were cached
    _check(te, reqs, {rid: first[rid] for rid in range(len(reqs))})
    _check(te, reqs, {rid - len(reqs): results[rid] for rid in range(len(reqs), 2 * len(reqs))})


def test_serving_cache_respects_budget(te):
    """Idle cached unions count against the budget and are evicted to admit new work."""
    from thunderegg_gb300.serve import Server, request_bytes

    reqs = _requests(te, 4)
    per = max(request_bytes(r.levels, r.opts) for r in reqs)
    srv = Server(budget_bytes=2 * per, steps_per_round=3)
    for r in reqs:
        srv.submit(r)
    results = srv.run()
    assert srv.stats["max_active_bytes"] <= 2 * per
    assert srv.active_bytes + srv._idle_cache_bytes() <= 2 * per
    assert srv.stats["union_evictions"] >= 1
    _check(te, reqs, results)


def test_serving_slot_fill(te):
    """A request on the mesh of a free slot starts in it while the batch keeps
    iterating (te_bicgstab_batch_reset); the running solves are not restarted
    and every result still matches its solo solve."""
    from thunderegg_gb300 import mesh as M
    from thunderegg_gb300 import problems as PB
    from thunderegg_gb300.gmg import GmgOptions
    from thunderegg_gb300.serve import Request, Server

    rng = np.random.default_rng(41)
    circ = M.circle_mesh(n=16, lo=2, hi=4)
    opts = GmgOptions(scheme=1, smoother=0, cycle_dtype=te.TE_F32, bicgstab_flags=1)
    reqs = [Request(circ, PB.sine_modes_rhs(circ[0], rng), opts) for _ in range(7)]
    srv = Server(budget_bytes=64 << 30, steps_per_round=2)
    for r in reqs[:5]:
        srv.submit(r)  # five members in a batch of six: one free slot
    srv.step()
    srv.step()
    srv.submit(reqs[5])  # takes the free slot
    srv.step()
    srv.submit(reqs[6])  # waits for a slot freed by a finished request, or a re-form
    results = srv.run()
    assert srv.stats["slot_fills"] >= 1
    assert results[5].restarts == 0
    assert all(results[i].restarts == 0 for i in range(5)) or srv.stats["reforms"] > 1
    _check(te, reqs, results)


def test_serving_packs_depths_into_one_class(te):
    """Solves of one patch size but different depths (uniform L1, L3 and a circle mesh of five
    levels) form one class: the union pads the shallower hierarchies with copies of their
    coarsest level, every result still matches its solo solve."""
    from thunderegg_gb300 import mesh as M
    from thunderegg_gb300 import problems as PB
    from thunderegg_gb300.gmg import GmgOptions
    from thunderegg_gb300.serve import Request, Server

    rng = np.random.default_rng(41)
    opts = GmgOptions(scheme=1, smoother=0, cycle_dtype=te.TE_F32, bicgstab_flags=1)
    meshes = [M.uniform_mesh(2, 1, 16), M.uniform_mesh(2, 3, 16), M.circle_mesh(n=16, lo=2, hi=4)]
    assert len({len(m) for m in meshes}) == 3
    reqs = [Request(m, PB.sine_modes_rhs(m[0], rng), opts) for m in meshes for _ in range(2)]
    with Server(budget_bytes=50e9, steps_per_round=2) as srv:
        for r in reqs:
            srv.submit(r)
        res = srv.run()
        assert len(srv.classes) == 1
        assert srv.stats["max_batch"] >= len(reqs)
    _check(te, reqs, res)
