"""The serving loop's scheduling on the CPU (thunderegg_gb300.serve.Server).

The device objects (_Union: a union hierarchy's solver and buffers; _Batch: its
resumable slot-mode BiCGStab run) are replaced by fakes in which request i
needs a given number of iterations, so admission against the memory budget,
the union cache and its LRU eviction, the bucketed batch sizes with free
slots, slot fills, restarts from the true residual and re-forms are checked
without a GPU.  The GPU tests (test_gpu_serve.py) check the same loop's
numerical results.
"""
import numpy as np
import pytest

import thunderegg_gb300.serve as S
from thunderegg_gb300 import mesh as M
from thunderegg_gb300.gmg import GmgOptions

MESH = None


def mesh():
    global MESH
    if MESH is None:
        # 0 and 2: two meshes of one class (same shape and depth); 1: another class
        MESH = (M.uniform_mesh(2, 2, 8), M.uniform_mesh(2, 3, 8), M.uniform_mesh(2, 2, 8))
    return MESH


class _X:
    def __init__(self, v):
        self.v = v

    def cpu(self):
        return self

    def numpy(self):
        return self.v

    def clone(self):
        return _X(self.v)


class FakeUnion:
    built = []

    def __init__(self, reqs, opts):
        self.reqs = list(reqs)
        self.keep = [(r.levels, r.coeffs) for r in reqs]
        self.bytes = sum(S.request_bytes(r.levels, r.opts) for r in reqs)
        self.busy = False
        FakeUnion.built.append(len(reqs))


class FakeBatch:
    """Slot batch: the request in slot i needs int(req.f[0]) iterations in total; a
    re-formed member keeps its count; slots beyond the members start free.  A
    request with f[1] = k fails its true-residual check k times: each failed
    finish restarts it for one more iteration."""

    def __init__(self, members, x_parts, un):
        self.un = un
        un.busy = True
        self.h = object()
        self.B = len(un.keep)
        assert self.B >= len(members)
        self.slot_key = [(id(lv), id(c)) for lv, c in un.keep]
        self.slots = list(members) + [None] * (self.B - len(members))
        self.base_its = [m.iterations for m in members] + [0] * (self.B - len(members))
        self.done = [0] * self.B
        self.extra = [0] * self.B  # iterations added by restarts
        self.fails = [self._fails(m) for m in members] + [0] * (self.B - len(members))
        self.puts = 0

    @staticmethod
    def _fails(m):
        return int(m.req.f[1]) if len(m.req.f) > 1 else 0

    @property
    def members(self):
        return [m for m in self.slots if m is not None]

    def free_slot(self, req):
        key = (id(req.levels), id(req.coeffs))
        for i, m in enumerate(self.slots):
            if m is None and self.slot_key[i] == key:
                return i
        return -1

    def put(self, i, member):
        assert self.slots[i] is None and self.slot_key[i] == (id(member.req.levels), id(member.req.coeffs))
        self.slots[i] = member
        self.base_its[i] = member.iterations
        self.done[i] = 0
        self.extra[i] = 0
        self.fails[i] = self._fails(member)
        self.puts += 1

    def _left(self, i):
        m = self.slots[i]
        return 0 if m is None else int(m.req.f[0]) + self.extra[i] - self.base_its[i] - self.done[i]

    def step(self, k):
        for i in range(self.B):
            self.done[i] += max(0, min(k, self._left(i)))
        return sum(1 for i in range(self.B) if self._left(i) > 0)

    def state(self):
        run = [1 if self._left(i) > 0 else 0 for i in range(self.B)]
        return list(self.done), [1e-11] * self.B, [0] * self.B, run

    def finish(self, slots):
        out = []
        for i in slots:
            assert self.slots[i] is not None and self._left(i) == 0
            if self.fails[i] > 0:  # restarted from its true residual
                self.fails[i] -= 1
                self.extra[i] += 1
                out.append(False)
            else:
                out.append(True)
        return out

    def slice_x(self, i):
        return _X(np.full(3, float(self.slots[i].rid)))

    def close(self):
        self.un.busy = False
        self.h = None


@pytest.fixture
def fake(monkeypatch):
    FakeUnion.built = []
    monkeypatch.setattr(S, "_Union", FakeUnion)
    monkeypatch.setattr(S, "_Batch", FakeBatch)

    class Lib:
        def te_bicgstab_batch_sync_x(self, h):
            return 0

    monkeypatch.setattr(S, "lib", lambda: Lib())
    monkeypatch.setattr(S, "check", lambda rc: rc)
    return FakeUnion


def req(iters, which=0):
    return S.Request(mesh()[which], np.array([float(iters)]), GmgOptions())


def run_checked(srv, max_rounds=10000):
    """Run to the end, checking the memory invariant after every round."""
    r = 0
    while not srv.idle() and r < max_rounds:
        srv.step()
        assert srv.active_bytes + srv._idle_cache_bytes() <= srv.budget
        r += 1
    assert srv.idle()
    return srv.results


def test_budget_bounds_active_requests(fake):
    per = S.request_bytes(mesh()[0], GmgOptions())
    srv = S.Server(budget_bytes=2 * per, steps_per_round=2)
    ids = [srv.submit(req(5 + i)) for i in range(5)]
    res = run_checked(srv)
    assert sorted(res) == ids
    assert srv.stats["max_active_bytes"] <= 2 * per
    assert srv.active_bytes == 0
    # each request ran exactly the iterations it needed, through any re-forms
    for i, rid in enumerate(ids):
        assert res[rid].iterations == 5 + i


def test_oversize_request_rejected(fake):
    from thunderegg_gb300.capi import TE_ERR_BUDGET, TeError

    srv = S.Server(budget_bytes=1000)
    with pytest.raises(TeError) as e:
        srv.submit(req(3))
    assert e.value.code == TE_ERR_BUDGET


def test_union_cache_reuses_member_sequences(fake):
    srv = S.Server(budget_bytes=1 << 40, steps_per_round=4)
    for _ in range(3):
        srv.submit(req(4))
    run_checked(srv)
    builds = srv.stats["union_builds"]
    for _ in range(3):
        srv.submit(req(4))
    run_checked(srv)
    assert srv.stats["union_builds"] == builds  # the same sequence of meshes: all from the cache
    assert srv.stats["union_hits"] >= 1


def test_batches_round_up_to_buckets_with_free_slots(fake):
    per = S.request_bytes(mesh()[0], GmgOptions())
    srv = S.Server(budget_bytes=1 << 40, steps_per_round=2)
    for _ in range(5):
        srv.submit(req(6))
    srv.step()  # admit and form the first batch
    assert FakeUnion.built[-1] == 6  # five members, rounded up to the bucket of six
    cls = next(iter(srv.classes.values()))
    assert cls["batch"].B == 6 and len(cls["batch"].members) == 5
    assert srv.active_bytes == 6 * per
    run_checked(srv)
    assert srv.active_bytes == 0


def test_no_free_slots_without_budget_room(fake):
    per = S.request_bytes(mesh()[0], GmgOptions())
    srv = S.Server(budget_bytes=5 * per, steps_per_round=2)
    for _ in range(5):
        srv.submit(req(6))
    srv.step()
    assert FakeUnion.built[-1] == 5
    run_checked(srv)


def test_idle_unions_evicted_lru_to_admit(fake):
    per0 = S.request_bytes(mesh()[0], GmgOptions())
    per1 = S.request_bytes(mesh()[1], GmgOptions())
    srv = S.Server(budget_bytes=per0 + per1 - 1, steps_per_round=8)
    srv.submit(req(3, 0))
    run_checked(srv)  # one idle cached union of mesh 0
    assert srv._idle_cache_bytes() == per0
    srv.submit(req(3, 1))  # needs the room the idle union holds
    run_checked(srv)
    assert srv.stats["union_evictions"] >= 1
    assert len(srv.results) == 2


def test_union_cache_key_includes_solver_options(fake):
    """Requests on the same mesh with different solver options never share a union."""
    srv = S.Server(budget_bytes=1 << 40, steps_per_round=4)
    srv.submit(req(3))
    run_checked(srv)
    builds = srv.stats["union_builds"]
    srv.submit(S.Request(mesh()[0], np.array([3.0]), GmgOptions(cycle_type="W")))
    run_checked(srv)
    assert srv.stats["union_builds"] == builds + 1


def test_new_requests_fill_free_slots_without_reform(fake):
    """A request on the mesh of a free slot starts in it while the others keep iterating:
    no new union, no re-form, no restart of the running solves."""
    srv = S.Server(budget_bytes=1 << 40, steps_per_round=2)
    first = [srv.submit(req(20)) for _ in range(3)]  # bucket of 3: no free slot
    short = srv.submit(req(2))  # waits a round, then the batch re-forms to 4 slots
    srv.step()
    srv.step()
    builds, reforms = srv.stats["union_builds"], srv.stats["reforms"]
    while short not in srv.results:
        srv.step()
    late = [srv.submit(req(4)) for _ in range(1)]  # the freed slot takes it
    res = run_checked(srv)
    assert srv.stats["slot_fills"] >= 1
    assert srv.stats["union_builds"] == builds and srv.stats["reforms"] == reforms
    for rid in first:
        assert res[rid].iterations == 20
    assert res[late[0]].iterations == 4 and res[late[0]].restarts == 0


def test_other_mesh_reforms_and_carries_iterations(fake):
    """A waiting request of another mesh finds no slot: the batch re-forms with it and the
    running requests carry their iteration counts (one restart each)."""
    srv = S.Server(budget_bytes=1 << 40, steps_per_round=2)
    a = [srv.submit(req(12, 0)) for _ in range(2)]
    srv.step()
    srv.step()
    b = srv.submit(req(5, 2))
    res = run_checked(srv)
    for rid in a:
        assert res[rid].iterations == 12 and res[rid].restarts == 1
    assert res[b].iterations == 5
    assert srv.stats["reforms"] >= 2


def test_slot_reservation_counts_waiting_requests(fake):
    """Two arrivals for one free slot: only the first is admitted without memory."""
    per = S.request_bytes(mesh()[0], GmgOptions())
    srv = S.Server(budget_bytes=1 << 40, steps_per_round=1)
    [srv.submit(req(30)) for _ in range(2)]
    srv.submit(req(1))
    srv.step()
    cls = next(iter(srv.classes.values()))
    assert cls["batch"].B == 3
    while any(m is not None and int(m.req.f[0]) == 1 for m in cls["batch"].slots):
        srv.step()
    cls["batch"].step(0)
    srv.queue = []
    srv.submit(req(3))
    srv.submit(req(3))
    srv._admit()
    assert sorted(cls["bytes"].values()) == [0, per]
    run_checked(srv)
    assert srv.active_bytes == 0


def test_restarted_slots_stay_until_confirmed(fake):
    """A slot whose true residual fails the check restarts in place: its request keeps the
    slot, iterates again and retires only once confirmed."""
    srv = S.Server(budget_bytes=1 << 40, steps_per_round=2)
    plain = srv.submit(req(4))
    retried = srv.submit(S.Request(mesh()[0], np.array([4.0, 2.0]), GmgOptions()))
    res = run_checked(srv)
    assert res[plain].iterations == 4
    assert res[retried].iterations == 6  # two restarts of one iteration each
    assert srv.stats["reforms"] == 1 and srv.active_bytes == 0


def test_close_releases_everything(fake):
    srv = S.Server(budget_bytes=1 << 40, steps_per_round=1)
    with srv:
        for _ in range(3):
            srv.submit(req(10))
        srv.submit(req(10, 1))
        srv.step()
        batches = [c["batch"] for c in srv.classes.values()]
        assert all(b is not None for b in batches)
    assert all(b.h is None and not b.un.busy for b in batches)  # destroyed, unions released
    assert srv.unions == {} and srv.active_bytes == 0 and srv.idle() and srv.pool is None
