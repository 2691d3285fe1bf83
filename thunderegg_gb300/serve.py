"""Continuous batching of independent Poisson solves on one GPU.

A request is one GMG-preconditioned BiCGStab solve on its own mesh
hierarchy.  Requests whose hierarchies share patch shape and solver options
form a class, whatever their depth; the active requests of a class are packed
into one union hierarchy (mesh.union_hierarchy, shallower members padded with
copies of their coarsest level by mesh.pad_hierarchy), so every per-level kernel of the
V-cycle and every Krylov kernel runs over all of them in one launch (one CUDA
graph replay per iteration).  A batch is a fixed set of slots, one solve each
(TE_BICGSTAB_SLOTS): the server steps each class's batch a few iterations at a
time (te_bicgstab_batch_step), and between steps it

  * admits queued requests while the estimated device memory of the live
    batches, the requests waiting for a slot and the idle cached unions stays
    within the budget,
  * puts a waiting request into a free slot built on its mesh
    (te_bicgstab_batch_reset): its right-hand side and initial iterate are
    copied into the slot and its solve starts while the other slots keep
    iterating,
  * finishes the slots whose solves stopped, together
    (te_bicgstab_batch_finish_slots: one FP64 residual pass; each true
    residual either confirms its solve, whose result is copied out and whose
    slot is freed, or restarts it),
  * re-forms a class's batch when requests have waited without a slot of
    their mesh: the new union hierarchy is built (rounded up to a bucket size,
    the extra slots free), every continuing request's current iterate and
    right-hand side are copied into it, and its BiCGStab restarts from that
    iterate (its residual keeps decreasing; only the Krylov space is rebuilt).

A union hierarchy depends only on its members' meshes (and coefficients), not
on their right-hand sides, so the device objects of every union built are kept
in a per-server cache keyed by the members' mesh sequence, together with the
batch's x and b buffers (so the cycle's and the iteration's captured CUDA
graphs are replayed, not captured again).  Idle cache entries count against
the memory budget and are evicted least recently used when an admission needs
the room.

Each request stops on its own residual test; its arithmetic never mixes with
other requests' (per-patch kernels, per-solve reductions), so its result
matches a solve of the same request alone within the solver tolerance.

Every class has its own CUDA stream (its handles bind to it when its unions
are built), and the batches of different classes are stepped concurrently
from worker threads (the step entry point releases the interpreter lock), so
one class's kernels fill the GPU while another waits on its host-side
convergence test.  Everything else -- admission, building unions, copying
iterates, retiring -- runs on the thread that owns the server.
"""
from __future__ import annotations

import contextlib
import ctypes
import dataclasses
import itertools
import time
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field

import numpy as np

from . import Vector
from . import mesh as M
from .capi import TE_BICGSTAB_SLOTS, check, lib
from .gmg import GmgOptions, GmgSolver


@dataclass
class Request:
    levels: list                     # the request's MeshLevel hierarchy (finest first)
    f: np.ndarray                    # right-hand side, finest level, padded layout (1 component)
    opts: GmgOptions = field(default_factory=GmgOptions)
    coeffs: list | None = None       # VarPoisson coefficients per level, or None
    u0: np.ndarray | None = None     # initial iterate (default 0)


@dataclass
class Result:
    u: np.ndarray
    iterations: int
    residual: float                  # final relative residual (FP64 true residual in the mixed mode)
    status: int
    latency_s: float                 # submit -> result copied out
    restarts: int                    # batch re-formations the request went through


def request_bytes(levels, opts: GmgOptions) -> int:
    """Device memory a request holds while active: cycle work buffers (f, u, r in
    the cycle's precision, plus the post-smooth corrections) on every level, the
    finest level's Krylov vectors, iterate, right-hand side and operator
    buffers, and the level tables."""
    w = 4 if opts.cycle_dtype != 0 else 8
    total = 0
    for k, lv in enumerate(levels):
        cells = lv.num_patches * int(np.prod(lv.padded_shape(1)[2:]))
        total += cells * 3 * w + lv.num_patches * 2 * lv.dim * lv.ns[0] ** (lv.dim - 1) * 4
        total += lv.num_patches * 512  # neighbour, ghost-call and plan tables
        if k == 0:
            total += cells * (8 * 8 + 8 * 3 + 8)  # Krylov vectors, float-float iterate, x and b, residual
    return int(total)


def _class_key(r: Request):
    """Requests batch together when their patch shape, coefficient use and every solver option
    agree, whatever their depth: a union pads its shallower members with copies of their
    coarsest level (mesh.pad_hierarchy), so their patches share every per-level launch."""
    lv = r.levels[0]
    return (lv.dim, tuple(lv.ns), lv.num_ghost, r.coeffs is not None) + dataclasses.astuple(r.opts)


class _Active:
    def __init__(self, rid, req, submitted):
        self.rid, self.req, self.submitted = rid, req, submitted
        self.iterations = 0
        self.restarts = 0
        self.x = None  # current iterate on the host between batches (numpy), None on the device


class _Union:
    """The device objects of one union hierarchy and its batch buffers (a cache entry)."""

    def __init__(self, reqs, opts):
        import torch

        depth = max(len(r.levels) for r in reqs)
        levels, offsets = M.union_hierarchy([M.pad_hierarchy(r.levels, depth) for r in reqs])
        coeffs = None
        if reqs[0].coeffs is not None:
            # a padded member's copied levels take the coefficients of its coarsest level
            coeffs = [np.concatenate([r.coeffs[min(k, len(r.coeffs) - 1)] for r in reqs], axis=0)
                      for k in range(len(levels))]
        self.solver = GmgSolver(levels, opts, coeffs)
        self.offsets = offsets[0]
        shape = self.solver.finest.padded_shape(1)
        # every patch range is written before a batch runs, so the buffers need no zero fill
        self.x = Vector(self.solver.finest, data=torch.empty(shape, dtype=torch.float64, device="cuda"))
        self.b = Vector(self.solver.finest, data=torch.empty(shape, dtype=torch.float64, device="cuda"))
        self.keep = [(r.levels, r.coeffs) for r in reqs]  # keeps the key's ids valid
        self.bytes = sum(request_bytes(r.levels, r.opts) for r in reqs)
        self.busy = False


def _union_key(reqs):
    # the class (patch shape, solver options) and the members' meshes and coefficients
    return (_class_key(reqs[0]),) + tuple((id(r.levels), id(r.coeffs)) for r in reqs)


# batch sizes a class's union is rounded up to (ratio <= 1.5), so that the
# unions of a busy class repeat and come from the cache
_BUCKETS = (1, 2, 3, 4, 6, 8, 12, 16, 24, 32, 48, 64, 96, 128, 192, 256)


def _bucket(n, cap):
    for s in _BUCKETS:
        if s >= n:
            return s if s <= cap else n
    return n


class _Batch:
    """One union-hierarchy batch of a class in slot mode (TE_BICGSTAB_SLOTS): slot i
    is solve i of the union.  A slot holds a request or is free (zero right-hand
    side, not iterating); a free slot takes a new request of the same mesh while
    the other slots keep iterating, and a stopped slot is finished on its own."""

    def __init__(self, members, x_parts, un):
        import torch

        self.un = un
        un.busy = True
        self.solver = un.solver
        self.offsets = un.offsets
        self.x, self.b = un.x, un.b
        self.B = len(self.offsets) - 1
        self.slot_key = [(id(lv), id(c)) for lv, c in un.keep]
        self.slots = list(members) + [None] * (self.B - len(members))
        self.base_its = [m.iterations for m in members] + [0] * (self.B - len(members))
        for i, m in enumerate(members):
            self._write(i, m.req.f, x_parts[i])
        if self.B > len(members):
            tail = slice(self.offsets[len(members)], self.offsets[self.B])
            self.b.t[tail].zero_()
            self.x.t[tail].zero_()
        torch.cuda.synchronize()
        offs = (ctypes.c_int * (self.B + 1))(*self.offsets)
        self.h = ctypes.c_void_p()
        o = self.solver.opts
        check(lib().te_bicgstab_batch_create(self.solver.ops[0].h, 1, self.x.ptr, self.b.ptr, self.solver.cycle.h,
                                             float(o.tol), int(o.max_it), int(o.bicgstab_flags) | TE_BICGSTAB_SLOTS,
                                             self.B, offs, ctypes.byref(self.h)))

    def _write(self, i, f, x0):
        import torch

        lo, hi = self.offsets[i], self.offsets[i + 1]
        self.b.t[lo:hi].copy_(torch.as_tensor(f.reshape(self.b.t[lo:hi].shape)))
        if isinstance(x0, torch.Tensor):
            self.x.t[lo:hi].copy_(x0)
        elif x0 is not None:
            self.x.t[lo:hi].copy_(torch.as_tensor(x0.reshape(self.x.t[lo:hi].shape)))
        else:
            self.x.t[lo:hi].zero_()

    @property
    def members(self):
        return [m for m in self.slots if m is not None]

    def free_slot(self, req):
        """A free slot built on req's mesh and coefficients, or -1."""
        key = (id(req.levels), id(req.coeffs))
        for i, m in enumerate(self.slots):
            if m is None and self.slot_key[i] == key:
                return i
        return -1

    def put(self, i, member):
        """Start member in free slot i; the other slots keep iterating."""
        import torch

        self._write(i, member.req.f, member.x)
        torch.cuda.current_stream().synchronize()
        check(lib().te_bicgstab_batch_reset(self.h, int(i)))
        self.slots[i] = member
        self.base_its[i] = member.iterations

    def step(self, k):
        n = ctypes.c_int(0)
        check(lib().te_bicgstab_batch_step(self.h, int(k), ctypes.byref(n)))
        return n.value

    def state(self):
        """Iterations, residuals, statuses and running flags of every slot."""
        B = self.B
        its, res = (ctypes.c_int * B)(), (ctypes.c_double * B)()
        st, run = (ctypes.c_int * B)(), (ctypes.c_int * B)()
        check(lib().te_bicgstab_batch_state(self.h, its, res, st, run))
        return list(its), list(res), list(st), list(run)

    def finish(self, slots):
        """The listed slots stopped: per slot True when its FP64 residual confirms it (x holds
        its result), False when it was restarted from that residual."""
        n = len(slots)
        arr, done = (ctypes.c_int * n)(*slots), (ctypes.c_int * n)()
        check(lib().te_bicgstab_batch_finish_slots(self.h, n, arr, done))
        return [bool(d) for d in done]

    def slice_x(self, i):
        lo, hi = self.offsets[i], self.offsets[i + 1]
        return self.x.t[lo:hi].clone()

    def close(self):
        if self.h:
            lib().te_bicgstab_batch_destroy(self.h)
            self.h = ctypes.c_void_p()
            self.un.busy = False


class Server:
    """Admits, batches, steps and retires requests.

    budget_bytes: device memory the live unions, the requests waiting for a slot
    and the idle cached unions may hold together (request_bytes per slot); a
    request larger than the budget alone is rejected (TE_ERR_BUDGET).
    steps_per_round: BiCGStab iterations a batch runs between scheduling
    decisions; max_batch: most slots per class batch."""

    def __init__(self, budget_bytes=150e9, steps_per_round=2, max_batch=64, cache=True, parallel=True):
        self.budget = int(budget_bytes)
        self.k = int(steps_per_round)
        self.max_batch = int(max_batch)
        self._ids = itertools.count()
        self.queue = []           # (rid, request, submit time, bytes)
        # class key -> {"active": [_Active] in a slot, "waiting": [_Active] without one, "batch": _Batch
        # or None, "bytes": rid -> bytes reserved while waiting, "wait_rounds": rounds a request waited}
        self.classes = {}
        self.results = {}
        self.active_bytes = 0     # live unions (every slot) + admitted requests waiting for a slot
        self.use_cache = bool(cache)
        self.parallel = bool(parallel)
        self.streams = {}         # class key -> its CUDA stream
        self.pool = None
        self.unions = {}          # union key -> _Union, least recently used first
        self.stats = {"rounds": 0, "reforms": 0, "max_batch": 0, "max_active_bytes": 0, "admitted": 0,
                      "union_builds": 0, "union_hits": 0, "union_evictions": 0, "slot_fills": 0}

    def _on_class_stream(self, key):
        """Context that makes the class's stream current (its handles bind to it)."""
        try:
            import torch
        except ImportError:
            return contextlib.nullcontext()
        if not self.parallel or not torch.cuda.is_available():
            return contextlib.nullcontext()
        if key not in self.streams:
            self.streams[key] = torch.cuda.Stream()
        return torch.cuda.stream(self.streams[key])

    # ---- union cache
    def _idle_cache_bytes(self):
        return sum(u.bytes for u in self.unions.values() if not u.busy)

    def _evict(self, need):
        """Drop idle cached unions, least recently used first, until `need` more bytes fit."""
        for key in list(self.unions):
            if self.active_bytes + need + self._idle_cache_bytes() <= self.budget:
                return
            if not self.unions[key].busy:
                del self.unions[key]
                self.stats["union_evictions"] += 1

    # ---- requests
    def submit(self, req: Request) -> int:
        nb = request_bytes(req.levels, req.opts)
        if nb > self.budget:
            from .capi import TE_ERR_BUDGET, TeError
            raise TeError(TE_ERR_BUDGET, f"request needs ~{nb} bytes, over the {self.budget}-byte budget")
        rid = next(self._ids)
        self.queue.append((rid, req, time.perf_counter(), nb))
        return rid

    def idle(self):
        return not self.queue and all(not c["active"] and not c["waiting"] for c in self.classes.values())

    # ---- scheduling
    def _free_slots(self, cls, req):
        """Free slots of req's mesh in the class's batch that no earlier waiting request claims."""
        b = cls["batch"]
        if b is None:
            return 0
        key = (id(req.levels), id(req.coeffs))
        free = sum(1 for i, m in enumerate(b.slots) if m is None and b.slot_key[i] == key)
        return free - sum(1 for a in cls["waiting"] if (id(a.req.levels), id(a.req.coeffs)) == key)

    def _admit(self):
        """Queue -> the class's waiting list while the budget has room.  A request that will
        take a free slot of its mesh needs no new memory; any other reserves its own bytes
        until a batch holds it."""
        keep = []
        for rid, req, t0, nb in self.queue:
            key = _class_key(req)
            cls = self.classes.setdefault(key, {"active": [], "waiting": [], "batch": None, "bytes": {},
                                                "wait_rounds": 0})
            need = 0 if self._free_slots(cls, req) > 0 else nb
            if need and self.active_bytes + need + self._idle_cache_bytes() > self.budget:
                self._evict(need)
            if self.active_bytes + need + self._idle_cache_bytes() <= self.budget and \
                    len(cls["active"]) + len(cls["waiting"]) < self.max_batch:
                a = _Active(rid, req, t0)
                a.x = req.u0
                cls["waiting"].append(a)
                cls["bytes"][rid] = need
                self.active_bytes += need
                self.stats["admitted"] += 1
            else:
                keep.append((rid, req, t0, nb))
        self.queue = keep
        self.stats["max_active_bytes"] = max(self.stats["max_active_bytes"], self.active_bytes)

    def _retire(self, a, u, its, res, st):
        self.results[a.rid] = Result(u=u, iterations=its, residual=res, status=st,
                                     latency_s=time.perf_counter() - a.submitted, restarts=a.restarts)

    def _form(self, cls):
        """A new batch of the class's waiting requests (continuing ones carry their iterate),
        rounded up to a bucket size with free slots of the last request's mesh when the
        budget has room.  The union's bytes replace the requests' reservations."""
        members = cls["waiting"]
        self.active_bytes -= sum(cls["bytes"].pop(m.rid, 0) for m in members)
        last = members[-1].req
        extra = _bucket(len(members), self.max_batch) - len(members)
        for pad in ((extra, 0) if extra else (0,)):
            reqs = [m.req for m in members] + [Request(last.levels, None, last.opts, last.coeffs)] * pad
            key = _union_key(reqs)
            un = self.unions.pop(key, None)  # out of the idle cache while it is weighed
            need = un.bytes if un is not None else sum(request_bytes(r.levels, r.opts) for r in reqs)
            if self.active_bytes + need + self._idle_cache_bytes() > self.budget:
                self._evict(need)
            if pad == 0 or self.active_bytes + need + self._idle_cache_bytes() <= self.budget:
                break
            if un is not None:
                self.unions[key] = un
        if un is None:
            un = _Union(reqs, members[0].req.opts)
            self.stats["union_builds"] += 1
        else:
            self.stats["union_hits"] += 1
        if self.use_cache:
            self.unions[key] = un  # most recently used last
        b = _Batch(members, [m.x for m in members], un)
        self.active_bytes += un.bytes
        self._evict(0)  # the idle cache shrinks to what the budget leaves
        cls["batch"], cls["active"], cls["waiting"], cls["wait_rounds"] = b, list(members), [], 0
        self.stats["reforms"] += 1
        self.stats["max_batch"] = max(self.stats["max_batch"], b.B)
        self.stats["max_active_bytes"] = max(self.stats["max_active_bytes"], self.active_bytes)

    def _close(self, cls):
        """Release the class's batch: its union becomes an idle cache entry."""
        b = cls["batch"]
        b.close()
        self.active_bytes -= b.un.bytes
        cls["batch"] = None

    def _place(self, cls):
        """Waiting requests into free slots of their mesh; a new batch when the class has
        none, or when requests have waited without a slot (the batch then grows)."""
        b = cls["batch"]
        if b is None:
            if cls["waiting"]:
                self._form(cls)
            return
        still = []
        for a in cls["waiting"]:
            i = b.free_slot(a.req)
            if i < 0:
                still.append(a)
                continue
            b.put(i, a)
            self.active_bytes -= cls["bytes"].pop(a.rid, 0)
            cls["active"].append(a)
            self.stats["slot_fills"] += 1
        cls["waiting"] = still
        if not still:
            cls["wait_rounds"] = 0
            return
        cls["wait_rounds"] += 1
        if cls["active"] and 2 * len(still) < b.B and cls["wait_rounds"] < 2:
            return  # let a few more arrivals gather before the batch is re-formed
        # re-form: continuing requests carry their iterates (their Krylov spaces restart)
        check(lib().te_bicgstab_batch_sync_x(b.h))
        its, _, _, _ = b.state()
        carried = []
        for i, m in enumerate(b.slots):
            if m is not None:
                m.x = b.slice_x(i)
                m.iterations = b.base_its[i] + its[i]
                m.restarts += 1
                carried.append(m)
        self._close(cls)
        for m in carried:  # reserved again until the new union holds them
            cls["bytes"][m.rid] = request_bytes(m.req.levels, m.req.opts)
            self.active_bytes += cls["bytes"][m.rid]
        cls["waiting"] = carried + still
        self._form(cls)

    def _harvest(self, cls):
        """Finish the stopped slots: retire confirmed requests and free their slots; a batch
        with no requests left is closed."""
        b = cls["batch"]
        if b is None:
            return
        _, _, _, run = b.state()
        stopped = [i for i, m in enumerate(b.slots) if m is not None and not run[i]]
        if stopped:
            done = b.finish(stopped)
            its, res, st, _ = b.state()
            for i, ok in zip(stopped, done):
                if not ok:
                    continue  # restarted from its true residual
                m = b.slots[i]
                self._retire(m, b.slice_x(i).cpu().numpy(), b.base_its[i] + its[i], res[i], st[i])
                b.slots[i] = None
                cls["active"].remove(m)
        if not cls["active"] and not cls["waiting"]:
            self._close(cls)

    def step(self):
        """One scheduling round: admit, place waiting requests into free slots (or
        re-form), advance every batch by up to steps_per_round iterations, finish
        stopped slots and retire their requests."""
        self.stats["rounds"] += 1
        self._admit()
        for key, cls in self.classes.items():
            with self._on_class_stream(key):
                self._place(cls)
        running = [cls["batch"] for cls in self.classes.values() if cls["batch"] is not None]
        if self.parallel and len(running) > 1:
            if self.pool is None:
                self.pool = ThreadPoolExecutor(max_workers=8)
            list(self.pool.map(lambda b: b.step(self.k), running))
        else:
            for b in running:
                b.step(self.k)
        for key, cls in self.classes.items():
            with self._on_class_stream(key):
                self._harvest(cls)
        return not self.idle()

    def run(self, max_rounds=10**9):
        r = 0
        while not self.idle() and r < max_rounds:
            self.step()
            r += 1
        return self.results

    def close(self):
        """Destroy the running batches, drop the cached unions (their device memory goes
        with them) and stop the stepping threads.  Requests still queued or running are
        dropped without a result."""
        for cls in self.classes.values():
            if cls["batch"] is not None:
                self._close(cls)
            cls["active"], cls["waiting"] = [], []
            cls["bytes"].clear()
        self.unions.clear()
        self.queue = []
        self.active_bytes = 0
        if self.pool is not None:
            self.pool.shutdown(wait=True)
            self.pool = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
        return False


class NativeServer:
    """The C ABI's serving loop (te_serve_*, include/te_gpu.h): continuous batching of the
    same kind as Server, run by the library itself for callers outside Python.  Supports
    Poisson requests with V-cycle-preconditioned BiCGStab (GmgOptions with cycle_type "V",
    krylov "bicgstab", no coefficients, no boundary-ghost extrapolation)."""

    def __init__(self, budget_bytes=150e9, steps_per_round=2, max_batch=64):
        from .capi import TeServeOpts

        o = TeServeOpts(float(budget_bytes), int(steps_per_round), int(max_batch))
        h = ctypes.c_void_p()
        check(lib().te_serve_create(ctypes.byref(o), ctypes.byref(h)))
        self.h = h
        self._f = {}

    @staticmethod
    def solve_opts(o: GmgOptions):
        from .capi import TeSolveOpts

        if o.cycle_type != "V" or o.krylov != "bicgstab" or o.extrapolate_boundary_ghosts:
            raise ValueError("the native server runs V-cycle-preconditioned BiCGStab without extrapolation")
        return TeSolveOpts(o.scheme, o.fill_type, o.smoother, o.inner_tol, o.inner_max_it,
                           int(o.inner_continue_on_breakdown), o.pre_sweeps, o.post_sweeps, o.coarse_sweeps,
                           o.tol, o.max_it, o.cycle_dtype, o.bicgstab_flags, o.tc_precision)

    def submit(self, levels, f, opts: GmgOptions = GmgOptions()) -> int:
        from .capi import TeLevelDesc

        descs = (TeLevelDesc * len(levels))(*[lv.to_desc() for lv in levels])
        so = self.solve_opts(opts)
        fa = np.ascontiguousarray(f, dtype=np.float64)
        rid = ctypes.c_longlong()
        check(lib().te_serve_submit(self.h, descs, len(levels), ctypes.byref(so),
                                    fa.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ctypes.byref(rid)))
        self._f[rid.value] = fa.shape
        return rid.value

    def step(self) -> int:
        n = ctypes.c_int()
        check(lib().te_serve_step(self.h, ctypes.byref(n)))
        return n.value

    def poll(self, rid):
        """The request's Result once it has finished (returned once), else None."""
        from .capi import TE_PENDING, TeServeResult

        shape = self._f[rid]
        u = np.empty(shape, dtype=np.float64)
        r = TeServeResult()
        rc = lib().te_serve_poll(self.h, rid, u.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ctypes.byref(r))
        if rc == TE_PENDING:
            return None
        check(rc)
        del self._f[rid]
        return Result(u, r.iterations, r.residual, r.status, r.latency_s, r.restarts)

    def stats(self) -> dict:
        from .capi import TeServeCounters

        c = TeServeCounters()
        check(lib().te_serve_stats(self.h, ctypes.byref(c)))
        return {name: getattr(c, name) for name, _ in TeServeCounters._fields_}

    def run(self, ids, max_rounds=10**9):
        """Step until every listed request has finished; {id: Result}."""
        out, r = {}, 0
        while len(out) < len(ids) and r < max_rounds:
            self.step()
            r += 1
            for i in ids:
                if i not in out:
                    res = self.poll(i)
                    if res is not None:
                        out[i] = res
        return out

    def close(self):
        if self.h:
            check(lib().te_serve_destroy(self.h))
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
        return False
