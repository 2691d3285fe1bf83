"""Continuous batching of independent Poisson solves on one GPU.

A request is one GMG-preconditioned BiCGStab solve on its own mesh
hierarchy.  Requests whose hierarchies share patch shape, depth and solver
options form a class; the active requests of a class are packed into one
union hierarchy (mesh.union_hierarchy), so every per-level kernel of the
V-cycle and every Krylov kernel runs over all of them in one launch (one CUDA
graph replay per iteration).  The server steps each class's batch a few
iterations at a time (te_bicgstab_batch_step).  Between steps it

  * admits queued requests while the estimated device memory of all active
    requests stays within the budget,
  * retires requests that have finished (their result is copied out and
    their memory is released),
  * re-forms a class's batch when its membership changes: the new union
    hierarchy is built, every continuing request's current iterate and
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
from .capi import check, lib
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
    """Requests batch together when their patch shape, depth, coefficient use and every
    solver option agree."""
    lv = r.levels[0]
    return (lv.dim, tuple(lv.ns), lv.num_ghost, len(r.levels), r.coeffs is not None) + dataclasses.astuple(r.opts)


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

        levels, offsets = M.union_hierarchy([r.levels for r in reqs])
        coeffs = None
        if reqs[0].coeffs is not None:
            coeffs = [np.concatenate([r.coeffs[k] for r in reqs], axis=0) for k in range(len(levels))]
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
    # the class (patch shape, depth, solver options) and the members' meshes and coefficients
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
    """One union-hierarchy batch of a class and its stepping BiCGStab run.  The
    union may hold phantom slots after the members (zero right-hand side: their
    solves are finished at the start and the Krylov kernels skip them)."""

    def __init__(self, members, x_parts, un, phantom_bytes=0):
        import torch

        self.members = list(members)  # this batch's members, in patch order
        self.un = un
        un.busy = True
        self.solver = un.solver
        self.offsets = un.offsets
        self.x, self.b = un.x, un.b
        self.phantom_bytes = phantom_bytes
        for i, m in enumerate(members):
            lo, hi = self.offsets[i], self.offsets[i + 1]
            self.b.t[lo:hi].copy_(torch.as_tensor(m.req.f.reshape(self.b.t[lo:hi].shape)), non_blocking=False)
            src = x_parts[i]
            if isinstance(src, torch.Tensor):
                self.x.t[lo:hi].copy_(src)
            elif src is not None:
                self.x.t[lo:hi].copy_(torch.as_tensor(src.reshape(self.x.t[lo:hi].shape)))
            else:
                self.x.t[lo:hi].zero_()
        B = len(self.offsets) - 1  # members, then phantom slots
        if B > len(members):
            tail = slice(self.offsets[len(members)], self.offsets[B])
            self.b.t[tail].zero_()
            self.x.t[tail].zero_()
        torch.cuda.synchronize()
        offs = (ctypes.c_int * (B + 1))(*self.offsets)
        self.h = ctypes.c_void_p()
        o = self.solver.opts
        check(lib().te_bicgstab_batch_create(self.solver.ops[0].h, 1, self.x.ptr, self.b.ptr, self.solver.cycle.h,
                                             float(o.tol), int(o.max_it), int(o.bicgstab_flags), B, offs,
                                             ctypes.byref(self.h)))
        self.base_its = [m.iterations for m in members]

    def step(self, k):
        n = ctypes.c_int(0)
        check(lib().te_bicgstab_batch_step(self.h, int(k), ctypes.byref(n)))
        return n.value

    def state(self):
        """Iterations, residuals, statuses and running flags of the members (phantoms left out)."""
        B = len(self.offsets) - 1
        its, res = (ctypes.c_int * B)(), (ctypes.c_double * B)()
        st, run = (ctypes.c_int * B)(), (ctypes.c_int * B)()
        check(lib().te_bicgstab_batch_state(self.h, its, res, st, run))
        n = len(self.members)
        return list(its)[:n], list(res)[:n], list(st)[:n], list(run)[:n]

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

    budget_bytes: device memory the active requests may hold (request_bytes);
    a request larger than the budget alone is rejected (TE_ERR_BUDGET).
    steps_per_round: BiCGStab iterations a batch runs between scheduling
    decisions; max_batch: most requests per class batch."""

    def __init__(self, budget_bytes=150e9, steps_per_round=2, max_batch=64, cache=True, parallel=True):
        self.budget = int(budget_bytes)
        self.k = int(steps_per_round)
        self.max_batch = int(max_batch)
        self._ids = itertools.count()
        self.queue = []           # (rid, request, submit time, bytes)
        self.classes = {}         # key -> {"active": [_Active], "batch": _Batch or None, "dirty": bool}
        self.results = {}
        self.active_bytes = 0
        self.use_cache = bool(cache)
        self.parallel = bool(parallel)
        self.streams = {}         # class key -> its CUDA stream
        self.pool = None
        self.unions = {}          # union key -> _Union, least recently used first
        self.stats = {"rounds": 0, "reforms": 0, "max_batch": 0, "max_active_bytes": 0, "admitted": 0,
                      "union_builds": 0, "union_hits": 0, "union_evictions": 0}

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

    def _union(self, reqs, opts):
        key = _union_key(reqs)
        un = self.unions.pop(key, None)
        if un is None:
            un = _Union(reqs, opts)
            self.stats["union_builds"] += 1
        else:
            self.stats["union_hits"] += 1
        if self.use_cache:
            self.unions[key] = un  # most recently used last
        return un

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
        return not self.queue and all(not c["active"] for c in self.classes.values())

    # ---- scheduling
    def _admit(self):
        keep = []
        for rid, req, t0, nb in self.queue:
            key = _class_key(req)
            cls = self.classes.setdefault(key, {"active": [], "batch": None, "dirty": False, "bytes": {}})
            if self.active_bytes + nb > self.budget:
                self._evict(nb)
            if self.active_bytes + nb <= self.budget and len(cls["active"]) < self.max_batch:
                a = _Active(rid, req, t0)
                a.x = req.u0
                cls["active"].append(a)
                cls["bytes"][rid] = nb
                cls["waiting"] = cls.get("waiting", 0) + 1
                if cls["batch"] is None:
                    cls["dirty"] = True
                self.active_bytes += nb
                self.stats["admitted"] += 1
            else:
                keep.append((rid, req, t0, nb))
        self.queue = keep
        self.stats["max_active_bytes"] = max(self.stats["max_active_bytes"], self.active_bytes)
        self._evict(0)

    def _close(self, b):
        b.close()
        self.active_bytes -= b.phantom_bytes
        b.phantom_bytes = 0

    def _retire(self, cls, a, u, its, res, st):
        self.results[a.rid] = Result(u=u, iterations=its, residual=res, status=st,
                                     latency_s=time.perf_counter() - a.submitted, restarts=a.restarts)
        self.active_bytes -= cls["bytes"].pop(a.rid)

    def _reform(self, key, cls):
        old = cls["batch"]
        if old is not None:
            # carry every continuing request's iterate (device copy) into the new batch
            check(lib().te_bicgstab_batch_sync_x(old.h))
            its, _, _, _ = old.state()
            pos = {m.rid: i for i, m in enumerate(old.members)}
            for m in cls["active"]:
                if m.rid in pos:
                    i = pos[m.rid]
                    m.x = old.slice_x(i)
                    m.iterations = old.base_its[i] + its[i]
                    m.restarts += 1
            self._close(old)
            cls["batch"] = None
        cls["dirty"] = False
        cls["waiting"] = 0
        cls["wait_rounds"] = 0
        while cls["active"]:
            members = cls["active"]
            reqs = [m.req for m in members]
            # phantom slots round the batch up to a bucket size, when the budget has room for them
            last = members[-1].req
            extra = _bucket(len(members), self.max_batch) - len(members)
            pbytes = extra * request_bytes(last.levels, last.opts)
            if extra and self.active_bytes + self._idle_cache_bytes() + pbytes > self.budget:
                self._evict(pbytes)
            if extra and self.active_bytes + self._idle_cache_bytes() + pbytes > self.budget:
                extra, pbytes = 0, 0
            reqs += [Request(last.levels, None, last.opts, last.coeffs)] * extra
            self.active_bytes += pbytes
            b = _Batch(members, [m.x for m in members], self._union(reqs, members[0].req.opts), pbytes)
            self.stats["reforms"] += 1
            self.stats["max_batch"] = max(self.stats["max_batch"], len(members))
            its, res, st, run = b.state()
            # requests already finished when the batch starts (their FP64 residual is within tolerance,
            # or they broke down or ran out of iterations) leave now; the rest run without them
            fin = [i for i in range(len(members)) if not run[i]]
            if not fin or len(fin) == len(members):
                cls["batch"] = b
                if len(fin) == len(members):
                    self._collect(cls)
                return
            for i in fin:
                self._retire(cls, members[i], b.slice_x(i).cpu().numpy(), b.base_its[i] + its[i], res[i], st[i])
            gone = {members[i].rid for i in fin}
            cls["active"] = [m for m in members if m.rid not in gone]
            for m in cls["active"]:
                m.x = b.slice_x(members.index(m))
            self._close(b)

    def _collect(self, cls):
        """Retire every request of the class's batch once the whole batch has finished."""
        b = cls["batch"]
        if b.step(0) != 0:
            return
        its, res, st, run = b.state()
        for i, m in enumerate(b.members):
            self._retire(cls, m, b.slice_x(i).cpu().numpy(), b.base_its[i] + its[i], res[i], st[i])
        gone = {m.rid for m in b.members}
        cls["active"] = [m for m in cls["active"] if m.rid not in gone]
        self._close(b)
        cls["batch"] = None
        if cls["active"]:
            cls["dirty"] = True

    def step(self):
        """One scheduling round: admit, re-form changed batches, advance every batch
        by up to steps_per_round iterations, retire finished requests."""
        self.stats["rounds"] += 1
        self._admit()
        for key, cls in self.classes.items():
            if cls["dirty"]:
                with self._on_class_stream(key):
                    self._reform(key, cls)
        running = [cls["batch"] for cls in self.classes.values() if cls["batch"] is not None]
        if self.parallel and len(running) > 1:
            if self.pool is None:
                self.pool = ThreadPoolExecutor(max_workers=8)
            list(self.pool.map(lambda b: b.step(self.k), running))
        else:
            for b in running:
                b.step(self.k)
        for key, cls in self.classes.items():
            b = cls["batch"]
            if b is None:
                continue
            its, res, st, run = b.state()
            stopped = len(run) - sum(run)
            waiting = cls.get("waiting", 0)
            if waiting:
                cls["wait_rounds"] = cls.get("wait_rounds", 0) + 1
            if stopped == len(run):
                with self._on_class_stream(key):
                    self._collect(cls)
            elif (stopped and (self.queue or waiting or 4 * stopped >= len(run))) or \
                    (waiting and (2 * waiting >= len(run) or cls.get("wait_rounds", 0) >= 3)):
                # retire stopped requests and let admitted ones join: re-form at the next round.
                # Admitted requests join a running batch once they are half its size or have
                # waited three rounds, so that arrivals do not rebuild the batch one by one.
                cls["dirty"] = True
        return not self.idle()

    def run(self, max_rounds=10**9):
        r = 0
        while not self.idle() and r < max_rounds:
            self.step()
            r += 1
        return self.results
