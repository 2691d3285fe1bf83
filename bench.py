"""Benchmark: solves/s and latency of the adaptive 2D Poisson GMG solve on GB300.

Workload (one "step" = one complete solve to a 1e-10 relative FP64 residual):
  2D Poisson -Lap(u) = f on the unit square, quadtree refined from level 3 to
  level 7 where a leaf box meets the circle r = 0.3 about (0.5, 0.5), 2:1
  balanced (1444 leaves, 8 GMG levels), 32x32-cell patches, u = exp(xy),
  Dirichlet data from u; BiQuadratic ghost filling, DFT patch smoother,
  V(1,1) cycle, BiCGStab outer solver.
  value: mixed precision (FP32 V-cycle with 3xTF32 tensor-core transforms,
         float-float BiCGStab, FP64 initial and final residuals), served as
         a batch of --batch independent solves per step (one right-hand side
         each), inputs resident in HBM.  Single-solve latency and the plain
         FP64 drop-in (one solve at a time) are reported beside it.
  e2e:   the same solve through the C ABI from pinned host buffers: f copied
         host->device and u device->host inside the timed region.
  L2: flushed (256 MiB write) between timed steps, outside the step timing.

--impl reference times the CPU restatement of the reference's algorithm
(oracle/, FP64, same workload) on the host cores, one solve per process.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "solves/s and p99 latency: mixed-prec served vs plain FP64 GMG, 1e-10 resid"
WORKLOAD = ("2D adaptive Poisson, circle r=0.3 quadtree L3-7 2:1 balanced, 1444 patches 32x32, "
            "u=exp(xy) Dirichlet, BiQuadratic, DFT smoother, V(1,1), BiCGStab to 1e-10")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--fp64-steps", type=int, default=5)
    ap.add_argument("--batch", type=int, default=16, help="solves served per step")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--stream", type=int, default=40,
                    help="requests in the serving-stream measurement (0: skip)")
    ap.add_argument("--stream-rate", type=float, default=50.0, help="Poisson arrival rate, requests/s")
    ap.add_argument("--c5-rates", default="10,40,160", help="config-5 stream: arrival rates swept, requests/s")
    ap.add_argument("--c5-requests", type=int, default=60, help="config-5 stream: requests per rate (0: skip)")
    ap.add_argument("--no-extra", action="store_true", help="skip the config-3 and config-4 measurements")
    ap.add_argument("--kernels", action="store_true",
                    help="only time the drop-in level kernels against HBM (one JSON line)")
    ap.add_argument("--only-mixed", action="store_true",
                    help="time the mixed-precision solves only (for profiler captures)")
    return ap.parse_args()


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# ---------------------------------------------------------------------------
# CPU legs (the oracle is test infrastructure: used here only as the baseline)
# ---------------------------------------------------------------------------
def _cpu_solve_worker(q, ready=None, go=None):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    from thunderegg_gb300 import problems as PB

    levels, f, _ = PB.config2()
    cfg = orc.gmg_config(scheme=1, smoother=0, tol=1e-10)
    O = orc.Oracle("teo")
    if ready is not None:  # the mesh is built: wait until every worker is, then solve together
        ready.put(1)
        go.wait()
    t = time.perf_counter()
    u, its, res, rc = O.solve(levels, f, cfg)
    q.put((time.perf_counter() - t, its, rc))


# FP64 oracle solutions of the benchmark problems, for the error of every GPU result
# against an FP64 oracle solve.  Each job runs in its own spawned process, started
# before the GPU work and collected after it; the solution goes through a temporary
# .npy file (config 3's is 191 MB).
ORACLE_JOBS = ("config1", "config2", "config3", "config4_0", "config4_1", "config4_2", "config4_3")
CONFIG4_CHECKED = 4  # config-4 solves compared with the oracle (the first ones of the 32)


def _oracle_ref_worker(name, outdir):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np

    import oracle as orc
    from thunderegg_gb300 import problems as PB

    O = orc.Oracle("teo")
    coeffs = None
    if name == "config1":
        # the plain method: BiCGStab patch smoother (inner 1e-12 / 1000 / continue on breakdown),
        # the reference's BiCGStab update rule; the GPU config-1 drop-in runs the same rule
        levels, f, _ = PB.config1()
        cfg = orc.gmg_config(scheme=0, smoother=1, inner_tol=1e-12, inner_max_it=1000, tol=1e-10)
    elif name == "config2":
        levels, f, _ = PB.config2()
        cfg = orc.gmg_config(scheme=1, smoother=0, tol=1e-10, precond_exit=1)
    elif name == "config3":
        levels, f, _ = PB.config3()
        cfg = orc.gmg_config(scheme=2, smoother=0, tol=1e-10, precond_exit=1)
    else:
        k = int(name.split("_")[1])
        levels, f, coeffs = PB.config4(num_solves=k + 1)[k]
        cfg = orc.gmg_config(scheme=1, smoother=1, op_kind=1, inner_tol=1e-12, tol=1e-10, precond_exit=1)
    t = time.perf_counter()
    u, its, res, rc = O.solve(levels, f, cfg, coeffs=coeffs)
    sec = time.perf_counter() - t
    path = os.path.join(outdir, f"{name}.npy")
    np.save(path, u)
    return name, path, its, res, rc, sec


class OracleRefs:
    """The oracle's FP64 solutions, computed in spawned processes beside the GPU work."""

    def __init__(self, names=ORACLE_JOBS):
        import multiprocessing as mp

        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as orc

        orc.build()
        self.dir = tempfile.mkdtemp(prefix="te_oracle_refs_")
        self.pool = mp.get_context("spawn").Pool(min(len(names), max(1, (os.cpu_count() or 2) // 2)))
        self.jobs = {n: self.pool.apply_async(_oracle_ref_worker, (n, self.dir)) for n in names}
        self.info = {}

    def get(self, name, timeout=900):
        import numpy as np

        n, path, its, res, rc, sec = self.jobs[name].get(timeout=timeout)
        self.info[name] = {"outer_iterations": its, "final_rel_residual": res, "status": rc, "cpu_seconds": sec}
        return np.load(path)

    def close(self):
        import shutil

        self.pool.terminate()
        shutil.rmtree(self.dir, ignore_errors=True)


def err_vs(u, ref, lv):
    """max |u - ref| / max |ref| over the interior cells of the finest level."""
    import numpy as np

    from thunderegg_gb300 import problems as PB

    a = PB.interior_view(lv, np.asarray(u))
    b = PB.interior_view(lv, np.asarray(ref))
    return float(np.abs(a - b).max() / np.abs(b).max())


def cpu_solves(nproc):
    """Run nproc independent solves in parallel processes; returns (wall, [times]).  The wall
    runs from the moment every process has built its mesh to the last solution: process start-up
    and the Python mesh build are outside it."""
    import multiprocessing as mp

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc

    orc.build()
    ctx = mp.get_context("spawn")
    q, ready, go = ctx.Queue(), ctx.Queue(), ctx.Event()
    procs = [ctx.Process(target=_cpu_solve_worker, args=(q, ready, go)) for _ in range(nproc)]
    for p in procs:
        p.start()
    for _ in procs:
        ready.get()
    t = time.perf_counter()
    go.set()
    out = [q.get() for _ in procs]
    wall = time.perf_counter() - t
    for p in procs:
        p.join()
    return wall, out


def run_reference(args):
    rank, world, local = dist_info()
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    steps, warm = max(1, args.steps), max(0, args.warmup)
    # bounded: each step is one round of `cores` parallel solves (about 5 s on 16 Grace cores);
    # at most 20 timed rounds and 3 warm-up rounds, so a run ends within two minutes
    rounds, warm = min(steps, 20), min(warm, 3)
    for _ in range(warm):
        cpu_solves(cores)
    walls, its = [], None
    for _ in range(rounds):
        w, out = cpu_solves(cores)
        walls.append(w)
        its = out[0][1]
    total = sum(walls)
    value = rounds * cores / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": args.gpus,
        "steps": rounds, "warmup": warm, "ms_per_step": 1000 * total / rounds,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": {"workload": WORKLOAD, "outer_iterations": its},
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": cores, "kind": "port",
                         "sample": f"{rounds} rounds of {cores} independent full solves, one process per core"},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------
class Clocks:
    def __init__(self, index):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={index}", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except FileNotFoundError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait()
        self.f.seek(0)
        out = clock_summary(self.f.read())
        os.unlink(self.f.name)
        return out


def clock_summary(text):
    """Median SM clock, maximum SM clock and the throttle reasons seen in nvidia-smi's CSV samples
    (index, clocks.sm, clocks.max.sm, power.draw, active reasons, hw_slowdown, hw_thermal_slowdown,
    sw_thermal_slowdown, sw_power_cap); lines that do not parse are skipped."""
    sm, mx, reasons = [], None, set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    for line in text.splitlines():
        parts = [x.strip() for x in line.split(",")]
        if len(parts) < 9:
            continue
        try:
            sm.append(float(parts[1]))
            mx = float(parts[2])
        except ValueError:
            continue
        for n, v in zip(names, parts[5:9]):
            if v.lower() == "active":
                reasons.add(n)
    return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
            "samples": len(sm)}


def _phase_bytes(name, levels, dtype_bytes):
    """Algorithmic bytes of one launch of a fused V-cycle phase on level k:
    interior cells only, each value read or written once; ghost gathers count
    2D/n reads per cell (one face row of neighbour values per patch side)."""
    k = int(name.split()[0][1:])
    lv = levels[k]
    cells = lv.num_cells
    D, n = lv.dim, lv.ns[0]
    w = dtype_bytes
    wf = wo = w  # the mixed-precision solve runs the cycle FP32 in and out on every level
    ghost = w * 2 * D / n
    if "pre-smooth" in name:
        return cells * (wf + w)
    if "restrict" in name:
        return cells * (w + wf + ghost + w / (1 << D))
    face = 2 * D / n  # side-face cells per cell
    if "post-corrections" in name:
        # corrections written; own two boundary layers, the neighbours' two face layers and the
        # coarse values under them read (FP32)
        return cells * 4 * face * (1 + 2 + 2 + 1)
    if name.endswith("post-smooth") and "interpolate" not in name:
        return cells * (wf + 4 * face + wo)  # tensor-core solve: f and the corrections in, u out
    return cells * (w + w / (1 << D) + wf + ghost + wo)


def _ghost_bytes(lv, w):
    """Compulsory DRAM bytes of one side-ghost fill of a level at 32-byte sector
    granularity: for every patch side with a neighbour, the ghost face is
    written and one face of neighbour values is read.  A face across axis 0 is
    a column (one sector per cell); the other faces are rows of n cells."""
    import numpy as np

    D, n = lv.dim, lv.ns[0]
    side0 = 4 if D == 2 else 20
    per = n ** (D - 1)
    total = 0
    for s in range(2 * D):
        sides = int(np.count_nonzero(lv.nbr_type[:, side0 + s] >= 0))
        total += sides * 2 * per * (32 if s // 2 == 0 else w)
    return total


def level_kernel_rooflines(te, solver, hbm, reps=15, warm=3):
    """Device time of each drop-in level kernel (one ABI call on the solver's
    finest level, or between its two finest levels), L2 flushed before every
    call, median over `reps`, against the kernel's algorithmic bytes:
      ghost_fill       sector-granular ghost faces written + neighbour faces read
      operator_apply   ghost fill + u read + f written (padded: f's ghosts are set)
      restrict         fine interior read + coarse padded written
      interpolate      coarse interior read + fine interior read and written
      vec_add_scaled   x, a read, x written (interior)
      vec_dot          x, y read (interior); the call returns the value to the host"""
    import numpy as np
    import torch

    lib = te.capi.lib()
    f0, f1 = solver.levels[0], solver.levels[1]
    d0, d1 = solver.domains[0], solver.domains[1]
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    rng = np.random.default_rng(7)
    out = []
    for dt, w in ((te.TE_F64, 8), (te.TE_F32, 4)):
        u = te.Vector.from_numpy(d0, rng.standard_normal(f0.padded_shape(1)), dtype=dt)
        f = te.Vector(d0, 1, dt)
        a = te.Vector.from_numpy(d0, rng.standard_normal(f0.padded_shape(1)), dtype=dt)
        c = te.Vector.from_numpy(d1, rng.standard_normal(f1.padded_shape(1)), dtype=dt)
        ci = te.Vector(d1, 1, dt)
        i0 = f0.num_cells * w
        i1 = f1.num_cells * w
        p0 = f0.num_patches * f0.patch_stride(1) * w
        p1 = f1.num_patches * f1.patch_stride(1) * w
        g = _ghost_bytes(f0, w)
        rs, ip = solver.restrictors[0], solver.interpolators[1]
        calls = [
            ("ghost_fill", g, lambda: solver.fillers[0].fillGhost(u)),
            ("operator_apply", g + 2 * p0, lambda: solver.ops[0].apply(u, f)),
            ("restrict", i0 + p1, lambda: te.capi.check(lib.te_restrict(rs.h, 1, dt, u.ptr, ci.ptr))),
            ("interpolate", i1 + 2 * i0, lambda: ip.interpolate(c, u)),
            ("vec_add_scaled", 3 * i0, lambda: u.addScaled(1e-3, a)),
            ("vec_dot", 2 * i0, lambda: u.dot(a)),
        ]
        for name, nbytes, fn in calls:
            times = []
            for i in range(warm + reps):
                flush.fill_(i & 0xFF)
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                fn()
                e1.record(stream)
                torch.cuda.synchronize()
                if i >= warm:
                    times.append(e0.elapsed_time(e1) / 1000.0)
            t = statistics.median(times)
            gbs = nbytes / t / 1e9
            out.append({"kernel": name, "dtype": "f64" if w == 8 else "f32", "us": round(1e6 * t, 2),
                        "algorithmic_bytes": int(nbytes), "achieved_gbs": round(gbs, 1),
                        "frac": round(gbs / hbm, 3)})
    return {"level": f"{f0.num_patches} patches of {f0.ns[0]}^{f0.dim} (+ {f1.num_patches} coarse)",
            "peak_gbs": hbm, "l2": "flushed before every call", "kernels": out}


def fp64_krylov_measure(te, blevels, offsets, fB, reps=3):
    """The served config-2 batch with the outer BiCGStab in FP64 (TE_BICGSTAB_FP64_OUTER: FP64
    vectors, inner products and updates) around the same FP32 V-cycle, beside the default
    float-float loop: what keeping the Krylov arithmetic in FP64 costs on GB300."""
    import torch

    from thunderegg_gb300.gmg import GmgOptions, GmgSolver

    s = GmgSolver(blevels, GmgOptions(scheme=1, smoother=0, tol=1e-10, cycle_dtype=te.TE_F32,
                                      bicgstab_flags=1 | te.capi.TE_BICGSTAB_FP64_OUTER))
    u = te.Vector(s.finest)
    stream = torch.cuda.current_stream()
    times, its = [], None
    for r in range(reps + 1):
        u.t.zero_()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        its, res, st = s.solve_batched(fB, u, offsets[0])
        e1.record(stream)
        torch.cuda.synchronize()
        if r > 0:
            times.append(e0.elapsed_time(e1) / 1000.0)
    B = len(offsets[0]) - 1
    t = statistics.median(times)
    out = {"ms_per_batch": 1000 * t, "solves_per_s": B / t, "outer_iterations": max(its),
           "max_final_rel_residual": max(res),
           "form": "FP32 V-cycle (3xTF32 transforms) inside an FP64 BiCGStab (TE_BICGSTAB_FP64_OUTER)"}
    del s, u
    return out


def batch_scaling_measure(te, sizes=(1, 4, 16, 32, 64), reps=3):
    """Served config-2 batches of B solves (union hierarchies, the benchmark RHS plus
    seeded sine modes): solves/s and batch latency per B, CUDA events around each
    solve_batched call (median of `reps` after one warm-up), L2 flushed between."""
    import numpy as np
    import torch

    from thunderegg_gb300 import mesh as M
    from thunderegg_gb300 import problems as PB
    from thunderegg_gb300.gmg import GmgOptions, GmgSolver

    levels, f_np, _ = PB.config2()
    rng = np.random.default_rng(77)
    opts = GmgOptions(scheme=1, smoother=0, tol=1e-10, cycle_dtype=te.TE_F32, bicgstab_flags=1)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    out = {}
    for B in sizes:
        blevels, offsets = M.union_hierarchy([levels] * B)
        s = GmgSolver(blevels, opts)
        fs = np.concatenate([f_np + 0.1 * PB.sine_modes_rhs(levels[0], rng) for _ in range(B)], axis=0)
        fv, uv = te.Vector.from_numpy(s.finest, fs), te.Vector(s.finest)
        times = []
        for i in range(reps + 1):
            flush.fill_(i & 0xFF)
            uv.t.zero_()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            s.solve_batched(fv, uv, offsets[0])
            e1.record(stream)
            torch.cuda.synchronize()
            if i:
                times.append(e0.elapsed_time(e1) / 1000.0)
        t = statistics.median(times)
        out[str(B)] = {"solves_per_s": B / t, "batch_ms": 1000 * t}
        del s, fv, uv
    return out


def solver_variants_measure(te, reps=3):
    """One solve at a time with the other cycles and Krylov solvers of the API,
    device time per solve (CUDA events, median of `reps` after one warm-up),
    outer iterations and the true FP64 residual.  W and FMG cycles run the
    config-2 problem.  CG runs unpreconditioned on a uniform 2D mesh (32 x 32
    patches of 32^2: no coarse-fine faces, a symmetric operator) with a
    sine-mode RHS: the reference's CG applies Mr on the right (A Mr p), which
    is not symmetric, and with the multigrid cycle as Mr it diverges on these
    problems in the reference itself (the oracle reproduces it bit for bit)."""
    import numpy as np
    import torch

    from thunderegg_gb300 import mesh as M
    from thunderegg_gb300 import problems as PB
    from thunderegg_gb300.gmg import GmgOptions, GmgSolver

    levels, f_np, _ = PB.config2()
    uni = M.uniform_mesh(2, 5, 32)
    f_uni = PB.sine_modes_rhs(uni[0], np.random.default_rng(3))
    stream = torch.cuda.current_stream()
    out = {}
    c2 = (levels, f_np, "config 2 (circle L3-7, 1444 patches of 32^2)")
    u2 = (uni, f_uni, "2D uniform L5, 1024 patches of 32^2")
    variants = [("bicgstab_W_cycle_mixed", c2, dict(cycle_type="W", cycle_dtype=te.TE_F32, bicgstab_flags=1)),
                ("bicgstab_FMG_cycle_mixed", c2, dict(cycle_type="F", cycle_dtype=te.TE_F32, bicgstab_flags=1)),
                ("bicgstab_W_cycle_fp64", c2, dict(cycle_type="W", cycle_dtype=te.TE_F64, bicgstab_flags=1)),
                ("bicgstab_V_cycle_mixed_uniform", u2, dict(cycle_dtype=te.TE_F32, bicgstab_flags=1)),
                ("cg_unpreconditioned_fp64_uniform", u2, dict(krylov="cg", max_it=5000))]
    for name, (lv, f_np, what), kw in variants:
        pre = not name.startswith("cg_unpreconditioned")
        s = GmgSolver(lv, GmgOptions(scheme=1, smoother=0, tol=1e-10, **kw))
        fv = te.Vector.from_numpy(s.finest, f_np)
        uv = te.Vector(s.finest)
        times, its = [], 0
        for i in range(reps + 1):
            uv.t.zero_()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            its = s.solve(fv, uv, precondition=pre)
            e1.record(stream)
            torch.cuda.synchronize()
            if i:
                times.append(e0.elapsed_time(e1) / 1000.0)
        t = statistics.median(times)
        out[name] = {"problem": what, "solves_per_s": 1.0 / t, "ms": 1000 * t, "outer_iterations": its,
                     "true_rel_residual_fp64": s.residual(fv, uv)}
    return out


def tuner_report(te):
    """The autotuner's choices so far: per kernel and shape, the chosen candidate, the default
    (candidate 0) and the default's time over the chosen one's."""
    import ctypes

    lib = te.capi.lib()
    need = ctypes.c_int(0)
    te.capi.check(lib.te_tune_report(None, 0, ctypes.byref(need)))
    buf = ctypes.create_string_buffer(max(1, need.value))
    te.capi.check(lib.te_tune_report(buf, need.value, ctypes.byref(need)))
    import re

    rows = {}
    entries = json.loads(buf.value.decode() or "[]")
    for r in entries:
        ms = r["ms"]
        default = next(iter(ms)) if ms else None
        gain = None
        if ms and ms.get(default) and ms.get(r["choice"]):
            gain = ms[default] / ms[r["choice"]]
        shape = r["key"].split("|", 1)[1]
        m = re.search(r"P~2\^(\d+)", shape)
        bucket = int(m.group(1)) if m else 0
        group = re.sub(r" P~2\^\d+", "", shape)
        row = {"kernel_shape": shape, "choice": r["choice"], "default": default, "gain_over_default": gain,
               "candidates_ms": ms}
        # one line per kernel and shape: its largest patch-count bucket (the timed levels)
        if group not in rows or bucket > rows[group][0]:
            rows[group] = (bucket, row)
    return {"tuned_shapes": len(entries), "largest_level_per_shape": [v[1] for v in rows.values()]}


def replica_throughput(local_seconds, local_solves, device="cuda"):
    """Whole-job throughput of independent replicas (one process per GPU, no data
    exchange): every rank's solves summed, divided by the slowest rank's time.
    Returns (solves/s, max seconds, total solves); single process without a
    process group: the local numbers."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return local_solves / local_seconds, local_seconds, local_solves
    t = torch.tensor([float(local_seconds)], dtype=torch.float64, device=device)
    n = torch.tensor([float(local_solves)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(n, op=dist.ReduceOp.SUM)
    return float(n.item()) / float(t.item()), float(t.item()), float(n.item())


def config1_measure(te, reps=3):
    """Config 1, the plain method as the FP64 GPU drop-in: 2D uniform L2 (16 patches of
    32^2), f = -2 pi^2 sin(pi x) sin(pi y), u = 0 Dirichlet, BiLinear, BiCGStab patch
    smoother (inner BiCGStab tol 1e-12, 1000 iterations, continue on breakdown), V(1,1)
    to 1 patch, BiCGStab to 1e-10 with the reference's update rule; one solve at a time,
    device time per solve (CUDA events, median of `reps` after one warm-up).  Returns
    (record, solution)."""
    import numpy as np
    import torch

    from thunderegg_gb300 import problems as PB
    from thunderegg_gb300.gmg import GmgOptions, GmgSolver

    levels, f, exact = PB.config1()
    s = GmgSolver(levels, GmgOptions(scheme=0, smoother=1, inner_tol=1e-12, inner_max_it=1000,
                                     inner_continue_on_breakdown=True, tol=1e-10, bicgstab_flags=0))
    fv, uv = te.Vector.from_numpy(s.finest, f), te.Vector(s.finest)
    stream = torch.cuda.current_stream()
    times, its = [], 0
    # clocks and wall times of the timed solves beside their device times: this measurement has
    # read from 190 to 416 ms per solve across full runs with the same kernel choices
    clk = Clocks(dist_info()[2])
    walls = []
    for r in range(reps + 1):
        uv.t.zero_()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        w0 = time.perf_counter()
        e0.record(stream)
        its = s.solve(fv, uv)
        e1.record(stream)
        torch.cuda.synchronize()
        if r:
            times.append(e0.elapsed_time(e1) / 1000.0)
            walls.append(time.perf_counter() - w0)
    clocks = clk.stop()
    u = uv.numpy()
    t = float(np.median(times))
    rec = {"workload": "2D uniform L2, 16 patches of 32^2, BiLinear, BiCGStab patch smoother (inner 1e-12/1000/"
                       "continue), V(1,1), BiCGStab (reference update rule) to 1e-10, FP64",
           "seconds_per_solve": t, "solves_per_s": 1.0 / t, "outer_iterations": its,
           "rep_seconds": [round(x, 4) for x in times], "rep_wall_seconds": [round(x, 4) for x in walls],
           "clocks": clocks,
           "true_rel_residual_fp64": s.residual(fv, uv),
           "max_err_vs_exact": float(np.abs(PB.interior_view(levels[0], u) - PB.interior_view(levels[0], exact)).max())}
    return rec, u


def config3_measure(te, reps=3):
    """Config 3: 3D uniform octree L4 (4096 patches of 16^3, 16.8M cells), TriLinear,
    DFT smoother, u = 0, RHS i.i.d. N(0,1) (seed 0); mixed precision (FP32 V-cycle
    with tensor-core transforms, float-float BiCGStab) and the FP64 drop-in, both
    to a 1e-10 FP64 residual; error of the mixed solution against the FP64 one."""
    import numpy as np
    import torch

    from thunderegg_gb300 import problems as PB
    from thunderegg_gb300.gmg import GmgOptions, GmgSolver

    levels, f, _ = PB.config3()
    out = {}
    sols = {}
    # bf16_ir: the form the configuration names -- FP32 V-cycle whose DFT transforms run as per-patch-
    # scaled BF16 tensor-core contractions (FP32 accumulation), inside FP64 iterative refinement
    for name, opts in (("bf16_ir", GmgOptions(scheme=2, smoother=0, cycle_dtype=te.TE_F32, krylov="ir",
                                              tc_precision=te.capi.TE_TC_BF16, max_it=200)),
                       ("mixed", GmgOptions(scheme=2, smoother=0, cycle_dtype=te.TE_F32, bicgstab_flags=1)),
                       ("fp64", GmgOptions(scheme=2, smoother=0, cycle_dtype=te.TE_F64, bicgstab_flags=1))):
        s = GmgSolver(levels, opts)
        fv, uv = te.Vector.from_numpy(s.finest, f), te.Vector(s.finest)
        times, its = [], 0
        for r in range(reps + 1):
            uv.t.zero_()
            torch.cuda.synchronize()
            t = time.perf_counter()
            its = s.solve(fv, uv)
            torch.cuda.synchronize()
            if r:
                times.append(time.perf_counter() - t)
        out[name] = {"seconds_per_solve": float(np.median(times)), "outer_iterations": its,
                     "true_rel_residual_fp64": s.residual(fv, uv)}
        sols[name] = uv.numpy()
    inner = (Ellipsis, slice(1, -1), slice(1, -1), slice(1, -1))
    d = sols["mixed"][inner] - sols["fp64"][inner]
    out["mixed_vs_fp64_rel_err"] = float(np.abs(d).max() / np.abs(sols["fp64"][inner]).max())
    out["speedup_mixed_vs_fp64"] = out["fp64"]["seconds_per_solve"] / out["mixed"]["seconds_per_solve"]
    out["speedup_bf16_ir_vs_fp64"] = out["fp64"]["seconds_per_solve"] / out["bf16_ir"]["seconds_per_solve"]
    out["forms"] = {"bf16_ir": "FP32 V-cycle, BF16 tensor-core transforms (per-patch power-of-two scaling, FP32 "
                               "accumulation), FP64 iterative refinement",
                    "mixed": "FP32 V-cycle, 3xTF32 tensor-core transforms, float-float BiCGStab with FP64 residual "
                             "checks",
                    "fp64": "FP64 V-cycle and BiCGStab (the plain drop-in)"}
    out["cells"] = int(levels[0].num_cells)
    out["cell_updates_per_s_mixed"] = levels[0].num_cells * out["mixed"]["outer_iterations"] / \
        out["mixed"]["seconds_per_solve"]
    return out, sols


def config4_measure(te):
    """Config 4: 32 variable-coefficient solves on their own random quadtrees (16^2
    patches, BiQuadratic, BiCGStab patch smoother), FP32 V-cycle and float-float
    BiCGStab to 1e-10, served together (the server packs solves of equal depth into
    one launch per level)."""
    import numpy as np

    from thunderegg_gb300 import problems as PB
    from thunderegg_gb300.gmg import GmgOptions
    from thunderegg_gb300.serve import Request, Server

    probs = PB.config4()
    # the FP32 cycle's patch smoother stops at 1e-5 relative (its 1e-12 default is below FP32 resolution
    # and would run every inner solve to its iteration limit)
    opts = GmgOptions(scheme=1, smoother=1, cycle_dtype=te.TE_F32, bicgstab_flags=1, inner_tol=1e-5)
    reqs = [Request(lv, f, opts, coeffs=c) for lv, f, c in probs]
    warm = Server(budget_bytes=150e9, steps_per_round=4)
    for r in reqs[:4]:
        warm.submit(r)
    warm.run()
    srv = Server(budget_bytes=150e9, steps_per_round=4)
    t = time.perf_counter()
    ids = [srv.submit(r) for r in reqs]
    res = srv.run()
    wall = time.perf_counter() - t
    sols = [res[i].u for i in ids[:CONFIG4_CHECKED]]
    return {"solves": len(reqs), "solves_per_s": len(reqs) / wall, "seconds": wall,
            "max_rel_residual": max(r.residual for r in res.values()),
            "mean_iterations": float(np.mean([r.iterations for r in res.values()])),
            "depth_classes": len(srv.classes), "max_batch": srv.stats["max_batch"], "inner_tol": 1e-5,
            "patches_total": int(sum(lv[0].num_patches for lv, _, _ in probs))}, sols, [lv for lv, _, _ in probs]


def serving_stream(args, te):
    """Config-5-style stream through the continuous-batching server: requests
    with Poisson arrivals at --stream-rate, a mix of 2D quadtrees (circle-adaptive
    L3-6 with 32x32 patches, uniform L4 with 32x32, uniform L5 with 16x16) and 3D
    octrees (uniform L3 with 16^3 or 8^3), each RHS a seeded sum of 8 sine modes,
    u = 0 Dirichlet, solved to a 1e-10 FP64 residual under a 150 GB budget.
    Latency is measured from each request's scheduled arrival to its result."""
    import numpy as np

    from thunderegg_gb300 import mesh as M
    from thunderegg_gb300 import problems as PB
    from thunderegg_gb300.gmg import GmgOptions
    from thunderegg_gb300.serve import Request, Server

    rng = np.random.default_rng(2024)
    o2 = GmgOptions(scheme=1, smoother=0, cycle_dtype=te.TE_F32, bicgstab_flags=1)
    o3 = GmgOptions(scheme=2, smoother=0, cycle_dtype=te.TE_F32, bicgstab_flags=1)
    kinds = [(0.30, lambda: M.circle_mesh(n=32, lo=3, hi=6), o2), (0.20, lambda: M.uniform_mesh(2, 4, 32), o2),
             (0.20, lambda: M.uniform_mesh(2, 5, 16), o2), (0.15, lambda: M.uniform_mesh(3, 3, 16, connect="face"), o3),
             (0.15, lambda: M.uniform_mesh(3, 3, 8, connect="face"), o3)]
    meshes = [k[1]() for k in kinds]
    probs = np.array([k[0] for k in kinds])
    reqs = []
    for _ in range(args.stream):
        i = int(rng.choice(len(kinds), p=probs))
        levels = meshes[i]
        reqs.append(Request(levels, PB.sine_modes_rhs(levels[0], rng), kinds[i][2]))
    arrivals = np.cumsum(rng.exponential(1.0 / args.stream_rate, size=len(reqs)))
    srv = Server(budget_bytes=150e9, steps_per_round=2)
    # warm-up: one request of every kind (builds, graph captures) before the clock starts
    for i in range(len(kinds)):
        srv.submit(Request(meshes[i], PB.sine_modes_rhs(meshes[i][0], rng), kinds[i][2]))
    srv.run()
    srv.results = {}
    builds0, hits0, reforms0 = srv.stats["union_builds"], srv.stats["union_hits"], srv.stats["reforms"]
    fills0 = srv.stats["slot_fills"]
    t0 = time.perf_counter()
    ids, nxt = {}, 0
    while nxt < len(reqs) or not srv.idle():
        now = time.perf_counter() - t0
        while nxt < len(reqs) and arrivals[nxt] <= now:
            ids[srv.submit(reqs[nxt])] = nxt
            nxt += 1
        if srv.idle():
            time.sleep(max(0.0, min(arrivals[nxt] - now, 0.01)))
            continue
        srv.step()
    wall = time.perf_counter() - t0
    lat, res_max, its = [], 0.0, []
    for rid, r in srv.results.items():
        k = ids[rid]
        lat.append(r.latency_s)
        res_max = max(res_max, r.residual)
        its.append(r.iterations)
    lat.sort()
    pick = lambda q: lat[min(len(lat) - 1, int(round(q * (len(lat) - 1))))]  # noqa: E731
    return {"requests": len(reqs), "arrival_rate_per_s": args.stream_rate, "solves_per_s": len(reqs) / wall,
            "latency_ms_p50": 1000 * pick(0.5), "latency_ms_p99": 1000 * pick(0.99),
            "max_rel_residual": res_max, "mean_iterations": float(np.mean(its)),
            "max_batch": srv.stats["max_batch"], "reforms": srv.stats["reforms"] - reforms0,
            "slot_fills": srv.stats["slot_fills"] - fills0,
            "union_builds": srv.stats["union_builds"] - builds0, "union_cache_hits": srv.stats["union_hits"] - hits0,
            "mix": "0.7 x 2D (circle L3-6 32^2, uniform L4 32^2, uniform L5 16^2), "
                   "0.3 x 3D (uniform L3 16^3, uniform L3 8^3); 150 GB budget",
            "latency_from": "scheduled arrival"}


def config5_stream(args, te):
    """Config 5's serving stream: requests with Poisson arrivals at several rates.  Each request is,
    with probability 0.7, a 2D quadtree -- uniform at a level drawn from 2..6, or circle-adaptive
    L3-7 -- with n x n patches, n drawn from {16, 32, 64}; otherwise a 3D uniform octree at a level
    drawn from 2..4 with 8^3 or 16^3 patches.  Right-hand side: a seeded sum of 8 sine modes,
    u = 0 Dirichlet; mixed precision (FP32 V-cycle, tensor-core transforms where the patch shape
    allows) to a 1e-10 FP64 residual; 150 GB budget; solves of one patch size share launches
    whatever their depth.  Latency is measured from each request's scheduled arrival.  Beside it:
    the plain FP64 drop-in's time for the same request list, one solve at a time (each distinct
    mesh timed once, CUDA events)."""
    import numpy as np
    import torch

    from thunderegg_gb300 import mesh as M
    from thunderegg_gb300 import problems as PB
    from thunderegg_gb300.gmg import GmgOptions, GmgSolver
    from thunderegg_gb300.serve import Request, Server

    rng = np.random.default_rng(5)
    meshes = {}

    def mesh(kind):
        if kind not in meshes:
            d, shape, lvl, n = kind
            if shape == "circle":
                meshes[kind] = M.circle_mesh(n=n, lo=3, hi=7)
            else:
                meshes[kind] = M.uniform_mesh(d, lvl, n, connect="full" if d == 2 else "face")
        return meshes[kind]

    def draw():
        if rng.random() < 0.7:
            n = int(rng.choice([16, 32, 64]))
            if rng.random() < 0.5:
                return (2, "uniform", int(rng.integers(2, 7)), n)
            return (2, "circle", 7, n)
        return (3, "uniform", int(rng.integers(2, 5)), int(rng.choice([8, 16])))

    def opts(kind, dtype):
        return GmgOptions(scheme=1 if kind[0] == 2 else 2, smoother=0, cycle_dtype=dtype, bicgstab_flags=1)

    rates = [float(x) for x in args.c5_rates.split(",")]
    per_rate = args.c5_requests
    streams = []
    for rate in rates:
        kinds = [draw() for _ in range(per_rate)]
        reqs = [Request(mesh(k), PB.sine_modes_rhs(mesh(k)[0], rng), opts(k, te.TE_F32)) for k in kinds]
        arrivals = np.cumsum(rng.exponential(1.0 / rate, size=per_rate))
        streams.append((rate, kinds, reqs, arrivals))
    srv = Server(budget_bytes=150e9, steps_per_round=2)
    # warm-up: one request of every distinct mesh (tuning, graph captures) before the clocks start
    for k in sorted({k for _, kinds, _, _ in streams for k in kinds}):
        srv.submit(Request(mesh(k), PB.sine_modes_rhs(mesh(k)[0], rng), opts(k, te.TE_F32)))
    srv.run()
    out = []
    for rate, kinds, reqs, arrivals in streams:
        srv.results = {}
        builds0, hits0 = srv.stats["union_builds"], srv.stats["union_hits"]
        t0 = time.perf_counter()
        ids, nxt = {}, 0
        while nxt < len(reqs) or not srv.idle():
            now = time.perf_counter() - t0
            while nxt < len(reqs) and arrivals[nxt] <= now:
                ids[srv.submit(reqs[nxt])] = nxt
                nxt += 1
            if srv.idle():
                time.sleep(max(0.0, min(arrivals[nxt] - now, 0.01)))
                continue
            srv.step()
        wall = time.perf_counter() - t0
        lat = sorted(r.latency_s for r in srv.results.values())
        pick = lambda q: lat[min(len(lat) - 1, int(round(q * (len(lat) - 1))))]  # noqa: E731
        out.append({"arrival_rate_per_s": rate, "requests": len(reqs), "solves_per_s": len(reqs) / wall,
                    "latency_ms_p50": 1000 * pick(0.5), "latency_ms_p99": 1000 * pick(0.99),
                    "max_rel_residual": max(r.residual for r in srv.results.values()),
                    "union_builds": srv.stats["union_builds"] - builds0,
                    "union_cache_hits": srv.stats["union_hits"] - hits0})
    srv.close()
    # the same request lists through the C ABI's native serving loop (te_serve_*)
    from thunderegg_gb300.serve import NativeServer

    nsrv = NativeServer(budget_bytes=150e9, steps_per_round=2)
    warm = [nsrv.submit(mesh(k), PB.sine_modes_rhs(mesh(k)[0], rng), opts(k, te.TE_F32))
            for k in sorted({k for _, kinds, _, _ in streams for k in kinds})]
    nsrv.run(warm)
    for o, (rate, kinds, reqs, arrivals) in zip(out, streams):
        st0 = nsrv.stats()
        t0 = time.perf_counter()
        pending, nxt, lat, res_max = {}, 0, [], 0.0
        while nxt < len(reqs) or pending:
            now = time.perf_counter() - t0
            while nxt < len(reqs) and arrivals[nxt] <= now:
                pending[nsrv.submit(reqs[nxt].levels, reqs[nxt].f, reqs[nxt].opts)] = arrivals[nxt]
                nxt += 1
            if not pending:
                time.sleep(max(0.0, min(arrivals[nxt] - now, 0.01)))
                continue
            nsrv.step()
            for rid in list(pending):
                r = nsrv.poll(rid)
                if r is not None:
                    lat.append(time.perf_counter() - t0 - pending.pop(rid))
                    res_max = max(res_max, r.residual)
        wall = time.perf_counter() - t0
        lat.sort()
        pick = lambda q: lat[min(len(lat) - 1, int(round(q * (len(lat) - 1))))]  # noqa: E731
        st1 = nsrv.stats()
        o["native_server"] = {"solves_per_s": len(reqs) / wall, "latency_ms_p50": 1000 * pick(0.5),
                              "latency_ms_p99": 1000 * pick(0.99), "max_rel_residual": res_max,
                              "union_builds": st1["union_builds"] - st0["union_builds"],
                              "union_cache_hits": st1["union_cache_hits"] - st0["union_cache_hits"],
                              "slot_fills": st1["slot_fills"] - st0["slot_fills"],
                              "host_s": {k: round(st1[k] - st0[k], 4) for k in ("build_s", "form_s", "step_s",
                                                                                 "finish_s")}}
    nsrv.close()
    # the plain FP64 drop-in, one solve at a time, over the same request lists
    stream = torch.cuda.current_stream()
    fp64_s = {}
    for k in sorted({k for _, kinds, _, _ in streams for k in kinds}):
        s = GmgSolver(mesh(k), opts(k, te.TE_F64))
        fv = te.Vector.from_numpy(s.finest, PB.sine_modes_rhs(mesh(k)[0], rng))
        uv = te.Vector(s.finest)
        for r in range(2):
            uv.t.zero_()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            s.solve(fv, uv)
            e1.record(stream)
            torch.cuda.synchronize()
        fp64_s[k] = e0.elapsed_time(e1) / 1000.0
        del s, fv, uv
    for o, (_, kinds, _, _) in zip(out, streams):
        t = sum(fp64_s[k] for k in kinds)
        o["fp64_dropin_one_at_a_time_solves_per_s"] = len(kinds) / t
        o["served_vs_fp64_dropin"] = o["solves_per_s"] / (len(kinds) / t)
    return {"rates": out, "requests_per_rate": per_rate,
            "mix": "0.7 x 2D (uniform L2-6 or circle L3-7; 16^2/32^2/64^2), 0.3 x 3D (uniform L2-4; 8^3/16^3); "
                   "8 random sine modes, u = 0; 150 GB budget",
            "distinct_meshes": len(fp64_s), "latency_from": "scheduled arrival",
            "requests_note": "bounded count per rate (the configuration names 10,000) so the default run "
                             "finishes in minutes"}


def run_gpu(args):
    import numpy as np
    import torch

    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    import thunderegg_gb300 as te
    from thunderegg_gb300 import build as tb
    from thunderegg_gb300 import mesh as M
    from thunderegg_gb300 import problems as PB
    from thunderegg_gb300.gmg import GmgOptions, GmgSolver

    tb.build()
    L = te.capi.lib()
    B = args.batch
    extra = not args.no_extra and not args.only_mixed and rank == 0
    # FP64 oracle solutions, computed on host cores while the GPU legs run
    refs = None
    if rank == 0 and not args.kernels and not args.only_mixed:
        names = [n for n in ORACLE_JOBS if extra or n in ("config2",)]
        refs = OracleRefs(names)
    levels, f_np, exact = PB.config2()
    rng = np.random.default_rng(2024)
    # B independent right-hand sides on the same mesh: the benchmark problem plus
    # seeded sine-mode perturbations (each solve is a full, distinct solve)
    fs = [f_np] + [f_np + 0.1 * PB.sine_modes_rhs(levels[0], rng) for _ in range(B - 1)]
    mixed_opts = GmgOptions(scheme=1, smoother=0, tol=1e-10, cycle_dtype=te.TE_F32, bicgstab_flags=1)
    fp64_opts = GmgOptions(scheme=1, smoother=0, tol=1e-10, cycle_dtype=te.TE_F64, bicgstab_flags=1)
    blevels, offsets = M.union_hierarchy([levels] * B)
    served = GmgSolver(blevels, mixed_opts)
    single = GmgSolver(levels, mixed_opts)
    fp64 = GmgSolver(levels, fp64_opts)
    fB_np = np.concatenate(fs, axis=0)
    fB = te.Vector.from_numpy(served.finest, fB_np)
    uB = te.Vector(served.finest)
    f1 = te.Vector.from_numpy(single.finest, f_np)
    u1 = te.Vector(single.finest)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm = peaks.get("hbm_gbs", 6800.0)
    if args.kernels:
        if rank == 0:
            lk = level_kernel_rooflines(te, served, hbm)
            lk["peak_source"] = "measured" if peaks else "fallback"
            print(json.dumps({"level_kernels": lk}), flush=True)
        return

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    def timed(step, k, warm):
        times, out = [], None
        for i in range(warm + k):
            flush.fill_(i & 0xFF)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            out = step()
            e1.record(stream)
            torch.cuda.synchronize()
            if i >= warm:
                times.append(e0.elapsed_time(e1) / 1000.0)
        return times, out

    def served_step():
        uB.t.zero_()
        return served.solve_batched(fB, uB, offsets[0])

    # ---- headline: mixed precision, B solves served per step, inputs in HBM
    barrier()
    launches0 = L.te_kernel_launch_count()
    clk = Clocks(local)
    t_wall = time.perf_counter()
    times, (its, res, st) = timed(served_step, args.steps, args.warmup)
    t_wall = time.perf_counter() - t_wall
    clocks = clk.stop()
    launches = (L.te_kernel_launch_count() - launches0) * args.steps // (args.steps + args.warmup)
    barrier()
    value, total, _ = replica_throughput(sum(times), B * args.steps)
    true_res = []
    uB_np = uB.numpy()
    for b in range(B):
        sl = slice(offsets[0][b], offsets[0][b + 1])
        uu = te.Vector.from_numpy(single.finest, uB_np[sl])
        ff = te.Vector.from_numpy(single.finest, fB_np[sl])
        true_res.append(single.residual(ff, uu))
    err = float(np.abs(PB.interior_view(levels[0], uB_np[:levels[0].num_patches])
                       - PB.interior_view(levels[0], exact)).max())

    if args.only_mixed:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": "solves/s", "batch": B,
                              "ms_per_step": 1000 * total / args.steps, "outer_iterations": max(its),
                              "max_true_rel_residual": max(true_res), "gpu_launches": int(launches),
                              "clocks": clocks}), flush=True)
        return

    # ---- one solve at a time (latency), mixed and plain FP64 drop-in
    def single_step(s, f, u):
        def run():
            u.t.zero_()
            return s.solve(f, u)
        return run

    lat, its1 = timed(single_step(single, f1, u1), args.steps, 2)
    u_single = u1.numpy()
    d_times, d_its = timed(single_step(fp64, f1, u1), args.fp64_steps, 1)
    d_res = fp64.residual(f1, u1)
    u_fp64 = u1.numpy()

    # ---- e2e: the served step through the C ABI from pinned host memory.  Every step copies its
    # right-hand sides host->device and its solutions device->host inside the timed region; the
    # copies run on a copy stream, overlapped with the neighbouring steps' solves (step k+1's
    # inputs go up and step k-1's results come down while step k solves; device buffers are
    # double-buffered).  Time: CUDA events from before the first upload to after the last download.
    hf = torch.from_numpy(fB_np).pin_memory()
    hu = [torch.empty(fB_np.shape, dtype=torch.float64).pin_memory() for _ in range(2)]
    fBs = [fB, te.Vector.from_numpy(served.finest, fB_np)]
    uBs = [uB, te.Vector(served.finest)]
    cstream = torch.cuda.Stream()

    def e2e_run(k_steps):
        ev_up = [torch.cuda.Event() for _ in range(k_steps)]
        ev_done = [torch.cuda.Event() for _ in range(k_steps)]
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        cstream.wait_stream(stream)
        with torch.cuda.stream(cstream):
            fBs[0].t.copy_(hf, non_blocking=True)
            ev_up[0].record(cstream)
        for k in range(k_steps):
            with torch.cuda.stream(cstream):
                if k + 1 < k_steps:
                    if k >= 1:
                        cstream.wait_event(ev_done[k - 1])  # step k-1 no longer reads its input buffer
                    fBs[(k + 1) % 2].t.copy_(hf, non_blocking=True)
                    ev_up[k + 1].record(cstream)
                if k >= 1:
                    cstream.wait_event(ev_done[k - 1])
                    hu[(k - 1) % 2].copy_(uBs[(k - 1) % 2].t, non_blocking=True)
            stream.wait_event(ev_up[k])
            uBs[k % 2].t.zero_()
            served.solve_batched(fBs[k % 2], uBs[k % 2], offsets[0])
            ev_done[k].record(stream)
        with torch.cuda.stream(cstream):
            cstream.wait_event(ev_done[k_steps - 1])
            hu[(k_steps - 1) % 2].copy_(uBs[(k_steps - 1) % 2].t, non_blocking=True)
        stream.wait_stream(cstream)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1000.0

    e2e_run(2)  # warm-up: graphs of the second buffer set
    k_e2e = max(4, args.steps)
    e_time = e2e_run(k_e2e)
    e2e = world * B * k_e2e / e_time
    e2e_copy_gbs = 2 * fB_np.nbytes * k_e2e / e_time / 1e9

    # ---- dominant kernel: per-phase device times of the served batch's V-cycle, averaged over
    # several eager applications (CUDA events on the cycle's stream around each launch)
    mp = te.Vector(served.finest)
    reps = 5
    acc_ph = {}
    for _ in range(reps):
        for n_, t_ in served.cycle.timings(fB, mp):
            acc_ph[n_] = acc_ph.get(n_, 0.0) + t_ / reps
    phases = sorted(acc_ph.items(), key=lambda x: -x[1])
    top_name, top_ms = phases[0]
    alg = _phase_bytes(top_name, blevels, 4)
    # DRAM bytes of one launch of the phase from an ncu capture of this workload (when recorded)
    traffic = None
    try:
        tb = json.load(open(os.path.join(ROOT, "profiles", "dram_bytes_config2_served_b16.json")))
        if B == 16 and world == 1:
            traffic = tb["bytes_per_launch"].get(top_name)
    except Exception:
        pass
    achieved = alg / (top_ms / 1000.0) / 1e9
    cyc_total = sum(t for _, t in phases)

    # measurements beside the headline, after its timed region: a failure in one is
    # recorded in its key (the traceback goes to stderr) and the line still prints
    def optional(fn, *a):
        try:
            return fn(*a)
        except Exception as e:  # noqa: BLE001
            import traceback

            traceback.print_exc()
            return {"error": f"{type(e).__name__}: {e}"}

    stream = optional(serving_stream, args, te) if (args.stream > 0 and not args.only_mixed and rank == 0) else None
    c5 = optional(config5_stream, args, te) if (extra and args.c5_requests > 0) else None
    c1 = optional(config1_measure, te) if extra else None
    c3 = optional(config3_measure, te) if extra else None
    c4 = optional(config4_measure, te) if extra else None
    lk = optional(level_kernel_rooflines, te, served, hbm) if extra else None
    sv = optional(solver_variants_measure, te) if extra else None
    bs = optional(batch_scaling_measure, te) if extra else None
    fk = optional(fp64_krylov_measure, te, blevels, offsets, fB) if extra else None

    # error of every result against the oracle's FP64 solve of the same problem
    oracle_err = None
    if refs is not None:
        def compare():
            P0 = levels[0].num_patches
            lv0 = levels[0]
            r2 = refs.get("config2")
            out = {"config2_served_batch_solve0": err_vs(uB_np[:P0], r2, lv0),
                   "config2_e2e_solve0": err_vs(hu[(k_e2e - 1) % 2].numpy()[:P0], r2, lv0),
                   "config2_single_mixed": err_vs(u_single, r2, lv0),
                   "config2_fp64_dropin": err_vs(u_fp64, r2, lv0)}
            if isinstance(c1, tuple):
                from thunderegg_gb300 import problems as PB

                out["config1_fp64_dropin"] = err_vs(c1[1], refs.get("config1"), PB.config1()[0][0])
            if isinstance(c3, tuple):
                from thunderegg_gb300 import problems as PB

                r3 = refs.get("config3")
                lv3 = PB.config3()[0][0]
                out["config3_bf16_ir"] = err_vs(c3[1]["bf16_ir"], r3, lv3)
                out["config3_mixed"] = err_vs(c3[1]["mixed"], r3, lv3)
                out["config3_fp64_dropin"] = err_vs(c3[1]["fp64"], r3, lv3)
                del r3
            if isinstance(c4, tuple):
                out["config4_mixed_served"] = [err_vs(u, refs.get(f"config4_{k}"), c4[2][k][0])
                                               for k, u in enumerate(c4[1])]
            out["oracle"] = {"kind": "port (CPU restatement of the reference, FP64)",
                             "solves": refs.info,
                             "bicgstab_update": "config1: the reference's rule; others: alpha*M p on the early "
                                                "exit, as the GPU solves they are compared with",
                             "measure": "max |u - u_oracle| / max |u_oracle| over finest interior cells"}
            return out

        oracle_err = optional(compare)
        refs.close()
    c1 = c1[0] if isinstance(c1, tuple) else c1
    c3 = c3[0] if isinstance(c3, tuple) else c3
    c4 = c4[0] if isinstance(c4, tuple) else c4

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        w, out = cpu_solves(1)
        cpu = {"value": 1.0 / out[0][0], "unit": "solves/s", "cores": 1, "kind": "port",
               "sample": "one full FP64 solve of the same workload by the CPU restatement, 1 core"}

    def pct(v, q):
        v = sorted(v)
        return v[min(len(v) - 1, int(round(q * (len(v) - 1))))]

    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000 * total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 V-cycle (3xTF32 transforms) + float-float Krylov, f64 residual check", "data": "synthetic",
        "config": {"workload": WORKLOAD, "served_batch": B, "patches_per_solve": levels[0].num_patches,
                   "levels": len(levels), "cells_per_solve": levels[0].num_cells,
                   "rhs": "benchmark RHS + seeded sine-mode perturbations (one per solve)",
                   "l2": "flushed between steps (256 MiB write), outside step timing",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "latency_ms": {"served_batch_p50": 1000 * pct(times, 0.5), "served_batch_p99": 1000 * pct(times, 0.99),
                       "single_solve_p50": 1000 * pct(lat, 0.5), "single_solve_p99": 1000 * pct(lat, 0.99)},
        "single_solve_mixed": {"value": len(lat) / sum(lat), "unit": "solves/s", "outer_iterations": its1},
        "outer_iterations": max(its), "max_true_rel_residual_fp64": max(true_res), "max_err_vs_exact": err,
        # finest-level cells x outer BiCGStab iterations per second (each iteration: two V-cycles,
        # two operator applications)
        "cell_updates_per_s": value * levels[0].num_cells * max(its),
        "fp64_dropin": {"value": len(d_times) / sum(d_times), "unit": "solves/s",
                        "latency_ms_p50": 1000 * pct(d_times, 0.5), "outer_iterations": d_its,
                        "final_rel_residual_fp64": d_res},
        "speedup_served_vs_fp64_dropin": value / world / (len(d_times) / sum(d_times)),
        "e2e": {"value": e2e, "unit": "solves/s", "h2d_bytes_per_step": int(fB_np.nbytes),
                "d2h_bytes_per_step": int(fB_np.nbytes), "steps": k_e2e,
                "copies": "pinned host buffers, copy stream overlapped with the neighbouring steps' solves",
                "copy_gbs_sustained": e2e_copy_gbs},
        "gpu_launches": int(launches),
        "roofline": {"kernel": f"{top_name} (fused V-cycle phase, served batch)", "bound": "hbm",
                     "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": traffic, "peak_source": "measured" if peaks else "fallback",
                     "launch_ms": top_ms, "algorithmic_bytes": alg,
                     "share_of_vcycle": top_ms / cyc_total if cyc_total else None},
        "vcycle_phases_ms": [[n, round(t, 4)] for n, t in phases[:6]],
        "err_vs_oracle": oracle_err,
        "autotuner": optional(tuner_report, te),
        "cpu_baseline": cpu,
        "clocks": clocks,
        "wall_s_timed": t_wall,
        "serving_stream": stream,
        "config5_stream": c5,
        "config1": c1,
        "config3": c3,
        "config4": c4,
        "level_kernels": lk,
        "solver_variants": sv,
        "batch_scaling": bs,
        "served_fp64_krylov": fk,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
