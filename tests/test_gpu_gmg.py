"""GMG cycles (V, W, FMG) and BiCGStab solves on the GPU against the CPU oracle.

V-cycle applications agree with the oracle to 1e-11 (FP64).  Solves reach the
same iteration count and the same solution to the solver tolerance; with the
preconditioned early-exit update the true FP64 residual is below the tolerance.
"""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


def _setup(te, levels, scheme, smoother, seed, coeffs=None, **kw):
    from oracle import gmg_config
    from thunderegg_gb300.gmg import GmgOptions, GmgSolver

    opts = GmgOptions(scheme=scheme, smoother=smoother, **kw)
    s = GmgSolver(levels, opts, coeffs)
    cfg = gmg_config(scheme=scheme, smoother=smoother, op_kind=1 if coeffs is not None else 0,
                     tol=opts.tol, pre_sweeps=opts.pre_sweeps, post_sweeps=opts.post_sweeps,
                     coarse_sweeps=opts.coarse_sweeps)
    rng = np.random.default_rng(seed)
    f = rng.standard_normal(levels[0].padded_shape(1))
    return s, cfg, f


def meshes():
    from thunderegg_gb300 import mesh as M

    return [("2d_uniform", M.uniform_mesh(2, 2, 8), 0), ("2d_circle", M.circle_mesh(n=8, lo=2, hi=5), 1),
            ("3d_random", M.random_mesh(5, n=4, dim=3, lo=1, hi=3), 2)]


@pytest.mark.parametrize("idx", range(3))
@pytest.mark.parametrize("smoother", (0, 1))
def test_vcycle_fp64(te, oracle, idx, smoother):
    name, levels, scheme = meshes()[idx]
    s, cfg, f = _setup(te, levels, scheme, smoother, 10 + idx)
    want = oracle.vcycle(levels, f, cfg)
    fv = te.Vector.from_numpy(s.finest, f)
    uv = te.Vector(s.finest)
    s.cycle.apply(fv, uv)
    g = levels[0].num_ghost
    inner = (Ellipsis,) + tuple(slice(g, -g) for _ in range(levels[0].dim))
    tol = 1e-11 if smoother == 0 else 1e-7
    assert rel_err(uv.numpy()[inner], want[inner]) <= tol


@pytest.mark.parametrize("idx", range(3))
def test_solve_fp64_matches_oracle(te, oracle, idx):
    name, levels, scheme = meshes()[idx]
    s, cfg, f = _setup(te, levels, scheme, 0, 20 + idx)
    u_o, its_o, _, rc = oracle.solve(levels, f, cfg)
    assert rc == 0
    fv = te.Vector.from_numpy(s.finest, f)
    uv = te.Vector(s.finest)
    its = s.solve(fv, uv)
    assert its == its_o
    g = levels[0].num_ghost
    inner = (Ellipsis,) + tuple(slice(g, -g) for _ in range(levels[0].dim))
    assert rel_err(uv.numpy()[inner], u_o[inner]) <= 1e-8


@pytest.mark.parametrize("idx", range(3))
@pytest.mark.parametrize("cycle_dtype", ("f64", "f32"))
def test_solve_reaches_tolerance(te, idx, cycle_dtype):
    name, levels, scheme = meshes()[idx]
    dt = te.TE_F64 if cycle_dtype == "f64" else te.TE_F32
    s, cfg, f = _setup(te, levels, scheme, 0, 30 + idx, cycle_dtype=dt, bicgstab_flags=1)
    fv = te.Vector.from_numpy(s.finest, f)
    uv = te.Vector(s.finest)
    its = s.solve(fv, uv)
    assert its < 40
    assert s.residual(fv, uv) <= 1e-10


@pytest.mark.parametrize("opts", [dict(extrapolate_boundary_ghosts=True),
                                  dict(pre_sweeps=0, post_sweeps=2, coarse_sweeps=2),
                                  dict(pre_sweeps=2, post_sweeps=0, coarse_sweeps=1)])
def test_vcycle_options(te, oracle, opts):
    """Cycle options and the unfused residual path (ghost extrapolation on)."""
    from oracle import gmg_config
    from thunderegg_gb300 import mesh as M
    from thunderegg_gb300.gmg import GmgOptions, GmgSolver

    levels = M.circle_mesh(n=8, lo=2, hi=5)
    o = GmgOptions(scheme=1, smoother=0, **opts)
    s = GmgSolver(levels, o)
    cfg = gmg_config(scheme=1, smoother=0, pre_sweeps=o.pre_sweeps, post_sweeps=o.post_sweeps,
                     coarse_sweeps=o.coarse_sweeps, extrapolate_boundary_ghosts=int(o.extrapolate_boundary_ghosts))
    f = np.random.default_rng(40).standard_normal(levels[0].padded_shape(1))
    want = oracle.vcycle(levels, f, cfg)
    for dt, tol in ((te.TE_F64, 1e-11), (te.TE_F32, 5e-5)):
        s2 = GmgSolver(levels, GmgOptions(scheme=1, smoother=0, cycle_dtype=dt, **opts))
        fv = te.Vector.from_numpy(s2.finest, f)
        uv = te.Vector(s2.finest)
        for _ in range(2):  # second application replays the captured graph
            s2.cycle.apply(fv, uv)
            g = levels[0].num_ghost
            inner = (Ellipsis, slice(g, -g), slice(g, -g))
            assert rel_err(uv.numpy()[inner], want[inner]) <= tol, (dt, opts)


def test_solve_no_preconditioner(te, oracle):
    from oracle import gmg_config
    from thunderegg_gb300 import mesh as M
    from thunderegg_gb300.gmg import GmgOptions, GmgSolver

    levels = M.uniform_mesh(2, 1, 8)
    s = GmgSolver(levels, GmgOptions(scheme=0, smoother=0, tol=1e-9))
    f = np.random.default_rng(41).standard_normal(levels[0].padded_shape(1))
    u_o, its_o, _, rc = oracle.solve(levels, f, gmg_config(scheme=0, tol=1e-9, use_precond=0))
    fv, uv = te.Vector.from_numpy(s.finest, f), te.Vector(s.finest)
    its = s.solve(fv, uv, precondition=False)
    assert abs(its - its_o) <= 1
    inner = (Ellipsis, slice(1, -1), slice(1, -1))
    assert rel_err(uv.numpy()[inner], u_o[inner]) <= 1e-7


def test_solve_repeated_and_launch_count(te):
    """Repeated solves replay cached graphs and give identical results."""
    from thunderegg_gb300 import mesh as M
    from thunderegg_gb300.gmg import GmgOptions, GmgSolver

    levels = M.circle_mesh(n=8, lo=2, hi=5)
    s = GmgSolver(levels, GmgOptions(scheme=1, smoother=0, cycle_dtype=te.TE_F32, bicgstab_flags=1))
    f = np.random.default_rng(42).standard_normal(levels[0].padded_shape(1))
    fv = te.Vector.from_numpy(s.finest, f)
    outs = []
    for _ in range(3):
        uv = te.Vector(s.finest)
        n0 = te.capi.lib().te_kernel_launch_count()
        its = s.solve(fv, uv)
        assert te.capi.lib().te_kernel_launch_count() - n0 > 10 * its
        outs.append(uv.numpy())
    assert np.array_equal(outs[0], outs[1]) and np.array_equal(outs[1], outs[2])


@pytest.mark.parametrize("idx", range(3))
@pytest.mark.parametrize("cycle_dtype", ("f64", "f32"))
def test_fused_cycle_matches_unfused(te, idx, cycle_dtype, monkeypatch):
    """The fused per-level kernels give the same V-cycle as the unfused sequence
    (ghost fill, apply, residual, restrict, interpolate, ghost fill, smooth)."""
    name, levels, scheme = meshes()[idx]
    from thunderegg_gb300.gmg import GmgOptions, GmgSolver

    dt = te.TE_F64 if cycle_dtype == "f64" else te.TE_F32
    f = np.random.default_rng(50 + idx).standard_normal(levels[0].padded_shape(1))
    outs = []
    for nofuse in ("0", "1"):
        monkeypatch.setenv("TE_NO_FUSION", nofuse)
        s = GmgSolver(levels, GmgOptions(scheme=scheme, smoother=0, cycle_dtype=dt))
        fv, uv = te.Vector.from_numpy(s.finest, f), te.Vector(s.finest)
        s.cycle.apply(fv, uv)
        outs.append(uv.numpy())
    g = levels[0].num_ghost
    inner = (Ellipsis,) + tuple(slice(g, -g) for _ in range(levels[0].dim))
    tol = 1e-12 if cycle_dtype == "f64" else 2e-5
    assert rel_err(outs[0][inner], outs[1][inner]) <= tol


@pytest.mark.parametrize("n", (8, 16))
def test_batched_solves_match_alone(te, n):
    """A batch of independent solves: each solve's result is bit-identical to
    the same solve alone (batch of one) and to the single-solve entry point.
    n = 16 takes the fused apply+dot kernels and the tensor-core transforms."""
    from thunderegg_gb300 import mesh as M
    from thunderegg_gb300 import problems as PB
    from thunderegg_gb300.gmg import GmgOptions, GmgSolver

    hiers = [M.circle_mesh(n=n, lo=2, hi=5 if n == 8 else 4) for _ in range(3)]
    rng = np.random.default_rng(60)
    fs = [PB.sine_modes_rhs(h[0], rng) for h in hiers]
    opts = GmgOptions(scheme=1, smoother=0, cycle_dtype=te.TE_F32, bicgstab_flags=1)
    levels, offsets = M.union_hierarchy(hiers)
    s = GmgSolver(levels, opts)
    fv = te.Vector.from_numpy(s.finest, np.concatenate(fs, axis=0))
    uv = te.Vector(s.finest)
    its, res, st = s.solve_batched(fv, uv, offsets[0])
    assert st == [0, 0, 0] and all(r <= 1e-10 for r in res)
    mixed = uv.numpy()
    for b in range(3):
        one = GmgSolver(hiers[b], opts)
        f1 = te.Vector.from_numpy(one.finest, fs[b])
        u1 = te.Vector(one.finest)
        its1, _, _ = one.solve_batched(f1, u1, [0, hiers[b][0].num_patches])
        assert its1[0] == its[b]
        part = mixed[offsets[0][b]:offsets[0][b + 1]]
        inner = (Ellipsis, slice(1, -1), slice(1, -1))
        assert np.array_equal(part[inner], u1.numpy()[inner])
        u2 = te.Vector(one.finest)
        assert one.solve(f1, u2) == its[b]
        assert np.array_equal(u2.numpy()[inner], part[inner])


@pytest.mark.parametrize("idx", range(3))
@pytest.mark.parametrize("cycle_type", ("W", "F"))
@pytest.mark.parametrize("smoother", (0, 1))
def test_w_and_fmg_cycles(te, oracle, idx, cycle_type, smoother):
    """WCycle (GMG/WCycle.h:50-84) and FMGCycle (GMG/FMGCycle.h:43-104) through
    CycleBuilder's cycle_type, FP64 and FP32, against the oracle (pinned to the
    reference's own cycles by tests/test_oracle_pin.py).  FP64 tolerance as the
    V-cycle; FP32 5e-5; the second application replays the captured graph."""
    from oracle import gmg_config
    from thunderegg_gb300.gmg import GmgOptions, GmgSolver

    name, levels, scheme = meshes()[idx]
    mid = 2 if smoother else 1
    cfg = gmg_config(scheme=scheme, smoother=smoother, cycle_type=cycle_type, mid_sweeps=mid)
    f = np.random.default_rng(50 + idx).standard_normal(levels[0].padded_shape(1))
    want = oracle.vcycle(levels, f, cfg)
    g = levels[0].num_ghost
    inner = (Ellipsis,) + tuple(slice(g, -g) for _ in range(levels[0].dim))
    tols = ((te.TE_F64, 1e-11 if smoother == 0 else 1e-7), (te.TE_F32, 5e-5))
    for dt, tol in tols:
        s = GmgSolver(levels, GmgOptions(scheme=scheme, smoother=smoother, cycle_type=cycle_type, mid_sweeps=mid,
                                         cycle_dtype=dt))
        fv = te.Vector.from_numpy(s.finest, f)
        uv = te.Vector(s.finest)
        for _ in range(2):
            s.cycle.apply(fv, uv)
            assert rel_err(uv.numpy()[inner], want[inner]) <= tol, (dt, cycle_type)


@pytest.mark.parametrize("cycle_type", ("W", "F"))
def test_solve_with_w_and_fmg_cycles(te, oracle, cycle_type):
    """GMG-preconditioned BiCGStab with the W / FMG cycle: the same iteration
    count and solution as the oracle (FP64 cycle), and the FP64 residual below
    the tolerance with the mixed-precision cycle."""
    from oracle import gmg_config
    from thunderegg_gb300.gmg import GmgOptions, GmgSolver

    name, levels, scheme = meshes()[1]
    f = np.random.default_rng(60).standard_normal(levels[0].padded_shape(1))
    u_o, its_o, _, rc = oracle.solve(levels, f, gmg_config(scheme=scheme, smoother=0, cycle_type=cycle_type))
    assert rc == 0
    s = GmgSolver(levels, GmgOptions(scheme=scheme, smoother=0, cycle_type=cycle_type))
    fv = te.Vector.from_numpy(s.finest, f)
    uv = te.Vector(s.finest)
    assert s.solve(fv, uv) == its_o
    inner = (Ellipsis, slice(1, -1), slice(1, -1))
    assert rel_err(uv.numpy()[inner], u_o[inner]) <= 1e-8
    s32 = GmgSolver(levels, GmgOptions(scheme=scheme, smoother=0, cycle_type=cycle_type, cycle_dtype=te.TE_F32,
                                       bicgstab_flags=1))
    uv = te.Vector(s32.finest)
    s32.solve(fv, uv)
    assert s32.residual(fv, uv) <= 1e-10


def test_unknown_cycle_type(te):
    from thunderegg_gb300 import mesh as M
    from thunderegg_gb300.capi import TE_ERR_UNSUPPORTED, TeError
    from thunderegg_gb300.gmg import GmgOptions, GmgSolver

    with pytest.raises(TeError) as e:
        GmgSolver(M.uniform_mesh(2, 2, 8), GmgOptions(cycle_type="X"))
    assert e.value.code == TE_ERR_UNSUPPORTED


@pytest.mark.parametrize("idx", range(3))
@pytest.mark.parametrize("cycle_type", ("V", "W"))
def test_cg_matches_oracle(te, oracle, idx, cycle_type):
    """Iterative::CG (Iterative/CG.h:126-194) preconditioned by the FP64 cycle:
    the oracle's iteration count (pinned to the reference's CG by
    tests/test_oracle_pin.py) and its solution to the solver tolerance, from a
    nonzero initial guess."""
    from oracle import gmg_config
    from thunderegg_gb300.gmg import GmgOptions, GmgSolver

    name, levels, scheme = meshes()[idx]
    rng = np.random.default_rng(70 + idx)
    f = rng.standard_normal(levels[0].padded_shape(1))
    u0 = rng.standard_normal(levels[0].padded_shape(1))
    u_o, its_o, _, rc = oracle.solve(levels, f, gmg_config(scheme=scheme, smoother=0, cycle_type=cycle_type,
                                                           krylov="cg"), u0=u0)
    assert rc == 0
    s = GmgSolver(levels, GmgOptions(scheme=scheme, smoother=0, cycle_type=cycle_type, krylov="cg"))
    fv = te.Vector.from_numpy(s.finest, f)
    uv = te.Vector.from_numpy(s.finest, u0)
    assert s.solve(fv, uv) == its_o
    g = levels[0].num_ghost
    inner = (Ellipsis,) + tuple(slice(g, -g) for _ in range(levels[0].dim))
    assert rel_err(uv.numpy()[inner], u_o[inner]) <= 1e-8
    assert s.residual(fv, uv) <= 1e-9


def test_cg_unpreconditioned_and_zero_rhs(te, oracle):
    """CG without a preconditioner runs the oracle's iterations; a zero
    right-hand side returns at once with the interior zeroed."""
    from oracle import gmg_config
    from thunderegg_gb300 import mesh as M
    from thunderegg_gb300.gmg import GmgOptions, GmgSolver

    levels = M.uniform_mesh(2, 2, 8)
    rng = np.random.default_rng(80)
    f = rng.standard_normal(levels[0].padded_shape(1))
    u_o, its_o, _, rc = oracle.solve(levels, f, gmg_config(scheme=0, krylov="cg", use_precond=0, tol=1e-9))
    s = GmgSolver(levels, GmgOptions(scheme=0, krylov="cg", tol=1e-9))
    fv = te.Vector.from_numpy(s.finest, f)
    uv = te.Vector(s.finest)
    its = s.solve(fv, uv, precondition=False)
    assert abs(its - its_o) <= 1  # unpreconditioned CG: reduction order may move the last iteration
    inner = (Ellipsis, slice(1, -1), slice(1, -1))
    assert rel_err(uv.numpy()[inner], u_o[inner]) <= 1e-7
    zv = te.Vector(s.finest)
    uv = te.Vector.from_numpy(s.finest, rng.standard_normal(levels[0].padded_shape(1)))
    assert s.solve(zv, uv) == 0
    assert np.all(uv.numpy()[inner] == 0.0)
