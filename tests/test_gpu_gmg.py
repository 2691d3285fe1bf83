"""GMG V-cycle and BiCGStab solves on the GPU against the CPU oracle.

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
