"""BF16 tensor-core transforms (per-patch scaled) and FP64 iterative refinement.

The BF16 patch solve keeps 8 significant bits per operand: it is compared with
the FP64 oracle at BF16_TOL (infinity-norm relative, per patch).  Its
per-patch power-of-two scaling makes each patch's result independent of the
patch's magnitude: patches scaled from 1e-30 to 1e30 (whose results span
1e-34 .. 1e26) keep the same relative error, and scaling a
patch by a power of two scales its result exactly.

Iterative refinement (x += M (b - A x), true FP64 residual every iteration)
with the FP32 cycle -- BF16 or 3xTF32 transforms -- reaches a 1e-10 relative
FP64 residual, and its solution agrees with the oracle's FP64 BiCGStab solve
within SOL_TOL.
"""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

BF16_TOL = 3e-2   # 8-bit operands over four transform passes
SOL_TOL = 1e-9    # two solutions at a relative residual <= 1e-10 (cond ~ 1e2..1e3 on these meshes)


def _meshes():
    from thunderegg_gb300 import mesh as M

    return {
        "2d_uniform_n16": (M.uniform_mesh(2, 2, 16), 0),
        "2d_uniform_n32": (M.uniform_mesh(2, 2, 32), 1),
        "2d_uniform_n64": (M.uniform_mesh(2, 1, 64), 1),
        "2d_circle_n16": (M.circle_mesh(n=16, lo=2, hi=4), 1),
        "3d_uniform_n16": (M.uniform_mesh(3, 1, 16), 2),
    }


def _inner(lv):
    g = lv.num_ghost
    return (Ellipsis,) + tuple(slice(g, -g) for _ in range(lv.dim))


def _bf16_solver(te, lv, scheme):
    dom = te.Domain(lv)
    filler = [te.BiLinearGhostFiller, te.BiQuadraticGhostFiller, te.TriLinearGhostFiller][scheme](dom)
    op = te.PoissonStarPatchOperator(dom, filler)
    ps = te.DFTPatchSolver(op, 0, te.capi.TE_TC_BF16)
    assert ps.uses_tensor_cores
    return dom, ps


def _per_patch_rel_err(got, want):
    P = want.shape[0]
    g = got.reshape(P, -1)
    w = want.reshape(P, -1)
    return float(max(np.abs(g[p] - w[p]).max() / max(np.abs(w[p]).max(), 1e-300) for p in range(P)))


@pytest.mark.parametrize("name", sorted(_meshes().keys()))
def test_bf16_patch_solve_matches_oracle(te, oracle, name):
    levels, sc = _meshes()[name]
    lv = levels[0]
    dom, ps = _bf16_solver(te, lv, sc)
    rng = np.random.default_rng(31)
    f = rng.standard_normal(lv.padded_shape(1))
    want, _ = oracle.patch_solver(lv, f, np.zeros_like(f), sc, smoother=0, mode=1)
    u = te.Vector(dom, 1, te.TE_F32)
    ps.apply(te.Vector.from_numpy(dom, f, dtype=te.TE_F32), u)
    inner = _inner(lv)
    err = _per_patch_rel_err(u.numpy()[inner], want[inner])
    print(f"{name}: BF16 patch solve, max per-patch rel err vs FP64 oracle {err:.2e}")
    assert err <= BF16_TOL


def test_bf16_per_patch_scaling(te, oracle):
    """Patch magnitudes from 1e-30 to 1e30: the per-patch relative error stays at the BF16 level,
    and multiplying a right-hand side by 2^k multiplies the solve by exactly 2^k."""
    levels, sc = _meshes()["2d_uniform_n32"]
    lv = levels[0]
    dom, ps = _bf16_solver(te, lv, sc)
    rng = np.random.default_rng(32)
    base = rng.standard_normal(lv.padded_shape(1)).astype(np.float32).astype(np.float64)
    mags = np.array([10.0 ** e for e in np.linspace(-30, 30, lv.num_patches)])
    f = base * mags[:, None, None, None]
    want, _ = oracle.patch_solver(lv, f, np.zeros_like(f), sc, smoother=0, mode=1)
    u = te.Vector(dom, 1, te.TE_F32)
    ps.apply(te.Vector.from_numpy(dom, f, dtype=te.TE_F32), u)
    inner = _inner(lv)
    got = u.numpy()[inner]
    assert np.all(np.isfinite(got))
    assert _per_patch_rel_err(got, want[inner]) <= BF16_TOL
    u1 = te.Vector(dom, 1, te.TE_F32)
    u2 = te.Vector(dom, 1, te.TE_F32)
    ps.apply(te.Vector.from_numpy(dom, base, dtype=te.TE_F32), u1)
    ps.apply(te.Vector.from_numpy(dom, base * 2.0 ** 40, dtype=te.TE_F32), u2)
    assert np.array_equal(u2.numpy(), u1.numpy() * 2.0 ** 40)


@pytest.mark.parametrize("name", ["2d_circle_n16", "3d_uniform_n16"])
@pytest.mark.parametrize("tc", ("bf16", "tf32x3"))
def test_ir_with_fp32_cycle_reaches_tolerance(te, oracle, name, tc):
    from oracle import gmg_config
    from thunderegg_gb300.gmg import GmgOptions, GmgSolver

    levels, sc = _meshes()[name]
    f = np.random.default_rng(33).standard_normal(levels[0].padded_shape(1))
    u_o, its_o, _, rc = oracle.solve(levels, f, gmg_config(scheme=sc, smoother=0, tol=1e-10, precond_exit=1))
    assert rc == 0
    prec = te.capi.TE_TC_BF16 if tc == "bf16" else te.capi.TE_TC_TF32X3
    s = GmgSolver(levels, GmgOptions(scheme=sc, smoother=0, cycle_dtype=te.TE_F32, krylov="ir", tc_precision=prec,
                                     max_it=200))
    fv, uv = te.Vector.from_numpy(s.finest, f), te.Vector(s.finest)
    its = s.solve(fv, uv)
    res = s.residual(fv, uv)
    inner = _inner(levels[0])
    err = rel_err(uv.numpy()[inner], u_o[inner])
    print(f"{name} IR ({tc} transforms): {its} iterations, true residual {res:.2e} "
          f"(reported {s.krylov.final_residual:.2e}), rel err vs oracle {err:.2e}")
    assert its < 200
    assert res <= 1e-10
    assert abs(res - s.krylov.final_residual) <= 1e-3 * res + 1e-16
    assert err <= SOL_TOL


def test_bicgstab_with_bf16_cycle_reaches_tolerance(te):
    from thunderegg_gb300.gmg import GmgOptions, GmgSolver

    levels, sc = _meshes()["2d_circle_n16"]
    f = np.random.default_rng(34).standard_normal(levels[0].padded_shape(1))
    s = GmgSolver(levels, GmgOptions(scheme=sc, smoother=0, cycle_dtype=te.TE_F32, bicgstab_flags=1,
                                     tc_precision=te.capi.TE_TC_BF16))
    fv, uv = te.Vector.from_numpy(s.finest, f), te.Vector(s.finest)
    its = s.solve(fv, uv)
    assert its < 60
    assert s.residual(fv, uv) <= 1e-10


def test_ir_fp64_cycle_and_edge_cases(te, oracle):
    from oracle import gmg_config
    from thunderegg_gb300.gmg import GmgOptions, GmgSolver

    levels, sc = _meshes()["2d_uniform_n16"]
    f = np.random.default_rng(35).standard_normal(levels[0].padded_shape(1))
    u_o, _, _, _ = oracle.solve(levels, f, gmg_config(scheme=sc, smoother=0, tol=1e-10, precond_exit=1))
    s = GmgSolver(levels, GmgOptions(scheme=sc, smoother=0, krylov="ir", max_it=200))
    fv, uv = te.Vector.from_numpy(s.finest, f), te.Vector(s.finest)
    s.solve(fv, uv)
    assert s.residual(fv, uv) <= 1e-10
    assert rel_err(uv.numpy()[_inner(levels[0])], u_o[_inner(levels[0])]) <= SOL_TOL
    # zero right-hand side: returns at once, x unchanged
    z = te.Vector(s.finest)
    x0 = np.random.default_rng(36).standard_normal(levels[0].padded_shape(1))
    xv = te.Vector.from_numpy(s.finest, x0)
    assert s.solve(z, xv) == 0
    assert np.array_equal(xv.numpy(), x0)
    # a non-finite right-hand side is a breakdown
    bad = f.copy()
    bad[0, 0, 3, 3] = np.nan
    with pytest.raises(te.BreakdownError):
        s.solve(te.Vector.from_numpy(s.finest, bad), te.Vector(s.finest))
    # the refinement needs a cycle
    with pytest.raises(RuntimeError):
        s.krylov.solve(s.ops[0], te.Vector(s.finest), fv, None)
