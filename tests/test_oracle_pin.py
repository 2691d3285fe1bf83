"""The CPU oracle (oracle/te_oracle.cpp) against ThunderEgg itself.

1. Against the committed golden fixtures (tests/golden/*.npz, written by
   tests/golden/make_golden.py from the reference compiled from its own
   sources): ghost fills, call tables, operator applies, RHS modification,
   both patch smoothers, restriction, interpolation, V-, W- and FMG cycles and a full
   GMG-BiCGStab solve.  The restatement reproduces them bit for bit.
2. Against the reference library live, where its sources are present.
"""
import glob
import os

import numpy as np
import pytest

from conftest import ROOT

GOLDEN = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "*.npz")))


def load(path):
    import sys

    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import make_golden as mg

    z = np.load(path)
    levels = mg.unpack_levels(z)
    schemes = tuple(int(s) for s in z["schemes"])
    return z, levels, schemes, mg.inputs(levels, schemes)


def test_golden_fixtures_present():
    assert len(GOLDEN) >= 6


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_oracle_matches_reference_fixtures(oracle, path):
    from oracle import gmg_config

    z, levels, schemes, inp = load(path)
    lv = levels[0]
    fts = (0, 2) if lv.dim == 2 else (0, 1, 2)
    for sc in schemes:
        for ft in fts:
            got = oracle.ghost_fill(lv, inp[f"fill_s{sc}_f{ft}_in"].copy(), sc, ft, 2)
            assert np.array_equal(got, z[f"fill_s{sc}_f{ft}_out"]), (sc, ft)
            assert np.array_equal(oracle.ghost_calls(lv, ft), z[f"calls_f{ft}"])
    sc = schemes[0]
    coeffs = inp["coeffs"]
    for kind in (0, 1):
        uo, fo = oracle.apply(lv, inp[f"apply_k{kind}_in"].copy(), sc, 0, kind, 0, coeffs if kind else None)
        assert np.array_equal(fo, z[f"apply_k{kind}_f"]) and np.array_equal(uo, z[f"apply_k{kind}_u"])
        got = oracle.modify_rhs(lv, uo, inp[f"modrhs_k{kind}_f"], sc, 0, kind, coeffs if kind else None)
        assert np.array_equal(got, z[f"modrhs_k{kind}_out"])
    for sm in (0, 1):
        for mode in (0, 1):
            got, _ = oracle.patch_solver(lv, inp["ps_f"], inp["ps_u"], sc, smoother=sm, mode=mode)
            assert np.array_equal(got, z[f"ps_s{sm}_m{mode}"]), (sm, mode)
    if len(levels) > 1:
        for ex in (0, 1):
            assert np.array_equal(oracle.restrict(levels[0], levels[1], inp["tr_fine"], ex), z[f"restrict_e{ex}"])
        assert np.array_equal(oracle.interpolate(levels[1], levels[0], inp["tr_coarse"], inp["tr_fine"]), z["interp"])
        cfg = gmg_config(scheme=sc, smoother=0, tol=1e-10)
        assert np.array_equal(oracle.vcycle(levels, inp["gmg_f"], cfg), z["vcycle"])
        for ct in ("W", "F"):
            cfg_t = gmg_config(scheme=sc, smoother=0, tol=1e-10, cycle_type=ct)
            assert np.array_equal(oracle.vcycle(levels, inp["gmg_f"], cfg_t), z[f"cycle_{ct}"]), ct
        u, its, res, rc = oracle.solve(levels, inp["gmg_f"], cfg)
        g = lv.num_ghost
        inner = (Ellipsis,) + tuple(slice(g, -g) for _ in range(lv.dim))
        assert its == int(z["solve_its"]) and np.array_equal(u[inner], z["solve_u"][inner])


def test_oracle_matches_reference_live(oracle, ref):
    """Oracle and reference on fresh meshes and inputs (reference sources needed)."""
    from oracle import gmg_config
    from thunderegg_gb300 import mesh as M

    rng = np.random.default_rng(99)
    for levels, sc in ((M.circle_mesh(n=6, lo=1, hi=4), 1), (M.random_mesh(11, n=4, dim=3, lo=1, hi=3), 2)):
        lv = levels[0]
        for ft in ((0, 2) if lv.dim == 2 else (0, 1, 2)):
            u = rng.standard_normal(lv.padded_shape(1))
            assert np.array_equal(oracle.ghost_fill(lv, u.copy(), sc, ft), ref.ghost_fill(lv, u.copy(), sc, ft))
            assert np.array_equal(oracle.ghost_calls(lv, ft), ref.ghost_calls(lv, ft))
        f = rng.standard_normal(lv.padded_shape(1))
        for sm in (0, 1):
            for ct in ("V", "W", "F"):
                cfg = gmg_config(scheme=sc, smoother=sm, cycle_type=ct, mid_sweeps=1 + sm)
                assert np.array_equal(oracle.vcycle(levels, f, cfg), ref.vcycle(levels, f, cfg)), (sm, ct)


def test_reference_bicgstab_early_exit_quirk(oracle):
    """The reference's BiCGStab adds alpha*p (not alpha*M p) on its early exit
    (Iterative/BiCGStab.h:160-168), so a preconditioned solve can stop with a
    true residual far above the tolerance.  The oracle reproduces that."""
    from oracle import gmg_config
    from thunderegg_gb300 import mesh as M

    levels = M.uniform_mesh(2, 2, 8)
    lv = levels[0]
    f = np.random.default_rng(0).standard_normal(lv.padded_shape(1))
    u, its, res, rc = oracle.solve(levels, f, gmg_config(scheme=0, tol=1e-10))
    _, Au = oracle.apply(lv, u.copy(), 0)
    inner = (Ellipsis, slice(1, -1), slice(1, -1))
    true_res = np.linalg.norm((f - Au)[inner]) / np.linalg.norm(f[inner])
    assert rc == 0 and its < 20 and true_res > 1e-8


def test_oracle_cg_matches_reference_live(oracle, ref):
    """The oracle's CG (te_oracle.cpp cg) against Iterative::CG itself, with and
    without the V/W/FMG cycle as preconditioner, from a nonzero initial guess,
    and the zero right-hand-side early return."""
    from oracle import gmg_config
    from thunderegg_gb300 import mesh as M

    rng = np.random.default_rng(7)
    for levels, sc in ((M.circle_mesh(n=6, lo=1, hi=4), 1), (M.random_mesh(11, n=4, dim=3, lo=1, hi=3), 2)):
        lv = levels[0]
        g = lv.num_ghost
        inner = (Ellipsis,) + tuple(slice(g, -g) for _ in range(lv.dim))
        f = rng.standard_normal(lv.padded_shape(1))
        u0 = rng.standard_normal(lv.padded_shape(1))
        for pre, ct in ((1, "V"), (1, "W"), (1, "F"), (0, "V")):
            cfg = gmg_config(scheme=sc, smoother=0, cycle_type=ct, tol=1e-10, krylov="cg", use_precond=pre,
                             max_it=200)
            a, b = oracle.solve(levels, f, cfg, u0=u0), ref.solve(levels, f, cfg, u0=u0)
            assert a[1] == b[1] and a[3] == b[3] and np.array_equal(a[0][inner], b[0][inner]), (pre, ct)
        z = np.zeros_like(f)
        a, b = oracle.solve(levels, z, gmg_config(scheme=sc, krylov="cg"), u0=u0), \
            ref.solve(levels, z, gmg_config(scheme=sc, krylov="cg"), u0=u0)
        assert a[1] == b[1] == 0 and np.array_equal(a[0][inner], b[0][inner])


def test_oracle_matches_reference_live_operators_and_transfers(oracle, ref):
    """The rows the cycle test does not reach directly, against the compiled reference:
    BiLinear fills, Poisson with Dirichlet and Neumann boundaries, VarPoisson, modifyRHS,
    both patch solvers (smooth and apply), the DFT solver with Neumann sides,
    restriction with and without boundary extrapolation, interpolation, and a
    VarPoisson BiCGStab solve."""
    from oracle import gmg_config
    from thunderegg_gb300 import mesh as M

    rng = np.random.default_rng(123)
    cases = ((M.random_mesh(3, n=6, dim=2, lo=1, hi=4), 0), (M.circle_mesh(n=6, lo=1, hi=4), 1),
             (M.random_mesh(11, n=4, dim=3, lo=1, hi=3), 2))
    for levels, sc in cases:
        lv = levels[0]
        shape = lv.padded_shape(1)
        u, f = rng.standard_normal(shape), rng.standard_normal(shape)
        coeffs = [1.0 + rng.random(l.padded_shape(1)) for l in levels]
        for ft in ((0, 2) if lv.dim == 2 else (0, 1, 2)):
            assert np.array_equal(oracle.ghost_fill(lv, u.copy(), sc, ft), ref.ghost_fill(lv, u.copy(), sc, ft))
        for kind, neumann in ((0, 0), (0, 1), (1, 0)):
            c = coeffs[0] if kind else None
            a, b = oracle.apply(lv, u.copy(), sc, kind=kind, neumann=neumann, coeffs=c), \
                ref.apply(lv, u.copy(), sc, kind=kind, neumann=neumann, coeffs=c)
            assert np.array_equal(a[1], b[1]), (sc, kind, neumann)
            if neumann == 0:
                assert np.array_equal(oracle.modify_rhs(lv, u, f, sc, kind=kind, coeffs=c),
                                      ref.modify_rhs(lv, u, f, sc, kind=kind, coeffs=c)), (sc, kind)
        for kind, smoother in ((0, 0), (0, 1), (1, 1)):
            c = coeffs[0] if kind else None
            for mode in (0, 1):
                a = oracle.patch_solver(lv, f, u, sc, kind=kind, coeffs=c, smoother=smoother, mode=mode)
                b = ref.patch_solver(lv, f, u, sc, kind=kind, coeffs=c, smoother=smoother, mode=mode)
                # the reference's PatchSolver does not report inner iterations (the wrapper gives -1)
                assert np.array_equal(a[0], b[0]), (sc, kind, smoother, mode)
        # the DFT solver with Neumann sides (DCT plans at the domain boundary, DFTPatchSolver.h:141-191)
        for mask in (1, (1 << (2 * lv.dim)) - 1):
            for mode in (0, 1):
                a = oracle.patch_solver(lv, f, u, sc, smoother=0, dft_neumann_mask=mask, mode=mode)
                b = ref.patch_solver(lv, f, u, sc, smoother=0, dft_neumann_mask=mask, mode=mode)
                assert np.array_equal(a[0], b[0]), (sc, mask, mode)
        for extrap in (0, 1):
            assert np.array_equal(oracle.restrict(lv, levels[1], u, extrap), ref.restrict(lv, levels[1], u, extrap))
        vc = rng.standard_normal(levels[1].padded_shape(1))
        assert np.array_equal(oracle.interpolate(levels[1], lv, vc, u), ref.interpolate(levels[1], lv, vc, u))
        # the solution's interior (its ghost cells hold whatever the last ghost fill left)
        g = lv.num_ghost
        inner = (Ellipsis,) + tuple(slice(g, -g) for _ in range(lv.dim))
        cfg = gmg_config(scheme=sc, op_kind=1, smoother=1, tol=1e-9, max_it=100)
        a, b = oracle.solve(levels, f, cfg, coeffs=coeffs), ref.solve(levels, f, cfg, coeffs=coeffs)
        assert a[1] == b[1] and a[3] == b[3] and np.array_equal(a[0][inner], b[0][inner]), sc


def _bc_meshes():
    from thunderegg_gb300 import mesh as M

    return [M.circle_mesh(n=8, lo=2, hi=4)[0], M.random_mesh(4, n=5, lo=1, hi=4)[0],
            M.random_mesh(5, n=4, dim=3, lo=1, hi=3)[0]]


# boundary data: a polynomial (exactly the same in every evaluation order) and a transcendental one
_BC_FUNCS = {
    2: (lambda x, y: 1.5 + x * x - 0.25 * x * y + y, lambda x, y: 2 * x - 0.25 * y, lambda x, y: 1.0 - 0.25 * x,
        lambda x, y: np.exp(x * y)),
    3: (lambda x, y, z: 1 + x * y - z * z + 0.5 * x, lambda x, y, z: y + 0.5, lambda x, y, z: x,
        lambda x, y, z: np.exp(x * y * z)),
}


@pytest.mark.parametrize("idx", range(3))
def test_oracle_bc_rhs_helpers_match_reference_live(oracle, ref, idx):
    """addDrichletBCToRHS / addNeumannBCToRHS (Poisson) and VarPoisson's addDrichletBCToRHS:
    the restatement adds the same terms to the same cells in the same order as the reference."""
    lv = _bc_meshes()[idx]
    D = lv.dim
    g, *grad, gexp = _BC_FUNCS[D]
    if D == 3:
        grad = [lambda x, y, z: y + 0.5, lambda x, y, z: x, lambda x, y, z: -2 * z]
    coef = (lambda x, y: 1 + 0.5 * x) if D == 2 else (lambda x, y, z: 1 + 0.5 * x * z)
    f = np.random.default_rng(50 + idx).standard_normal(lv.padded_shape(1))
    for kw in (dict(gfun=g), dict(gfun=gexp), dict(gfun=g, grad=grad, neumann=1), dict(gfun=g, hfun=coef, kind=1)):
        want = ref.add_bc_to_rhs(lv, f, **kw)
        got = oracle.add_bc_to_rhs(lv, f, **kw)
        assert np.array_equal(got, want), kw.keys()
        assert not np.array_equal(got, f)
