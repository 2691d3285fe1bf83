"""The float-float outer BiCGStab (mixed precision) against the FP64 outer loop and the oracle.

With an FP32 V-cycle as preconditioner the outer iteration runs in float-float
arithmetic (~48 significant bits).  Tolerances:
  true FP64 residual ||f - A u|| / ||f|| after the solve: <= 1e-10 (the target)
  iterations: within 1 of the FP64 outer loop with the same cycle
  solution vs the FP64-outer solution: <= 1e-8 relative (both stop at 1e-10)
"""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


def _cases():
    from thunderegg_gb300 import mesh as M

    return {
        "2d_circle_n16_dft": (M.circle_mesh(n=16, lo=2, hi=4), 1, 0, False),   # tensor-core DFT cycle
        "2d_circle_n8_dft": (M.circle_mesh(n=8, lo=2, hi=5), 1, 0, False),     # SIMT DFT cycle
        "2d_random_n8_bicg": (M.random_mesh(3, n=8, lo=1, hi=4), 0, 1, False),  # BiCGStab smoother, unfused
        "2d_random_n8_var": (M.random_mesh(4, n=8, lo=1, hi=4), 1, 1, True),    # VarPoisson
        "3d_uniform_n16_dft": (M.uniform_mesh(3, 1, 16), 2, 0, False),
    }


CASES = None


def cases():
    global CASES
    if CASES is None:
        CASES = _cases()
    return CASES


@pytest.mark.parametrize("name", ["2d_circle_n16_dft", "2d_circle_n8_dft", "2d_random_n8_bicg", "2d_random_n8_var",
                                  "3d_uniform_n16_dft"])
def test_float_float_outer_matches_fp64_outer(te, name):
    from thunderegg_gb300 import problems as PB
    from thunderegg_gb300.gmg import GmgOptions, GmgSolver

    levels, scheme, smoother, var = cases()[name]
    coeffs = PB.beta_coeffs(levels) if var else None
    f = np.random.default_rng(21).standard_normal(levels[0].padded_shape(1))
    sols, its = [], []
    for flags in (1, 1 | 2):  # float-float outer loop, then FP64 outer loop
        s = GmgSolver(levels, GmgOptions(scheme=scheme, smoother=smoother, cycle_dtype=te.TE_F32,
                                         bicgstab_flags=flags), coeffs)
        fv, uv = te.Vector.from_numpy(s.finest, f), te.Vector(s.finest)
        its.append(s.solve(fv, uv))
        assert s.residual(fv, uv) <= 1e-10, (name, flags)
        sols.append(uv.numpy())
    assert abs(its[0] - its[1]) <= 1, its
    g = levels[0].num_ghost
    inner = (Ellipsis,) + tuple(slice(g, -g) for _ in range(levels[0].dim))
    assert rel_err(sols[0][inner], sols[1][inner]) <= 1e-8


def test_float_float_outer_matches_oracle_solution(te, oracle):
    """The mixed-precision solve against the FP64 oracle solve of the same problem."""
    from oracle import gmg_config
    from thunderegg_gb300.gmg import GmgOptions, GmgSolver

    levels, scheme, smoother, _ = cases()["2d_circle_n8_dft"]
    f = np.random.default_rng(22).standard_normal(levels[0].padded_shape(1))
    u_o, its_o, _, rc = oracle.solve(levels, f, gmg_config(scheme=scheme, smoother=smoother, tol=1e-12))
    s = GmgSolver(levels, GmgOptions(scheme=scheme, smoother=smoother, cycle_dtype=te.TE_F32, bicgstab_flags=1))
    fv, uv = te.Vector.from_numpy(s.finest, f), te.Vector(s.finest)
    s.solve(fv, uv)
    assert s.residual(fv, uv) <= 1e-10
    inner = (Ellipsis, slice(1, -1), slice(1, -1))
    assert rel_err(uv.numpy()[inner], u_o[inner]) <= 1e-7


def test_float_float_nonzero_initial_guess(te):
    """x enters in FP64, is carried as float-float and leaves in FP64."""
    from thunderegg_gb300 import mesh as M
    from thunderegg_gb300.gmg import GmgOptions, GmgSolver

    levels = M.circle_mesh(n=16, lo=2, hi=4)
    rng = np.random.default_rng(23)
    f = rng.standard_normal(levels[0].padded_shape(1))
    u0 = rng.standard_normal(levels[0].padded_shape(1))
    s = GmgSolver(levels, GmgOptions(scheme=1, smoother=0, cycle_dtype=te.TE_F32, bicgstab_flags=1))
    fv, uv = te.Vector.from_numpy(s.finest, f), te.Vector.from_numpy(s.finest, u0)
    s.solve(fv, uv)
    assert s.residual(fv, uv) <= 1e-10
