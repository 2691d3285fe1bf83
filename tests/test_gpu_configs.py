"""The benchmark configurations at full size against the FP64 oracle.

Each GPU solve runs through the C ABI on exactly the oracle's inputs (mesh,
right-hand side, solver options) and is compared with oracle.solve:

  config 1  2D uniform L2, 16 patches of 32^2, BiLinear, BiCGStab patch smoother
            (inner BiCGStab tol 1e-12, 1000 iterations, continue on breakdown),
            V(1,1) to 1 patch, outer BiCGStab to 1e-10 -- the plain FP64 method
  config 2  2D circle-adaptive L3-7, 1444 patches of 32^2, BiQuadratic, DFT
            smoother: the FP64 drop-in and the mixed-precision solve
  config 3  3D uniform octree, TriLinear, DFT smoother, RHS N(0,1): at level 3
            (512 patches of 16^3, 2.1M cells) so the oracle finishes in seconds
  config 4  one variable-coefficient solve on its seeded random quadtree (16^2
            patches, BiQuadratic, BiCGStab patch smoother)

FP64 drop-in solves use the reference's BiCGStab update rule (flags 0) and
are compared with the oracle running the same rule: iteration counts equal,
solutions within SOL_TOL_FP64 (rounding differences only).  Mixed-precision
solves use the preconditioned early exit (flags 1); the oracle runs the same
rule in FP64, and the two converged solutions agree within SOL_TOL_MIXED.
Solutions are compared on interior cells, relative to max |u_oracle|.
"""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

# measured: FP64 drop-in 4e-16 .. 1.2e-13, mixed 3e-14 .. 2.7e-12
SOL_TOL_FP64 = 1e-12   # same iterations, same arithmetic up to summation order and FMA contraction
SOL_TOL_MIXED = 1e-10  # both at a true relative residual <= 1e-10 (the solver tolerance), different arithmetic


def _inner(lv):
    g = lv.num_ghost
    return (Ellipsis,) + tuple(slice(g, -g) for _ in range(lv.dim))


def _gpu_solve(te, levels, f, coeffs=None, **kw):
    from thunderegg_gb300.gmg import GmgOptions, GmgSolver

    s = GmgSolver(levels, GmgOptions(**kw), coeffs)
    fv = te.Vector.from_numpy(s.finest, f)
    uv = te.Vector(s.finest)
    its = s.solve(fv, uv)
    return uv.numpy(), its, s.residual(fv, uv)


def _oracle_solve(oracle, levels, f, coeffs=None, **kw):
    from oracle import gmg_config

    u, its, res, rc = oracle.solve(levels, f, gmg_config(**kw), coeffs=coeffs)
    assert rc == 0
    return u, its


def test_config1_fp64_dropin_matches_oracle(te, oracle):
    from thunderegg_gb300 import problems as PB

    levels, f, exact = PB.config1()
    assert [lv.num_patches for lv in levels] == [16, 4, 1]
    kw = dict(scheme=0, smoother=1, inner_tol=1e-12, inner_max_it=1000, inner_continue_on_breakdown=True, tol=1e-10)
    u_o, its_o = _oracle_solve(oracle, levels, f, scheme=0, smoother=1, inner_tol=1e-12, inner_max_it=1000,
                               inner_continue_on_breakdown=1, tol=1e-10)
    u, its, res = _gpu_solve(te, levels, f, **kw)
    inner = _inner(levels[0])
    err = rel_err(u[inner], u_o[inner])
    print(f"config1 fp64: its {its} (oracle {its_o}), true residual {res:.2e}, rel err vs oracle {err:.2e}")
    assert its == its_o
    assert err <= SOL_TOL_FP64
    # the discretisation error of the converged solution is the oracle's (about 5e-5 at h = 1/128)
    e_gpu = float(np.abs(u[inner] - exact[inner]).max())
    e_orc = float(np.abs(u_o[inner] - exact[inner]).max())
    assert abs(e_gpu - e_orc) <= 1e-9 and e_gpu < 1e-4


def test_config2_fp64_dropin_matches_oracle(te, oracle):
    from thunderegg_gb300 import problems as PB

    levels, f, _ = PB.config2()
    assert levels[0].num_patches == 1444 and len(levels) == 8
    u_o, its_o = _oracle_solve(oracle, levels, f, scheme=1, smoother=0, tol=1e-10)
    u, its, res = _gpu_solve(te, levels, f, scheme=1, smoother=0, tol=1e-10)
    inner = _inner(levels[0])
    err = rel_err(u[inner], u_o[inner])
    print(f"config2 fp64: its {its} (oracle {its_o}), true residual {res:.2e}, rel err vs oracle {err:.2e}")
    assert its == its_o
    assert err <= SOL_TOL_FP64


def test_config2_mixed_matches_oracle(te, oracle):
    from thunderegg_gb300 import problems as PB

    levels, f, _ = PB.config2()
    u_o, its_o = _oracle_solve(oracle, levels, f, scheme=1, smoother=0, tol=1e-10, precond_exit=1)
    u, its, res = _gpu_solve(te, levels, f, scheme=1, smoother=0, tol=1e-10, cycle_dtype=te.TE_F32,
                             bicgstab_flags=1)
    inner = _inner(levels[0])
    err = rel_err(u[inner], u_o[inner])
    print(f"config2 mixed: its {its} (oracle {its_o}), true residual {res:.2e}, rel err vs oracle {err:.2e}")
    assert res <= 1e-10
    assert abs(its - its_o) <= 2
    assert err <= SOL_TOL_MIXED


@pytest.mark.parametrize("cycle", ("fp64", "mixed"))
def test_config3_level3_matches_oracle(te, oracle, cycle):
    from thunderegg_gb300 import problems as PB

    levels, f, _ = PB.config3(level=3)
    assert levels[0].num_patches == 512 and levels[0].ns[0] == 16
    dt, flags = (te.TE_F64, 0) if cycle == "fp64" else (te.TE_F32, 1)
    u_o, its_o = _oracle_solve(oracle, levels, f, scheme=2, smoother=0, tol=1e-10, precond_exit=flags)
    u, its, res = _gpu_solve(te, levels, f, scheme=2, smoother=0, tol=1e-10, cycle_dtype=dt, bicgstab_flags=flags)
    inner = _inner(levels[0])
    err = rel_err(u[inner], u_o[inner])
    print(f"config3 L3 {cycle}: its {its} (oracle {its_o}), true residual {res:.2e}, rel err vs oracle {err:.2e}")
    if cycle == "fp64":
        assert its == its_o
        assert err <= SOL_TOL_FP64
    else:
        assert res <= 1e-10
        assert abs(its - its_o) <= 2
        assert err <= SOL_TOL_MIXED


@pytest.mark.parametrize("cycle", ("fp64", "mixed"))
def test_config4_varpoisson_tree_matches_oracle(te, oracle, cycle):
    from thunderegg_gb300 import problems as PB

    (levels, f, coeffs), = PB.config4(num_solves=1)
    assert levels[0].ns[0] == 16
    if cycle == "fp64":
        kw = dict(inner_tol=1e-12, cycle_dtype=te.TE_F64, bicgstab_flags=0)
        pe = 0
    else:
        # the FP32 cycle's patch smoother stops at 1e-5 relative: 1e-12 is below FP32 resolution
        kw = dict(inner_tol=1e-5, cycle_dtype=te.TE_F32, bicgstab_flags=1)
        pe = 1
    u_o, its_o = _oracle_solve(oracle, levels, f, coeffs=coeffs, scheme=1, smoother=1, op_kind=1, tol=1e-10,
                               inner_tol=1e-12, precond_exit=pe)
    u, its, res = _gpu_solve(te, levels, f, coeffs=coeffs, scheme=1, smoother=1, tol=1e-10, **kw)
    inner = _inner(levels[0])
    err = rel_err(u[inner], u_o[inner])
    print(f"config4 {cycle}: {levels[0].num_patches} patches, its {its} (oracle {its_o}), true residual {res:.2e}, "
          f"rel err vs oracle {err:.2e}")
    if cycle == "fp64":
        assert its == its_o
        assert err <= SOL_TOL_FP64
    else:
        assert res <= 1e-10
        assert err <= SOL_TOL_MIXED
