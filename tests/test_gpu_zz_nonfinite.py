"""A non-finite right-hand side or residual ends that solve with a breakdown
status instead of iterating on NaN to the iteration limit (host-side checks of
the per-solve scalars in csrc/te_krylov.cu).  The reference has no such check:
its comparisons with NaN are false, so it returns at once on a NaN right-hand
side and iterates to the limit on a NaN residual.  The other solves of a batch
are unaffected: their results stay bit-identical to the same solves alone.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_nan_rhs_is_a_breakdown_and_leaves_the_batch_intact(te):
    from thunderegg_gb300 import mesh as M
    from thunderegg_gb300 import problems as PB
    from thunderegg_gb300.capi import TE_ERR_BREAKDOWN
    from thunderegg_gb300.gmg import GmgOptions, GmgSolver

    hiers = [M.circle_mesh(n=8, lo=2, hi=5) for _ in range(3)]
    rng = np.random.default_rng(61)
    fs = [PB.sine_modes_rhs(h[0], rng) for h in hiers]
    fs[1][3, 0, 2, 2] = np.nan  # one interior cell of solve 1
    opts = GmgOptions(scheme=1, smoother=0, cycle_dtype=te.TE_F32, bicgstab_flags=1)
    levels, offsets = M.union_hierarchy(hiers)
    s = GmgSolver(levels, opts)
    fv = te.Vector.from_numpy(s.finest, np.concatenate(fs, axis=0))
    uv = te.Vector(s.finest)
    its, res, st = s.solve_batched(fv, uv, offsets[0])
    assert st[1] == TE_ERR_BREAKDOWN and its[1] == 0
    assert st[0] == 0 and st[2] == 0 and res[0] <= 1e-10 and res[2] <= 1e-10
    mixed = uv.numpy()
    inner = (Ellipsis, slice(1, -1), slice(1, -1))
    for b in (0, 2):
        one = GmgSolver(hiers[b], opts)
        u1 = te.Vector(one.finest)
        its1, _, _ = one.solve_batched(te.Vector.from_numpy(one.finest, fs[b]), u1, [0, hiers[b][0].num_patches])
        assert its1[0] == its[b]
        assert np.array_equal(mixed[offsets[0][b]:offsets[0][b + 1]][inner], u1.numpy()[inner])
    # the single-solve entry point raises the reference's exception type
    one = GmgSolver(hiers[1], opts)
    with pytest.raises(te.BreakdownError):
        one.solve(te.Vector.from_numpy(one.finest, fs[1]), te.Vector(one.finest))
