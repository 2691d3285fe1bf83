"""BiCGStab.solve(..., output=True, os=...) prints the reference's progress
lines ("%5d %16.8e", Iterative/BiCGStab.h:134-139,193-197): one before the
first iteration and one after each, and gives the same iterate and count as
the solve without output."""
import io

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_bicgstab_output_lines(te):
    from thunderegg_gb300 import mesh as M
    from thunderegg_gb300 import problems as PB
    from thunderegg_gb300.gmg import GmgOptions, GmgSolver

    levels = M.circle_mesh(n=8, lo=2, hi=4)
    s = GmgSolver(levels, GmgOptions(scheme=1, smoother=0, tol=1e-10))
    f = PB.sine_modes_rhs(levels[0], np.random.default_rng(62))
    fv = te.Vector.from_numpy(s.finest, f)
    quiet, loud = te.Vector(s.finest), te.Vector(s.finest)
    its = s.krylov.solve(s.ops[0], quiet, fv, s.cycle)
    buf = io.StringIO()
    its2 = s.krylov.solve(s.ops[0], loud, fv, s.cycle, output=True, os=buf)
    assert its2 == its
    lines = buf.getvalue().splitlines()
    assert len(lines) == its + 1
    for k, line in enumerate(lines):
        assert len(line) == 22 and int(line[:5]) == k  # "%5d %16.8e"
    assert float(lines[0][6:]) == pytest.approx(1.0)  # x = 0: the first residual is ||b|| / ||b||
    # the last line is the last full iteration's residual; a solve that stops on ||s||
    # (BiCGStab.h:160-166) prints nothing for that half step, as in the reference
    assert s.krylov.final_residual <= 1e-10
    assert np.array_equal(loud.numpy(), quiet.numpy())
