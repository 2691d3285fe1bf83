"""GPU path against ThunderEgg's own outputs (tests/golden/*.npz, written by
tests/golden/make_golden.py from the reference compiled from its sources).

Tolerances (max|gpu - ref| / max|ref|): FP64 ghost fill, apply, modifyRHS,
restriction, interpolation 1e-13; DFT patch solve and V-cycle 1e-12;
BiCGStab patch solver 1e-8 (inner tolerance 1e-12); converged solve: same
iteration count, solution within 1e-8.  Call tables are bit-exact.
"""
import glob
import os

import numpy as np
import pytest

from conftest import ROOT, rel_err
from test_oracle_pin import load

pytestmark = pytest.mark.gpu
GOLDEN = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "*.npz")))


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_gpu_matches_reference_fixtures(te, path):
    from thunderegg_gb300.gmg import GmgOptions, GmgSolver

    z, levels, schemes, inp = load(path)
    lv = levels[0]
    dom = te.Domain(lv)
    fillers = [te.BiLinearGhostFiller, te.BiQuadraticGhostFiller, te.TriLinearGhostFiller]
    g = lv.num_ghost
    inner = (Ellipsis,) + tuple(slice(g, -g) for _ in range(lv.dim))
    for sc in schemes:
        for ft in ((0, 2) if lv.dim == 2 else (0, 1, 2)):
            gf = fillers[sc](dom, ft)
            assert np.array_equal(gf.calls(), z[f"calls_f{ft}"])
            v = te.Vector.from_numpy(dom, inp[f"fill_s{sc}_f{ft}_in"])
            gf.fillGhost(v)
            assert rel_err(v.numpy(), z[f"fill_s{sc}_f{ft}_out"]) <= 1e-13, (sc, ft)
    sc = schemes[0]
    gf = fillers[sc](dom)
    for kind in (0, 1):
        if kind:
            op = te.VarPoissonStarPatchOperator(te.Vector.from_numpy(dom, inp["coeffs"]), dom, gf)
        else:
            op = te.PoissonStarPatchOperator(dom, gf)
        u = te.Vector.from_numpy(dom, inp[f"apply_k{kind}_in"])
        f = te.Vector(dom)
        op.apply(u, f)
        assert rel_err(f.numpy(), z[f"apply_k{kind}_f"]) <= 1e-13
        assert rel_err(u.numpy(), z[f"apply_k{kind}_u"]) <= 1e-13
        fm = te.Vector.from_numpy(dom, inp[f"modrhs_k{kind}_f"])
        op.modifyRHSForInternalBoundaryConditions(te.Vector.from_numpy(dom, z[f"apply_k{kind}_u"]), fm)
        assert rel_err(fm.numpy(), z[f"modrhs_k{kind}_out"]) <= 1e-13
    op = te.PoissonStarPatchOperator(dom, gf)
    for sm, tol in ((0, 1e-12), (1, 1e-8)):
        ps = te.DFTPatchSolver(op) if sm == 0 else te.BiCGStabPatchSolver(op, 1e-12, 1000, True)
        for mode in (0, 1):
            u = te.Vector.from_numpy(dom, inp["ps_u"])
            (ps.smooth if mode == 0 else ps.apply)(te.Vector.from_numpy(dom, inp["ps_f"]), u)
            assert rel_err(u.numpy()[inner], z[f"ps_s{sm}_m{mode}"][inner]) <= tol, (sm, mode)
    if len(levels) > 1:
        doms = [dom, te.Domain(levels[1])]
        for ex in (0, 1):
            r = te.LinearRestrictor(doms[0], doms[1], bool(ex))
            got = r.restrict(te.Vector.from_numpy(doms[0], inp["tr_fine"]))
            assert rel_err(got.numpy(), z[f"restrict_e{ex}"]) <= 1e-13
        fv = te.Vector.from_numpy(doms[0], inp["tr_fine"])
        te.DirectInterpolator(doms[1], doms[0]).interpolate(te.Vector.from_numpy(doms[1], inp["tr_coarse"]), fv)
        assert rel_err(fv.numpy(), z["interp"]) <= 1e-13
        s = GmgSolver(levels, GmgOptions(scheme=sc, smoother=0, tol=1e-10))
        fg = te.Vector.from_numpy(s.finest, inp["gmg_f"])
        uv = te.Vector(s.finest)
        s.cycle.apply(fg, uv)
        assert rel_err(uv.numpy()[inner], z["vcycle"][inner]) <= 1e-12
        uv = te.Vector(s.finest)
        its = s.solve(fg, uv)
        assert its == int(z["solve_its"])
        assert rel_err(uv.numpy()[inner], z["solve_u"][inner]) <= 1e-8
