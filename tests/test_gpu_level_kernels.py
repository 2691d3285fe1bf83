"""Constant-size level kernels against the CPU oracle, through the C ABI.

Levels of cubic patches with one ghost layer (2D n = 8, 16, 32, 64; 3D n = 8,
16) run ghost fill, operator apply, restriction and interpolation through
kernels with constant index arithmetic; other shapes (and any level with
TE_GENERIC_LEVEL_KERNELS=1) run the general kernels.  Both must match the
oracle.  Tolerances (infinity-norm relative): FP64 1e-13, FP32 2e-6.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _cases():
    from thunderegg_gb300 import mesh as M

    return {
        "2d_circle_16": (M.circle_mesh(n=16, lo=2, hi=4), (0, 1)),
        "2d_circle_32": (M.circle_mesh(n=32, lo=2, hi=4), (1,)),
        "2d_uniform_64": (M.uniform_mesh(2, 2, 64), (1,)),
        "3d_random_8": (M.random_mesh(5, n=8, dim=3, lo=1, hi=3), (2,)),
    }


CASES = None


def cases():
    global CASES
    if CASES is None:
        CASES = _cases()
    return CASES


NAMES = ["2d_circle_16", "2d_circle_32", "2d_uniform_64", "3d_random_8"]


@pytest.mark.parametrize("name", NAMES)
def test_ghost_fill_fixed_size(te, oracle, name):
    levels, schemes = cases()[name]
    lv = levels[0]
    rng = np.random.default_rng(11)
    dom = te.Domain(lv)
    fill_types = (0, 2) if lv.dim == 2 else (0, 1, 2)
    for sc in schemes:
        cls = [te.BiLinearGhostFiller, te.BiQuadraticGhostFiller, te.TriLinearGhostFiller][sc]
        for ft in fill_types:
            gf = cls(dom, ft)
            for nc in (1, 2):
                u = rng.standard_normal(lv.padded_shape(nc))
                want = oracle.ghost_fill(lv, u.copy(), sc, ft, nc)
                v = te.Vector.from_numpy(dom, u)
                gf.fillGhost(v)
                assert rel_err(v.numpy(), want) <= 1e-13, (sc, ft, nc)
                v32 = te.Vector.from_numpy(dom, u, dtype=te.TE_F32)
                gf.fillGhost(v32)
                assert rel_err(v32.numpy(), want) <= 2e-6, (sc, ft, nc)


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("kind", (0, 1))
def test_operator_apply_fixed_size(te, oracle, name, kind):
    levels, schemes = cases()[name]
    lv = levels[0]
    rng = np.random.default_rng(12)
    dom = te.Domain(lv)
    sc = schemes[-1]
    gf = [te.BiLinearGhostFiller, te.BiQuadraticGhostFiller, te.TriLinearGhostFiller][sc](dom)
    coeffs = 1 + 0.5 * rng.random(lv.padded_shape(1)) if kind else None
    if kind:
        op = te.VarPoissonStarPatchOperator(te.Vector.from_numpy(dom, coeffs), dom, gf)
    else:
        op = te.PoissonStarPatchOperator(dom, gf)
    for dt, tol, tol_f in ((te.TE_F64, 1e-13, 1e-13), (te.TE_F32, 2e-6, 8e-6)):
        u = rng.standard_normal(lv.padded_shape(1))
        uo, fo = oracle.apply(lv, u.copy(), sc, 0, kind, 0, coeffs)
        uv = te.Vector.from_numpy(dom, u, dtype=dt)
        fv = te.Vector(dom, 1, dt)
        fv.t.fill_(7.0)  # every cell of f is written (ghosts zero)
        op.apply(uv, fv)
        assert rel_err(fv.numpy(), fo) <= tol_f, dt
        assert rel_err(uv.numpy(), uo) <= tol, dt


@pytest.mark.parametrize("name", NAMES)
def test_transfers_fixed_size(te, oracle, name):
    levels, _ = cases()[name]
    rng = np.random.default_rng(13)
    fine, coarse = levels[0], levels[1]
    doms = [te.Domain(lv) for lv in (fine, coarse)]
    for nc in (1, 2):
        vf = rng.standard_normal(fine.padded_shape(nc))
        for ex in (False, True):
            want = np.stack([oracle.restrict(fine, coarse, np.ascontiguousarray(vf[:, c:c + 1]), int(ex))[:, 0]
                             for c in range(nc)], axis=1)
            r = te.LinearRestrictor(doms[0], doms[1], ex)
            for dt, tol in ((te.TE_F64, 1e-13), (te.TE_F32, 2e-6)):
                out = te.Vector(doms[1], nc, dt)
                out.t.fill_(7.0)  # every coarse cell is written (ghosts zero or extrapolated)
                from thunderegg_gb300.capi import check, lib

                check(lib().te_restrict(r.h, nc, dt, te.Vector.from_numpy(doms[0], vf, dtype=dt).ptr, out.ptr))
                assert rel_err(out.numpy(), want) <= tol, (nc, ex, dt)
        vc = rng.standard_normal(coarse.padded_shape(nc))
        want = np.stack([oracle.interpolate(coarse, fine, np.ascontiguousarray(vc[:, c:c + 1]),
                                            np.ascontiguousarray(vf[:, c:c + 1]))[:, 0] for c in range(nc)], axis=1)
        i = te.DirectInterpolator(doms[1], doms[0])
        for dt, tol in ((te.TE_F64, 1e-13), (te.TE_F32, 2e-6)):
            fv = te.Vector.from_numpy(doms[0], vf, dtype=dt)
            i.interpolate(te.Vector.from_numpy(doms[1], vc, dtype=dt), fv)
            assert rel_err(fv.numpy(), want) <= tol, (nc, dt)


def test_general_kernels_still_match():
    """The same checks (and the small-patch parity cases) with every level on
    the general kernels."""
    env = dict(os.environ, TE_GENERIC_LEVEL_KERNELS="1")
    cmd = [sys.executable, "-m", "pytest", "-q", "-x", "-m", "gpu", "-p", "no:cacheprovider",
           os.path.join(ROOT, "tests", "test_gpu_level_kernels.py"), os.path.join(ROOT, "tests", "test_gpu_parity.py"),
           "-k", "fixed_size or ghost_fill or operator_apply or transfers"]
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-2000:]
