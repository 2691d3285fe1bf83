"""GPU kernels against the CPU oracle, through the C ABI.

Tolerances (infinity-norm relative, max|gpu - oracle| / max|oracle|):
  FP64 ghost fill, operator apply, modifyRHS, restriction, interpolation: 1e-13
  FP64 DFT patch solve and V-cycle: 1e-12 (transform sums run in another order)
  FP64 BiCGStab patch smoother: 1e-8 (inner solves stop at 1e-12 relative residual)
  FP32 kernels: 2e-6 (single precision rounding)
Neighbour call tables are compared bit-exactly.
"""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

SCHEMES_2D = (0, 1)  # BiLinear, BiQuadratic


def _cases():
    from thunderegg_gb300 import mesh as M

    return {
        "2d_uniform": (M.uniform_mesh(2, 2, 8), SCHEMES_2D),
        "2d_circle": (M.circle_mesh(n=8, lo=2, hi=5), SCHEMES_2D),
        "2d_random": (M.random_mesh(3, n=6, lo=1, hi=4), SCHEMES_2D),
        "2d_random_odd": (M.random_mesh(4, n=5, lo=1, hi=4), (1,)),
        "3d_uniform": (M.uniform_mesh(3, 1, 4), (2,)),
        "3d_random": (M.random_mesh(5, n=4, dim=3, lo=1, hi=3), (2,)),
    }


CASES = None


def cases():
    global CASES
    if CASES is None:
        CASES = _cases()
    return CASES


CASE_NAMES = ["2d_uniform", "2d_circle", "2d_random", "2d_random_odd", "3d_uniform", "3d_random"]


def filler_cls(te, scheme):
    return [te.BiLinearGhostFiller, te.BiQuadraticGhostFiller, te.TriLinearGhostFiller][scheme]


def fill_types(dim):
    return (0, 2) if dim == 2 else (0, 1, 2)


@pytest.mark.parametrize("name", CASE_NAMES)
def test_ghost_fill(te, oracle, name):
    levels, schemes = cases()[name]
    lv = levels[0]
    rng = np.random.default_rng(1)
    dom = te.Domain(lv)
    for sc in schemes:
        for ft in fill_types(lv.dim):
            gf = filler_cls(te, sc)(dom, ft)
            # neighbour call table: bit-exact with the oracle's enumeration
            assert np.array_equal(gf.calls(), oracle.ghost_calls(lv, ft))
            for nc in (1, 2):
                u = rng.standard_normal(lv.padded_shape(nc))
                want = oracle.ghost_fill(lv, u.copy(), sc, ft, nc)
                v = te.Vector.from_numpy(dom, u)
                gf.fillGhost(v)
                assert rel_err(v.numpy(), want) <= 1e-13, (sc, ft, nc)
                v32 = te.Vector.from_numpy(dom, u, dtype=te.TE_F32)
                gf.fillGhost(v32)
                assert rel_err(v32.numpy(), want) <= 2e-6


@pytest.mark.parametrize("name", CASE_NAMES)
@pytest.mark.parametrize("kind", (0, 1))
def test_operator_apply(te, oracle, name, kind):
    levels, schemes = cases()[name]
    lv = levels[0]
    rng = np.random.default_rng(2)
    dom = te.Domain(lv)
    for sc in schemes:
        gf = filler_cls(te, sc)(dom)
        coeffs = 1 + 0.5 * rng.random(lv.padded_shape(1)) if kind else None
        if kind:
            op = te.VarPoissonStarPatchOperator(te.Vector.from_numpy(dom, coeffs), dom, gf)
        else:
            op = te.PoissonStarPatchOperator(dom, gf)
        # FP64: measured at most 2.3e-16 on these meshes (many cells bit-identical); FP32: rounding of
        # the single-precision stencil relative to the oracle's FP64 result
        for dt, tol, tol_f in ((te.TE_F64, 1e-13, 1e-13), (te.TE_F32, 2e-6, 8e-6)):
            u = rng.standard_normal(lv.padded_shape(1))
            uo, fo = oracle.apply(lv, u.copy(), sc, 0, kind, 0, coeffs)
            uv = te.Vector.from_numpy(dom, u, dtype=dt)
            fv = te.Vector(dom, 1, dt)
            fv.t.fill_(7.0)  # apply must overwrite f everywhere (setWithGhost(0))
            op.apply(uv, fv)
            assert rel_err(fv.numpy(), fo) <= tol_f, (sc, dt)
            assert rel_err(uv.numpy(), uo) <= tol, (sc, dt)  # ghosts of u are filled/mutated
            # modifyRHSForInternalBoundaryConditions
            f = rng.standard_normal(lv.padded_shape(1))
            want = oracle.modify_rhs(lv, uo, f, sc, 0, kind, coeffs)
            fv = te.Vector.from_numpy(dom, f, dtype=dt)
            op.modifyRHSForInternalBoundaryConditions(te.Vector.from_numpy(dom, uo, dtype=dt), fv)
            assert rel_err(fv.numpy(), want) <= tol_f


def test_poisson_neumann(te, oracle):
    from thunderegg_gb300 import mesh as M

    lv = M.circle_mesh(n=8, lo=2, hi=4)[0]
    rng = np.random.default_rng(3)
    dom = te.Domain(lv)
    gf = te.BiLinearGhostFiller(dom)
    op = te.PoissonStarPatchOperator(dom, gf, neumann=True)
    u = rng.standard_normal(lv.padded_shape(1))
    uo, fo = oracle.apply(lv, u.copy(), 0, 0, 0, 1)
    uv, fv = te.Vector.from_numpy(dom, u), te.Vector(dom)
    op.apply(uv, fv)
    assert rel_err(fv.numpy(), fo) <= 1e-13


@pytest.mark.parametrize("name", CASE_NAMES)
@pytest.mark.parametrize("smoother", (0, 1))
def test_patch_solvers(te, oracle, name, smoother):
    levels, schemes = cases()[name]
    lv = levels[0]
    rng = np.random.default_rng(4)
    dom = te.Domain(lv)
    sc = schemes[0]
    gf = filler_cls(te, sc)(dom)
    op = te.PoissonStarPatchOperator(dom, gf)
    ps = te.DFTPatchSolver(op) if smoother == 0 else te.BiCGStabPatchSolver(op, 1e-12, 1000, True)
    f = rng.standard_normal(lv.padded_shape(1))
    u = rng.standard_normal(lv.padded_shape(1))
    tol64 = 1e-12 if smoother == 0 else 1e-8
    for mode in (0, 1):
        want, _ = oracle.patch_solver(lv, f, u, sc, smoother=smoother, mode=mode)
        uv = te.Vector.from_numpy(dom, u)
        fv = te.Vector.from_numpy(dom, f)
        (ps.smooth if mode == 0 else ps.apply)(fv, uv)
        got = uv.numpy()
        g = lv.num_ghost
        inner = (Ellipsis,) + tuple(slice(g, -g) for _ in range(lv.dim))
        assert rel_err(got[inner], want[inner]) <= tol64, (mode,)
        if smoother == 0:
            u32 = te.Vector.from_numpy(dom, u, dtype=te.TE_F32)
            f32 = te.Vector.from_numpy(dom, f, dtype=te.TE_F32)
            (ps.smooth if mode == 0 else ps.apply)(f32, u32)
            assert rel_err(u32.numpy()[inner], want[inner]) <= 2e-5


@pytest.mark.parametrize("name", CASE_NAMES)
def test_transfers(te, oracle, name):
    levels, _ = cases()[name]
    rng = np.random.default_rng(5)
    doms = [te.Domain(lv) for lv in levels[:2]]
    fine, coarse = levels[0], levels[1]
    vf = rng.standard_normal(fine.padded_shape(1))
    for ex in (False, True):
        want = oracle.restrict(fine, coarse, vf, int(ex))
        r = te.LinearRestrictor(doms[0], doms[1], ex)
        got = r.restrict(te.Vector.from_numpy(doms[0], vf))
        assert rel_err(got.numpy(), want) <= 1e-13, ex
    vc = rng.standard_normal(coarse.padded_shape(1))
    want = oracle.interpolate(coarse, fine, vc, vf)
    i = te.DirectInterpolator(doms[1], doms[0])
    fv = te.Vector.from_numpy(doms[0], vf)
    i.interpolate(te.Vector.from_numpy(doms[1], vc), fv)
    assert rel_err(fv.numpy(), want) <= 1e-13


def test_vector_algebra(te):
    from thunderegg_gb300 import mesh as M

    lv = M.circle_mesh(n=8, lo=2, hi=4)[0]
    dom = te.Domain(lv)
    rng = np.random.default_rng(6)
    a, b, c = (rng.standard_normal(lv.padded_shape(2)) for _ in range(3))
    g = lv.num_ghost
    inner = (slice(None), slice(None)) + tuple(slice(g, -g) for _ in range(lv.dim))
    A, B, C = (te.Vector.from_numpy(dom, x) for x in (a, b, c))
    want = a.copy()
    want[inner] = a[inner] * 0.5 + b[inner] * 2.0 + c[inner] * -3.0
    A.scaleThenAddScaled(0.5, 2.0, B, -3.0, C)
    assert rel_err(A.numpy(), want) <= 1e-15
    assert abs(B.dot(C) - float(np.sum(b[inner] * c[inner]))) <= 1e-12 * abs(float(np.sum(np.abs(b * c))))
    assert abs(B.twoNorm() - float(np.sqrt(np.sum(b[inner] ** 2)))) <= 1e-13 * B.twoNorm()
    assert B.infNorm() == max(float(b[inner].max()), 0.0)
    B.set(3.0)
    want = b.copy()
    want[inner] = 3.0
    assert np.array_equal(B.numpy(), want)


@pytest.mark.parametrize("dim,level,n", [(2, 3, 32), (2, 2, 16), (3, 1, 16), (3, 1, 8)])
def test_dot_of_cubic_levels(te, dim, level, n):
    """Dot products of cubic levels (FP32: two cells per load, ghost cells masked): FP64 within
    1e-13 and FP32 within 1e-11 (Dot2 sums) of numpy's FP64 sum of the interior products.  The
    ghost cells hold NaN, which no result may see."""
    import torch
    from thunderegg_gb300 import mesh as M

    lv = M.uniform_mesh(dim, level, n)[0]
    dom = te.Domain(lv)
    rng = np.random.default_rng(11)
    g = lv.num_ghost
    inner = (slice(None), slice(None)) + tuple(slice(g, -g) for _ in range(dim))
    for dtype, tol in ((te.TE_F64, 1e-13), (te.TE_F32, 1e-11)):
        a, b = (rng.standard_normal(lv.padded_shape(1)) for _ in range(2))
        if dtype == te.TE_F32:
            a, b = a.astype(np.float32).astype(np.float64), b.astype(np.float32).astype(np.float64)
        want = float(np.sum(a[inner] * b[inner]))
        scale = float(np.sum(np.abs(a[inner] * b[inner])))
        an, bn = a.copy(), b.copy()
        mask = np.ones(an.shape, bool)
        mask[inner] = False
        an[mask] = np.nan
        bn[mask] = np.nan
        A, B = te.Vector.from_numpy(dom, an, dtype), te.Vector.from_numpy(dom, bn, dtype)
        got = A.dot(B)
        assert abs(got - want) <= tol * scale, (dtype, got, want)
        assert abs(A.dot(A) - float(np.sum(a[inner] ** 2))) <= tol * float(np.sum(a[inner] ** 2))
        # a view one element into a larger buffer is not aligned for paired loads: the general
        # kernel gives the same value to rounding
        tdt = torch.float64 if dtype == te.TE_F64 else torch.float32
        big = torch.empty(A.t.numel() + 1, dtype=tdt, device="cuda")
        big[1:] = A.t.reshape(-1)
        Au = te.Vector(dom, 1, dtype, big[1:].view(A.t.shape))
        assert abs(Au.dot(B) - want) <= tol * scale, dtype


def test_fftw_patch_solver_is_the_dft_solve(te, oracle):
    """FFTWPatchSolver (Poisson/FFTWPatchSolver.h) computes the DFT solve: on
    Dirichlet and mixed Neumann sides it matches the oracle's DFTPatchSolver,
    FP64 1e-12 and FP32 (tensor cores for the cubic n = 32 level) 2e-5."""
    from thunderegg_gb300 import mesh as M

    rng = np.random.default_rng(90)
    for levels, mask in ((M.circle_mesh(n=32, lo=2, hi=4), 0), (M.uniform_mesh(2, 2, 32), 0b0101)):
        lv = levels[0]
        dom = te.Domain(lv)
        gf = te.BiQuadraticGhostFiller(dom)
        op = te.PoissonStarPatchOperator(dom, gf)
        f = rng.standard_normal(lv.padded_shape(1))
        u0 = rng.standard_normal(lv.padded_shape(1))
        want, _ = oracle.patch_solver(lv, f, u0, 1, smoother=0, dft_neumann_mask=mask, mode=0)
        s = te.FFTWPatchSolver(op, mask)
        for dt, tol in ((te.TE_F64, 1e-12), (te.TE_F32, 2e-5)):
            uv = te.Vector.from_numpy(dom, u0, dtype=dt)
            s.smooth(te.Vector.from_numpy(dom, f, dtype=dt), uv)
            inner = (Ellipsis, slice(1, -1), slice(1, -1))
            assert rel_err(uv.numpy()[inner], want[inner]) <= tol, (mask, dt)


def _bc_cases():
    from thunderegg_gb300 import mesh as M

    return [M.circle_mesh(n=8, lo=2, hi=4)[0], M.random_mesh(4, n=5, lo=1, hi=4)[0],
            M.random_mesh(5, n=4, dim=3, lo=1, hi=3)[0]]


@pytest.mark.parametrize("idx", range(3))
def test_bc_rhs_helpers_match_oracle(te, oracle, idx):
    """addDrichletBCToRHS / addNeumannBCToRHS (Poisson) and VarPoisson's addDrichletBCToRHS on the
    device: bit for bit the oracle's FP64 result (pinned bit-exact to the reference) for polynomial
    boundary data; exp(x y) data within 1e-15 (numpy's vectorised exp may differ by an ulp)."""
    lv = _bc_cases()[idx]
    D = lv.dim
    dom = te.Domain(lv)
    gf = [te.BiQuadraticGhostFiller, te.TriLinearGhostFiller][D - 2](dom)  # BiLinear needs even n
    if D == 2:
        g = lambda x, y: 1.5 + x * x - 0.25 * x * y + y  # noqa: E731
        grad = [lambda x, y: 2 * x - 0.25 * y, lambda x, y: 1.0 - 0.25 * x]
        gexp = lambda x, y: np.exp(x * y)  # noqa: E731
        coef = lambda x, y: 1 + 0.5 * x  # noqa: E731
    else:
        g = lambda x, y, z: 1 + x * y - z * z + 0.5 * x  # noqa: E731
        grad = [lambda x, y, z: y + 0.5, lambda x, y, z: x, lambda x, y, z: -2 * z]
        gexp = lambda x, y, z: np.exp(x * y * z)  # noqa: E731
        coef = lambda x, y, z: 1 + 0.5 * x * z  # noqa: E731
    f = np.random.default_rng(60 + idx).standard_normal(lv.padded_shape(1))
    op = te.PoissonStarPatchOperator(dom, gf)
    cvec = te.Vector.from_numpy(dom, np.ones(lv.padded_shape(1)))
    vop = te.VarPoissonStarPatchOperator(cvec, dom, gf)
    cases = [("dirichlet", lambda v: op.addDrichletBCToRHS(v, g), dict(gfun=g), True),
             ("dirichlet exp", lambda v: op.addDrichletBCToRHS(v, gexp), dict(gfun=gexp), False),
             ("neumann", lambda v: op.addNeumannBCToRHS(v, g, grad), dict(gfun=g, grad=grad, neumann=1), True),
             ("varpoisson", lambda v: vop.addDrichletBCToRHS(v, g, coef), dict(gfun=g, hfun=coef, kind=1), True)]
    for name, run, kw, exact in cases:
        want = oracle.add_bc_to_rhs(lv, f, **kw)
        v = te.Vector.from_numpy(dom, f)
        run(v)
        got = v.numpy()
        if exact:
            assert np.array_equal(got, want), name
        else:
            assert rel_err(got, want) <= 1e-15, name
        v32 = te.Vector.from_numpy(dom, f, dtype=te.TE_F32)
        run(v32)
        assert rel_err(v32.numpy(), want) <= 2e-6, name
