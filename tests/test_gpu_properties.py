"""The reference's own hot-path tests, as properties of the GPU path.

ThunderEgg's tests check properties rather than golden values; the same
properties hold here through the C ABI:
  * the ghost fillers reproduce polynomial fields in the side ghosts
    (BiLinear: linear, test/BiLinearGhostFiller_MPI1.cpp:254-300; BiQuadratic:
    quadratic, test/BiQuadraticGhostFiller_MPI1.cpp:254-300; TriLinear: linear
    3D, test/TriLinearGhostFiller_MPI1.cpp:33-76), to 1e-12;
  * LinearRestrictor reproduces linear fields at the coarse cell centres
    (test/GMG/LinearRestrictor_MPI1.cpp:34-75);
  * the discrete solution converges at second order
    (test/Poisson/DFTPatchSolver_MPI1.cpp:36-199: log2(e_n / e_2n) > 1.8);
  * BiCGStab returns at once for a zero right-hand side and for an initial
    guess that already meets the tolerance (test/Iterative/BiCGStab_MPI1.cpp:93-240).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def padded_coords(lv):
    """Cell-centre coordinates of every padded cell: [P, (z), y, x, D]."""
    g = lv.num_ghost
    axes = []
    for a in range(lv.dim):
        i = np.arange(lv.ns[a] + 2 * g) - g + 0.5
        axes.append(lv.starts[:, a][:, None] + lv.spacings[:, a][:, None] * i[None, :])  # [P, n+2g]
    P = lv.num_patches
    shape = lv.padded_shape(1)[2:]
    out = np.zeros((P,) + shape + (lv.dim,))
    for a in range(lv.dim):
        sh = [P] + [1] * lv.dim
        sh[lv.dim - a] = shape[lv.dim - 1 - a]
        out[..., a] = axes[a].reshape(sh)
    return out


def side_ghost_mask(lv):
    """True on the side ghost cells (not edges or corners) of faces that have a neighbour."""
    from thunderegg_gb300 import mesh as M

    g, D = lv.num_ghost, lv.dim
    shape = lv.padded_shape(1)[2:]
    mask = np.zeros((lv.num_patches,) + shape, dtype=bool)
    inner = tuple(slice(g, -g) for _ in range(D))
    for p in range(lv.num_patches):
        for side in range(2 * D):
            if lv.nbr_type[p, M.side_slot(D, side)] < 0:
                continue
            axis, upper = side >> 1, side & 1
            sl = list(inner)
            sl[D - 1 - axis] = slice(shape[D - 1 - axis] - 1, None) if upper else slice(0, 1)
            mask[(p,) + tuple(sl)] = True
    return mask


@pytest.mark.parametrize("scheme", (0, 1, 2))
def test_ghost_fill_reproduces_polynomials(te, scheme):
    from thunderegg_gb300 import mesh as M

    if scheme == 0:
        levels, fn = M.circle_mesh(n=8, lo=2, hi=5), lambda x, y: 1 + 0.5 * x + 0.3 * y
    elif scheme == 1:
        levels, fn = M.circle_mesh(n=8, lo=2, hi=5), lambda x, y: 1 + x * x + 0.3 * x + 0.3 + 0.5 * y * y
    else:
        levels, fn = M.random_mesh(5, n=4, dim=3, lo=1, hi=3), lambda x, y, z: 1 + 0.5 * x + y + 7 * z
    lv = levels[0]
    xc = padded_coords(lv)
    exact = fn(*[xc[..., a] for a in range(lv.dim)])
    mask = side_ghost_mask(lv)
    assert mask.any()
    u = np.zeros(lv.padded_shape(1))
    g = lv.num_ghost
    inner = (slice(None),) + tuple(slice(g, -g) for _ in range(lv.dim))
    u[:, 0][inner] = exact[inner]
    dom = te.Domain(lv)
    filler = [te.BiLinearGhostFiller, te.BiQuadraticGhostFiller, te.TriLinearGhostFiller][scheme](dom)
    v = te.Vector.from_numpy(dom, u)
    filler.fillGhost(v)
    got = v.numpy()[:, 0]
    assert np.abs(got[mask] - exact[mask]).max() <= 1e-12 * np.abs(exact).max()


def test_restrictor_reproduces_linear_fields(te):
    from thunderegg_gb300 import mesh as M
    from thunderegg_gb300 import problems as PB

    levels = M.circle_mesh(n=8, lo=2, hi=5)
    fn = lambda x, y: 2 - 0.7 * x + 1.3 * y  # noqa: E731
    fine = PB.set_values(levels[0], fn)
    want = PB.interior_view(levels[1], PB.set_values(levels[1], fn))
    doms = [te.Domain(lv) for lv in levels[:2]]
    got = te.LinearRestrictor(doms[0], doms[1]).restrict(te.Vector.from_numpy(doms[0], fine))
    assert np.abs(PB.interior_view(levels[1], got.numpy()) - want).max() <= 1e-13


def test_second_order_convergence(te):
    """-Lap u = 2 pi^2 sin(pi x) sin(pi y), u = 0 on the boundary, on 4 x 4 patches of
    16^2 and of 32^2 cells: the FP64 solve's error drops by at least 2^1.8."""
    from thunderegg_gb300 import mesh as M
    from thunderegg_gb300 import problems as PB
    from thunderegg_gb300.gmg import GmgOptions, GmgSolver

    errs = []
    for n in (16, 32):
        levels = M.uniform_mesh(2, 2, n)
        lv = levels[0]
        f = PB.set_values(lv, lambda x, y: -2 * np.pi ** 2 * np.sin(np.pi * x) * np.sin(np.pi * y))
        exact = PB.interior_view(lv, PB.set_values(lv, lambda x, y: np.sin(np.pi * x) * np.sin(np.pi * y)))
        s = GmgSolver(levels, GmgOptions(scheme=0, smoother=0, tol=1e-12, bicgstab_flags=1))
        fv, uv = te.Vector.from_numpy(s.finest, f), te.Vector(s.finest)
        s.solve(fv, uv)
        errs.append(np.abs(PB.interior_view(lv, uv.numpy()) - exact).max())
    assert np.log2(errs[0] / errs[1]) > 1.8, errs


def test_bicgstab_zero_rhs_and_converged_guess(te):
    from thunderegg_gb300 import mesh as M
    from thunderegg_gb300.gmg import GmgOptions, GmgSolver

    levels = M.circle_mesh(n=8, lo=2, hi=4)
    s = GmgSolver(levels, GmgOptions(scheme=1, smoother=0, tol=1e-10))
    zero, uv = te.Vector(s.finest), te.Vector(s.finest)
    assert s.solve(zero, uv) == 0
    f = np.random.default_rng(3).standard_normal(levels[0].padded_shape(1))
    fv = te.Vector.from_numpy(s.finest, f)
    tight = GmgSolver(levels, GmgOptions(scheme=1, smoother=0, tol=1e-13, bicgstab_flags=1))
    tight.solve(fv, uv)
    assert s.solve(fv, uv) == 0  # already within 1e-10
