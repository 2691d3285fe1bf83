"""Synthetic workloads (meshes + right-hand sides) of the benchmark configurations.

Right-hand sides are built on the host with numpy, the way a ThunderEgg user
does with DomainTools::SetValues (DomainTools.h:281-305) and
StarPatchOperator::addDrichletBCToRHS (Poisson/StarPatchOperator.h:181-199).
The operator is the +Laplacian, so -Lap(u) = f is solved as A u = -f.
"""
from __future__ import annotations

import math

import numpy as np

from . import mesh as M


def interior_view(lvl: M.MeshLevel, v):
    g = lvl.num_ghost
    return v[(Ellipsis,) + tuple(slice(g, -g) for _ in range(lvl.dim))]


def set_values(lvl: M.MeshLevel, fn, ncomp=1):
    """Level vector with fn(x, y[, z]) at the cell centres, ghosts zero."""
    v = np.zeros(lvl.padded_shape(ncomp))
    xc = M.cell_centers(lvl)  # [P, (nz,) ny, nx, D]
    vals = fn(*[xc[..., a] for a in range(lvl.dim)])
    iv = interior_view(lvl, v)
    iv[:, 0] = vals
    return v


def add_dirichlet_bc(lvl: M.MeshLevel, f, gfn):
    """f += -2 g(x_b) / h^2 on cells next to a domain boundary (sides without a
    neighbour); x_b is the boundary point (DomainTools::GetRealCoordBound)."""
    D = lvl.dim
    iv = interior_view(lvl, f)
    for p in range(lvl.num_patches):
        for side in range(2 * D):
            if lvl.nbr_type[p, M.side_slot(D, side)] >= 0:
                continue
            axis, upper = side >> 1, side & 1
            h = lvl.spacings[p, axis]
            coords = []
            for a in range(D):
                if a == axis:
                    coords.append(np.array([lvl.starts[p, a] + (h * lvl.ns[a] if upper else 0.0)]))
                else:
                    i = np.arange(lvl.ns[a])
                    coords.append(lvl.starts[p, a] + lvl.spacings[p, a] / 2.0 + lvl.spacings[p, a] * i)
            grids = np.meshgrid(*coords, indexing="ij")  # axes in x, y, z order
            gv = gfn(*grids)  # shape (nx|1, ny|1, ...)
            gv = np.transpose(gv)  # to (z), y, x order
            sl = [slice(None)] * D
            sl[D - 1 - axis] = slice(-1, None) if upper else slice(0, 1)
            iv[p, 0][tuple(sl)] += -2.0 * gv / (h * h)
    return f


def config1():
    """2D uniform quadtree at level 2 (16 patches of 32x32), f = 2 pi^2 sin(pi x) sin(pi y),
    u = 0 Dirichlet; exact u = sin(pi x) sin(pi y)."""
    levels = M.uniform_mesh(2, 2, 32)
    f = set_values(levels[0], lambda x, y: -2 * math.pi ** 2 * np.sin(math.pi * x) * np.sin(math.pi * y))
    exact = set_values(levels[0], lambda x, y: np.sin(math.pi * x) * np.sin(math.pi * y))
    return levels, f, exact


def config2(n=32, lo=3, hi=7):
    """2D circle-adaptive quadtree (levels lo..hi, r = 0.3 about (0.5, 0.5), 2:1
    balanced), n x n patches; u = exp(x y), f = -Lap(u), Dirichlet data from u."""
    levels = M.circle_mesh(n=n, lo=lo, hi=hi)
    lap = lambda x, y: (x * x + y * y) * np.exp(x * y)  # noqa: E731
    f = set_values(levels[0], lap)
    add_dirichlet_bc(levels[0], f, lambda x, y: np.exp(x * y))
    exact = set_values(levels[0], lambda x, y: np.exp(x * y))
    return levels, f, exact


def config3(level=4, n=16, seed=0):
    """3D uniform octree, n^3 patches, RHS i.i.d. N(0,1) per cell (PCG64 seed)."""
    levels = M.uniform_mesh(3, level, n, connect="face")
    rng = np.random.default_rng(seed)
    f = np.zeros(levels[0].padded_shape(1))
    interior_view(levels[0], f)[...] = rng.standard_normal(interior_view(levels[0], f).shape)
    return levels, f, None


def sine_modes_rhs(lvl, rng, modes=8, kmax=8):
    """Sum of `modes` sine modes sin(k1 pi x) sin(k2 pi y) (sin(k3 pi z)) with
    N(0,1) amplitudes and mode numbers in [1, kmax]."""
    D = lvl.dim
    amps = rng.standard_normal(modes)
    ks = rng.integers(1, kmax + 1, size=(modes, D))

    def fn(*xs):
        out = 0.0
        for a, k in zip(amps, ks):
            term = a
            for d in range(D):
                term = term * np.sin(k[d] * math.pi * xs[d])
            out = out + term
        return out

    return set_values(lvl, fn)


def config4(num_solves=32, n=16, lo=2, hi=6, p=0.3):
    """Config 4: num_solves variable-coefficient problems, solve s on its own random
    quadtree (seed s, leaves refined with probability p from level lo to hi, 2:1
    balanced, n x n patches), beta = 1 + 0.9 sin(4 pi x) sin(4 pi y), and RHS a
    sum of 8 sine modes with N(0,1) amplitudes drawn from the same seed.
    Returns [(levels, f, coeffs)]."""
    out = []
    for s in range(num_solves):
        levels = M.random_mesh(s, n=n, lo=lo, hi=hi, p=p)
        rng = np.random.default_rng(s)
        out.append((levels, sine_modes_rhs(levels[0], rng), beta_coeffs(levels)))
    return out


def beta_coeffs(levels):
    """beta = 1 + 0.9 sin(4 pi x) sin(4 pi y) at cell centres and ghost centres of every level."""
    out = []
    for lvl in levels:
        v = np.zeros(lvl.padded_shape(1))
        g = lvl.num_ghost
        D = lvl.dim
        grids = []
        for a in range(D):
            i = np.arange(-g, lvl.ns[a] + g)
            grids.append(lvl.starts[:, a:a + 1] + lvl.spacings[:, a:a + 1] / 2.0 + lvl.spacings[:, a:a + 1] * i)
        # [P, ny+2g, nx+2g]
        x = grids[0][:, None, :]
        y = grids[1][:, :, None]
        v[:, 0] = 1 + 0.9 * np.sin(4 * math.pi * x) * np.sin(4 * math.pi * y)
        out.append(v)
    return out
