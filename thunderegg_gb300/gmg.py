"""Assemble a full GMG-preconditioned BiCGStab solve on the GPU.

This is the setup a ThunderEgg user writes by hand (see the reference's
CycleBuilder doc example, GMG/CycleBuilder.h:36-53): one Domain, ghost
filler, operator and smoother per level, LinearRestrictor/DirectInterpolator
between levels, a V-cycle, and Iterative::BiCGStab on the finest level.
"""
from __future__ import annotations

from dataclasses import dataclass

from . import (CG, BiCGStab, BiCGStabPatchSolver, BiLinearGhostFiller, BiQuadraticGhostFiller, CycleBuilder,
               CycleOpts, DFTPatchSolver, DirectInterpolator, Domain, IterativeRefinement, LinearRestrictor,
               PoissonStarPatchOperator, TriLinearGhostFiller, VarPoissonStarPatchOperator, Vector)
from .capi import TE_F64

SMOOTHER_DFT, SMOOTHER_BICGSTAB = 0, 1


@dataclass
class GmgOptions:
    scheme: int = 0                 # 0 BiLinear, 1 BiQuadratic, 2 TriLinear
    fill_type: int = 0
    smoother: int = SMOOTHER_DFT
    inner_tol: float = 1e-12        # BiCGStab patch smoother (pinned as in the oracle)
    inner_max_it: int = 1000
    inner_continue_on_breakdown: bool = True
    pre_sweeps: int = 1
    post_sweeps: int = 1
    coarse_sweeps: int = 1
    mid_sweeps: int = 1             # W and FMG cycles
    cycle_type: str = "V"           # "V", "W" or "F" (FMG)
    extrapolate_boundary_ghosts: bool = False
    tol: float = 1e-10
    max_it: int = 1000
    cycle_dtype: int = TE_F64       # TE_F32: mixed-precision V-cycle
    bicgstab_flags: int = 0         # 1: preconditioned early-exit update
    krylov: str = "bicgstab"        # outer solver: "bicgstab", "cg" or "ir" (FP64 iterative refinement)
    tc_precision: int = 0           # FP32 tensor-core transforms: 0 3xTF32, 1 BF16 (per-patch scaled)


def _tc_capable(op):
    """Levels whose FP32 DFT solves can run on the tensor cores: cubic patches of n = 16, 32, 64
    (2D) or 16 (3D) with one ghost layer; the solver itself checks the transform matrices."""
    lv = op.domain.level if hasattr(op, "domain") and hasattr(op.domain, "level") else None
    if lv is None:
        return True
    n = lv.ns[0]
    return (all(x == n for x in lv.ns) and lv.num_ghost == 1
            and ((lv.dim == 2 and n in (16, 32, 64)) or (lv.dim == 3 and n == 16)))


class GmgSolver:
    """All device objects of one multigrid hierarchy."""

    def __init__(self, levels, opts: GmgOptions = GmgOptions(), coeffs=None):
        self.levels = levels
        self.opts = opts
        fill_cls = [BiLinearGhostFiller, BiQuadraticGhostFiller, TriLinearGhostFiller][opts.scheme]
        self.domains = [Domain(lv) for lv in levels]
        self.fillers = [fill_cls(d, opts.fill_type) for d in self.domains]
        self.coeff_vecs = None
        if coeffs is not None:
            self.coeff_vecs = [Vector.from_numpy(d, c) for d, c in zip(self.domains, coeffs)]
            self.ops = [VarPoissonStarPatchOperator(c, d, g)
                        for c, d, g in zip(self.coeff_vecs, self.domains, self.fillers)]
        else:
            self.ops = [PoissonStarPatchOperator(d, g) for d, g in zip(self.domains, self.fillers)]
        if opts.smoother == SMOOTHER_DFT:
            self.smoothers = [DFTPatchSolver(op, 0, opts.tc_precision if _tc_capable(op) else 0) for op in self.ops]
        else:
            self.smoothers = [BiCGStabPatchSolver(op, opts.inner_tol, opts.inner_max_it,
                                                  opts.inner_continue_on_breakdown) for op in self.ops]
        n = len(levels)
        self.restrictors = [LinearRestrictor(self.domains[k], self.domains[k + 1], opts.extrapolate_boundary_ghosts)
                            for k in range(n - 1)]
        self.interpolators = [None] + [DirectInterpolator(self.domains[k], self.domains[k - 1])
                                       for k in range(1, n)]
        b = CycleBuilder(CycleOpts(opts.pre_sweeps, opts.post_sweeps, opts.mid_sweeps, opts.coarse_sweeps,
                                   opts.cycle_type))
        for k in range(n):
            if k == 0 and n > 1:
                b.addFinestLevel(self.ops[0], self.smoothers[0], self.restrictors[0])
            elif k + 1 < n:
                b.addIntermediateLevel(self.ops[k], self.smoothers[k], self.restrictors[k], self.interpolators[k])
            else:
                b.addCoarsestLevel(self.ops[k], self.smoothers[k], self.interpolators[k])
        self.cycle = b.getCycle(opts.cycle_dtype)
        if opts.krylov == "cg":
            self.krylov = CG(opts.tol, opts.max_it)
        elif opts.krylov == "ir":
            self.krylov = IterativeRefinement(opts.tol, opts.max_it)
        else:
            self.krylov = BiCGStab(opts.tol, opts.max_it, opts.bicgstab_flags)

    @property
    def finest(self):
        return self.domains[0]

    def solve(self, f: Vector, u: Vector, precondition=True):
        return self.krylov.solve(self.ops[0], u, f, self.cycle if precondition else None)

    def solve_batched(self, f: Vector, u: Vector, patch_offsets, precondition=True):
        """Independent solves whose finest patches are the ranges of patch_offsets
        (see mesh.union_hierarchy).  Returns (iterations, residuals, statuses)."""
        import ctypes

        from .capi import check, lib

        B = len(patch_offsets) - 1
        offs = (ctypes.c_int * (B + 1))(*patch_offsets)
        its = (ctypes.c_int * B)()
        res = (ctypes.c_double * B)()
        st = (ctypes.c_int * B)()
        rc = lib().te_bicgstab_solve_batched(self.ops[0].h, u.ncomp, u.ptr, f.ptr,
                                             self.cycle.h if precondition else None, float(self.opts.tol),
                                             int(self.opts.max_it), int(self.opts.bicgstab_flags), B, offs, its, res,
                                             st)
        if rc not in (0, 3):
            check(rc)
        return list(its), list(res), list(st)

    def residual(self, f: Vector, u: Vector):
        """||f - A u|| / ||f|| in FP64 on the device."""
        r = f.getZeroClone()
        self.ops[0].apply(u, r)
        r.scaleThenAdd(-1.0, f)
        return r.twoNorm() / f.twoNorm()
