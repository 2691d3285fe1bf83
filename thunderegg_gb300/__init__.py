"""GB300-native geometric-multigrid hot path of ThunderEgg.

Host-side mirror of ThunderEgg's operator/plugin API for the GMG path,
calling the CUDA kernels through the C ABI of ``include/te_gpu.h``:

=======================================  =========================================
ThunderEgg (src/ThunderEgg/...)           here
=======================================  =========================================
Domain<D>            (Domain.h)           :class:`Domain`
Vector<D>            (Vector.h)           :class:`Vector` (device storage, same layout)
BiLinearGhostFiller  (BiLinearGhostFiller.h)   :class:`BiLinearGhostFiller`
BiQuadraticGhostFiller                    :class:`BiQuadraticGhostFiller`
TriLinearGhostFiller                      :class:`TriLinearGhostFiller`
Poisson::StarPatchOperator                :class:`PoissonStarPatchOperator`
VarPoisson::StarPatchOperator             :class:`VarPoissonStarPatchOperator`
Poisson::DFTPatchSolver                   :class:`DFTPatchSolver`
Iterative::PatchSolver (BiCGStab inner)   :class:`BiCGStabPatchSolver`
GMG::LinearRestrictor / DirectInterpolator :class:`LinearRestrictor`, :class:`DirectInterpolator`
GMG::CycleOpts / CycleBuilder / VCycle    :class:`CycleOpts`, :class:`CycleBuilder`
Iterative::BiCGStab                       :class:`BiCGStab`
=======================================  =========================================

Device memory comes from PyTorch (plumbing only); every computation runs in
the te_gpu CUDA kernels.  There is no CPU fallback: without the built library
or a GPU, constructing any of these objects raises.
"""
from __future__ import annotations

import ctypes
import sys

import numpy as np

from . import capi, mesh
from .capi import (TE_F32, TE_F64, TE_FILL_CORNERS, TE_FILL_EDGES, TE_FILL_FACES, BreakdownError,
                   TeError, check, lib)

__all__ = ["Domain", "Vector", "BiLinearGhostFiller", "BiQuadraticGhostFiller", "TriLinearGhostFiller",
           "PoissonStarPatchOperator", "VarPoissonStarPatchOperator", "DFTPatchSolver",
           "BiCGStabPatchSolver", "LinearRestrictor", "DirectInterpolator", "CycleOpts", "CycleBuilder",
           "BiCGStab", "CG", "IterativeRefinement", "Cycle", "FFTWPatchSolver", "BreakdownError", "TeError", "mesh", "capi",
           "GhostFillingType", "TE_F32", "TE_F64", "TE_FILL_FACES", "TE_FILL_EDGES", "TE_FILL_CORNERS"]


class GhostFillingType:
    Faces = TE_FILL_FACES
    Edges = TE_FILL_EDGES
    Corners = TE_FILL_CORNERS


def _torch():
    import torch

    if not torch.cuda.is_available():
        raise RuntimeError("thunderegg_gb300 needs a CUDA GPU; no CPU fallback exists")
    return torch


def _bind_stream():
    torch = _torch()
    check(lib().te_set_stream(ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))


class _Handle:
    _destroy = None

    def __init__(self):
        self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            if self.h and self.h.value and self._destroy:
                getattr(lib(), self._destroy)(self.h)
                self.h = ctypes.c_void_p()
        except Exception:
            pass


class Domain(_Handle):
    """Domain<D> of one level; wraps a :class:`mesh.MeshLevel`."""

    _destroy = "te_domain_destroy"

    def __init__(self, level: mesh.MeshLevel):
        super().__init__()
        _bind_stream()
        self.level = level
        desc = level.to_desc()
        check(lib().te_domain_create(ctypes.byref(desc), ctypes.byref(self.h)))
        self.dim = level.dim
        self.ns = level.ns
        self.num_ghost = level.num_ghost

    def getNumLocalPatches(self):
        return self.level.num_patches

    def getNumLocalCells(self):
        return self.level.num_cells

    def padded_shape(self, ncomp=1):
        return self.level.padded_shape(ncomp)


class Vector:
    """Vector<D> on the GPU with ThunderEgg's layout (Vector.h:133-153)."""

    def __init__(self, domain: Domain, ncomp: int = 1, dtype=TE_F64, data=None):
        torch = _torch()
        self.domain = domain
        self.ncomp = ncomp
        self.dtype = dtype
        tdt = torch.float64 if dtype == TE_F64 else torch.float32
        if data is None:
            self.t = torch.zeros(domain.padded_shape(ncomp), dtype=tdt, device="cuda")
        else:
            self.t = data
            assert tuple(data.shape) == tuple(domain.padded_shape(ncomp)) and data.dtype == tdt
            assert data.is_contiguous() and data.is_cuda

    # -- plumbing -------------------------------------------------------------
    @property
    def ptr(self):
        return ctypes.c_void_p(self.t.data_ptr())

    @classmethod
    def from_numpy(cls, domain, arr, dtype=TE_F64):
        torch = _torch()
        arr = np.asarray(arr)
        ncomp = arr.shape[1]
        tdt = torch.float64 if dtype == TE_F64 else torch.float32
        t = torch.as_tensor(np.ascontiguousarray(arr), dtype=tdt).cuda()
        return cls(domain, ncomp, dtype, t)

    def numpy(self):
        _torch().cuda.synchronize()
        return self.t.detach().double().cpu().numpy()

    def _d(self):
        return self.domain.h

    # -- Vector<D> algebra (Vector.h:391-611) ---------------------------------
    def set(self, alpha):
        check(lib().te_vec_set(self._d(), self.ncomp, self.dtype, self.ptr, float(alpha), 0))

    def setWithGhost(self, alpha):
        check(lib().te_vec_set(self._d(), self.ncomp, self.dtype, self.ptr, float(alpha), 1))

    def scale(self, alpha):
        check(lib().te_vec_scale(self._d(), self.ncomp, self.dtype, self.ptr, float(alpha)))

    def shift(self, delta):
        check(lib().te_vec_shift(self._d(), self.ncomp, self.dtype, self.ptr, float(delta)))

    def copy(self, b):
        check(lib().te_vec_copy(self._d(), self.ncomp, self.dtype, self.ptr, b.ptr, 0))

    def copyWithGhost(self, b):
        check(lib().te_vec_copy(self._d(), self.ncomp, self.dtype, self.ptr, b.ptr, 1))

    def add(self, b):
        check(lib().te_vec_add(self._d(), self.ncomp, self.dtype, self.ptr, b.ptr))

    def addScaled(self, alpha, a, beta=None, b=None):
        if b is None:
            check(lib().te_vec_add_scaled(self._d(), self.ncomp, self.dtype, self.ptr, float(alpha), a.ptr))
        else:
            check(lib().te_vec_add_scaled2(self._d(), self.ncomp, self.dtype, self.ptr, float(alpha), a.ptr,
                                           float(beta), b.ptr))

    def scaleThenAdd(self, alpha, b):
        check(lib().te_vec_scale_then_add(self._d(), self.ncomp, self.dtype, self.ptr, float(alpha), b.ptr))

    def scaleThenAddScaled(self, alpha, beta, b, gamma=None, c=None):
        if c is None:
            check(lib().te_vec_scale_then_add_scaled(self._d(), self.ncomp, self.dtype, self.ptr, float(alpha),
                                                     float(beta), b.ptr))
        else:
            check(lib().te_vec_scale_then_add_scaled2(self._d(), self.ncomp, self.dtype, self.ptr, float(alpha),
                                                      float(beta), b.ptr, float(gamma), c.ptr))

    def twoNorm(self):
        out = ctypes.c_double()
        check(lib().te_vec_two_norm(self._d(), self.ncomp, self.dtype, self.ptr, ctypes.byref(out)))
        return out.value

    def infNorm(self):
        out = ctypes.c_double()
        check(lib().te_vec_inf_norm(self._d(), self.ncomp, self.dtype, self.ptr, ctypes.byref(out)))
        return out.value

    def dot(self, b):
        out = ctypes.c_double()
        check(lib().te_vec_dot(self._d(), self.ncomp, self.dtype, self.ptr, b.ptr, ctypes.byref(out)))
        return out.value

    def getZeroClone(self):
        return Vector(self.domain, self.ncomp, self.dtype)

    def clone(self):
        v = Vector(self.domain, self.ncomp, self.dtype)
        v.t.copy_(self.t)
        return v

    def getNumLocalPatches(self):
        return self.domain.getNumLocalPatches()

    def getNumComponents(self):
        return self.ncomp


class _GhostFiller(_Handle):
    _destroy = "te_ghost_filler_destroy"
    scheme = None

    def __init__(self, domain: Domain, fill_type=TE_FILL_FACES):
        super().__init__()
        _bind_stream()
        self.domain = domain
        self.fill_type = fill_type
        check(lib().te_ghost_filler_create(domain.h, self.scheme, fill_type, ctypes.byref(self.h)))

    def fillGhost(self, u: Vector):
        check(lib().te_ghost_fill(self.h, u.ncomp, u.dtype, u.ptr))

    def calls(self):
        n = lib().te_ghost_filler_num_calls(self.h)
        rows = np.zeros((max(n, 1), 6), np.int32)
        check(lib().te_ghost_filler_calls(self.h, rows.ctypes.data_as(ctypes.POINTER(ctypes.c_int))))
        return rows[:n]


class BiLinearGhostFiller(_GhostFiller):
    scheme = capi.TE_GHOST_BILINEAR


class BiQuadraticGhostFiller(_GhostFiller):
    scheme = capi.TE_GHOST_BIQUADRATIC


class TriLinearGhostFiller(_GhostFiller):
    scheme = capi.TE_GHOST_TRILINEAR


class _Operator(_Handle):
    _destroy = "te_operator_destroy"

    def apply(self, u: Vector, f: Vector):
        check(lib().te_operator_apply(self.h, u.ncomp, u.dtype, u.ptr, f.ptr))

    def modifyRHSForInternalBoundaryConditions(self, u: Vector, f: Vector):
        check(lib().te_operator_modify_rhs(self.h, u.ncomp, u.dtype, u.ptr, f.ptr))

    def getDomain(self):
        return self.domain

    def getGhostFiller(self):
        return self.ghost_filler

    def _boundary_values(self, *fns):
        """The functions evaluated at the boundary points (DomainTools::GetRealCoordBound),
        as device FP64 arrays [P][2D][face stride].  Each function takes the coordinate
        arrays x, y[, z] (numpy) and returns values of their shape."""
        torch = _torch()
        dom = self.domain
        D = dom.dim
        fs = int(lib().te_domain_face_stride(dom.h))
        pts = torch.empty((dom.level.num_patches, 2 * D, fs, D), dtype=torch.float64, device="cuda")
        check(lib().te_domain_boundary_points(dom.h, ctypes.c_void_p(pts.data_ptr())))
        X = pts.cpu().numpy()
        out = []
        for fn in fns:
            v = np.broadcast_to(np.asarray(fn(*[X[..., a] for a in range(D)]), dtype=np.float64), X.shape[:-1])
            out.append(torch.from_numpy(np.array(v, dtype=np.float64)).cuda())
        return out


class PoissonStarPatchOperator(_Operator):
    """Poisson::StarPatchOperator (Poisson/StarPatchOperator.h:52-63)."""

    def __init__(self, domain: Domain, ghost_filler: _GhostFiller, neumann: bool = False):
        super().__init__()
        _bind_stream()
        self.domain, self.ghost_filler = domain, ghost_filler
        check(lib().te_poisson_operator_create(domain.h, ghost_filler.h, int(neumann), ctypes.byref(self.h)))

    def addDrichletBCToRHS(self, f: Vector, gfunc):
        """Poisson/StarPatchOperator.h:187-204: f += -2 g(x_b) / h^2 next to every domain-boundary
        side, on the device; gfunc(x, y[, z]) takes numpy coordinate arrays."""
        (g,) = self._boundary_values(gfunc)
        check(lib().te_operator_add_dirichlet_bc_to_rhs(self.h, f.dtype, f.ptr, ctypes.c_void_p(g.data_ptr()), None))
        _torch().cuda.current_stream().synchronize()

    def addNeumannBCToRHS(self, f: Vector, gfunc, gfunc_grad):
        """Poisson/StarPatchOperator.h:212-242: f += dg/dn / h (lower sides), -= (upper sides);
        gfunc_grad[axis](x, y[, z]) is the derivative of gfunc along that axis (gfunc itself is
        not used, as in the reference)."""
        D = self.domain.dim
        vals = self._boundary_values(*gfunc_grad)
        # the derivative along each side's own axis
        sel = vals[0].clone()
        for side in range(2 * D):
            sel[:, side] = vals[side >> 1][:, side]
        check(lib().te_operator_add_neumann_bc_to_rhs(self.h, f.dtype, f.ptr, ctypes.c_void_p(sel.data_ptr())))
        _torch().cuda.current_stream().synchronize()


class VarPoissonStarPatchOperator(_Operator):
    """VarPoisson::StarPatchOperator (VarPoisson/StarPatchOperator.h:61-71)."""

    def __init__(self, coeffs: Vector, domain: Domain, ghost_filler: _GhostFiller):
        super().__init__()
        _bind_stream()
        assert coeffs.dtype == TE_F64 and coeffs.ncomp == 1
        self.domain, self.ghost_filler = domain, ghost_filler
        self._coeffs = coeffs
        check(lib().te_varpoisson_operator_create(domain.h, ghost_filler.h, coeffs.ptr, ctypes.byref(self.h)))

    def addDrichletBCToRHS(self, f: Vector, gfunc, hfunc):
        """VarPoisson/StarPatchOperator.h:194-219: f -= 2 g(x_b) h(x_b) / h^2 next to every
        domain-boundary side, on the device; hfunc is the coefficient."""
        g, c = self._boundary_values(gfunc, hfunc)
        check(lib().te_operator_add_dirichlet_bc_to_rhs(self.h, f.dtype, f.ptr, ctypes.c_void_p(g.data_ptr()),
                                                        ctypes.c_void_p(c.data_ptr())))
        _torch().cuda.current_stream().synchronize()


class _PatchSolver(_Handle):
    _destroy = "te_patch_solver_destroy"

    def smooth(self, f: Vector, u: Vector):
        check(lib().te_patch_solver_smooth(self.h, u.ncomp, u.dtype, f.ptr, u.ptr))

    def apply(self, f: Vector, u: Vector):
        check(lib().te_patch_solver_apply(self.h, u.ncomp, u.dtype, f.ptr, u.ptr))


class DFTPatchSolver(_PatchSolver):
    """Poisson::DFTPatchSolver (Poisson/DFTPatchSolver.h:385-450)."""

    def __init__(self, op: _Operator, neumann_mask: int = 0, tc_precision: int = capi.TE_TC_TF32X3):
        """tc_precision (no reference counterpart): the arithmetic of the FP32 tensor-core
        transforms, TE_TC_TF32X3 (3xTF32, about FP32 accuracy) or TE_TC_BF16 (BF16 operands,
        FP32 accumulation, per-patch power-of-two scaling)."""
        super().__init__()
        _bind_stream()
        self.op = op
        if tc_precision == capi.TE_TC_TF32X3:
            check(lib().te_dft_patch_solver_create(op.h, int(neumann_mask), ctypes.byref(self.h)))
        else:
            check(lib().te_dft_patch_solver_create_tc(op.h, int(neumann_mask), int(tc_precision),
                                                      ctypes.byref(self.h)))

    @property
    def uses_tensor_cores(self) -> bool:
        """True when the FP32 solves run as 3xTF32 tcgen05 contractions."""
        v = ctypes.c_int(0)
        check(lib().te_patch_solver_uses_tensor_cores(self.h, ctypes.byref(v)))
        return bool(v.value)


class FFTWPatchSolver(DFTPatchSolver):
    """Poisson::FFTWPatchSolver (Poisson/FFTWPatchSolver.h:189-308): the same
    solve as DFTPatchSolver -- per axis the FFTW r2r kinds RODFT10/01, REDFT10/01
    and REDFT11/RODFT11 are DST-II/III, DCT-II/III and DCT-IV/DST-IV, the
    eigenvalues are -sum 4/h^2 sin^2, the all-Neumann patch without neighbours
    drops its zero mode and the result is scaled by prod 1/(2n) (FFTW's
    unnormalised transforms carry the factor 2 that the DFT solver's matrices
    move into prod 2/n).  On the GPU the transforms run as dense contractions
    (tensor cores in FP32 for n <= 64), which beat an FFT at these sizes."""


class BiCGStabPatchSolver(_PatchSolver):
    """Iterative::PatchSolver with an inner Iterative::BiCGStab (Iterative/PatchSolver.h:121-175)."""

    def __init__(self, op: _Operator, tol: float = 1e-12, max_iterations: int = 1000,
                 continue_on_breakdown: bool = False):
        super().__init__()
        _bind_stream()
        self.op = op
        check(lib().te_bicgstab_patch_solver_create(op.h, float(tol), int(max_iterations),
                                                    int(continue_on_breakdown), ctypes.byref(self.h)))


class LinearRestrictor(_Handle):
    """GMG::LinearRestrictor (GMG/LinearRestrictor.h:166-191)."""

    _destroy = "te_restrictor_destroy"

    def __init__(self, fine: Domain, coarse: Domain, extrapolate_boundary_ghosts: bool = False):
        super().__init__()
        _bind_stream()
        self.fine, self.coarse = fine, coarse
        check(lib().te_linear_restrictor_create(fine.h, coarse.h, int(extrapolate_boundary_ghosts),
                                                ctypes.byref(self.h)))

    def restrict(self, fine: Vector) -> Vector:
        out = Vector(self.coarse, fine.ncomp, fine.dtype)
        check(lib().te_restrict(self.h, fine.ncomp, fine.dtype, fine.ptr, out.ptr))
        return out


class DirectInterpolator(_Handle):
    """GMG::DirectInterpolator (GMG/DirectInterpolator.h:40-91)."""

    _destroy = "te_interpolator_destroy"

    def __init__(self, coarse: Domain, fine: Domain):
        super().__init__()
        _bind_stream()
        self.coarse, self.fine = coarse, fine
        check(lib().te_direct_interpolator_create(coarse.h, fine.h, ctypes.byref(self.h)))

    def interpolate(self, coarse: Vector, fine: Vector):
        check(lib().te_interpolate(self.h, fine.ncomp, fine.dtype, coarse.ptr, fine.ptr))


class CycleOpts:
    """GMG::CycleOpts (GMG/CycleOpts.h:33-55)."""

    def __init__(self, pre_sweeps=1, post_sweeps=1, mid_sweeps=1, coarse_sweeps=1, cycle_type="V"):
        self.pre_sweeps, self.post_sweeps = pre_sweeps, post_sweeps
        self.mid_sweeps, self.coarse_sweeps = mid_sweeps, coarse_sweeps
        self.cycle_type = cycle_type  # "V", "W" or "F" (checked by CycleBuilder.getCycle)


class Cycle(_Handle):
    _destroy = "te_cycle_destroy"

    def apply(self, f: Vector, u: Vector):
        check(lib().te_cycle_apply(self.h, u.ncomp, f.ptr, u.ptr))

    def timings(self, f: Vector, u: Vector, max_entries=128):
        """[(phase name, milliseconds)] of one eager application (device events)."""
        names = ctypes.create_string_buffer(32 * max_entries)
        ms = (ctypes.c_double * max_entries)()
        n = ctypes.c_int(0)
        check(lib().te_cycle_timings(self.h, u.ncomp, f.ptr, u.ptr, max_entries, names, ms, ctypes.byref(n)))
        raw = names.raw
        return [(raw[32 * i:32 * i + 32].split(b"\0")[0].decode(), ms[i]) for i in range(n.value)]


class CycleBuilder:
    """GMG::CycleBuilder (GMG/CycleBuilder.h:86-192)."""

    def __init__(self, opts: CycleOpts):
        self.opts = opts
        self.levels = []
        self.has_coarsest = False

    def addFinestLevel(self, op, smoother, restrictor):
        if self.levels:
            raise TeError(capi.TE_ERR_INVALID, "addFinestLevel was already called")
        self.levels.append((op, smoother, restrictor, None))

    def addIntermediateLevel(self, op, smoother, restrictor, interpolator):
        if not self.levels:
            raise TeError(capi.TE_ERR_INVALID, "addFinestLevel has not been called yet")
        if self.has_coarsest:
            raise TeError(capi.TE_ERR_INVALID, "addCoarsestLevel has been called")
        self.levels.append((op, smoother, restrictor, interpolator))

    def addCoarsestLevel(self, op, smoother, interpolator):
        if not self.levels:
            raise TeError(capi.TE_ERR_INVALID, "addFinestLevel has not been called yet")
        if self.has_coarsest:
            raise TeError(capi.TE_ERR_INVALID, "addCoarsestLevel has already been called")
        self.has_coarsest = True
        self.levels.append((op, smoother, None, interpolator))

    def getCycle(self, dtype=TE_F64) -> Cycle:
        """The cycle of opts.cycle_type ("V", "W" or "F" for FMG, CycleBuilder.h:176-191);
        dtype=TE_F32 runs it in FP32 (f and u stay FP64)."""
        if not self.has_coarsest:
            raise TeError(capi.TE_ERR_INVALID, "addCoarsestLevel has not been called")
        types = {"V": capi.TE_CYCLE_V, "W": capi.TE_CYCLE_W, "F": capi.TE_CYCLE_FMG}
        if self.opts.cycle_type not in types:
            raise TeError(capi.TE_ERR_UNSUPPORTED, "Unsupported Cycle type: " + str(self.opts.cycle_type))
        arr = (capi.TeCycleLevel * len(self.levels))()
        for k, (op, sm, r, i) in enumerate(self.levels):
            arr[k].op = op.h.value
            arr[k].smoother = sm.h.value
            arr[k].restrictor = r.h.value if r is not None else None
            arr[k].interpolator = i.h.value if i is not None else None
        o = self.opts
        opts = capi.TeCycleOpts(o.pre_sweeps, o.post_sweeps, o.mid_sweeps, o.coarse_sweeps)
        c = Cycle()
        _bind_stream()
        check(lib().te_cycle_create(arr, len(self.levels), opts, types[self.opts.cycle_type], dtype,
                                    ctypes.byref(c.h)))
        c._keep = list(self.levels)
        return c


class BiCGStab:
    """Iterative::BiCGStab (Iterative/BiCGStab.h:40-204) on the GPU: FP64, or
    float-float (pairs of FP32 numbers) when the preconditioner is an FP32 cycle."""

    PRECONDITIONED_EXIT = 1
    FP64_OUTER = 2

    def __init__(self, tolerance=1e-12, max_iterations=1000, flags=0):
        self.tolerance, self.max_iterations, self.flags = tolerance, max_iterations, flags
        self.final_residual = None

    def setTolerance(self, tol):
        self.tolerance = tol

    def setMaxIterations(self, n):
        self.max_iterations = n

    def getTolerance(self):
        return self.tolerance

    def getMaxIterations(self):
        return self.max_iterations

    def solve(self, A, x: Vector, b: Vector, Mr=None, output=False, os=None):
        """Returns the iteration count.  With output=True, prints the reference's progress
        line "%5d %16.8e" (iteration, relative residual) to os (default stdout) before the
        first iteration and after each one (BiCGStab.h:134-139,193-197)."""
        if output:
            return self._solve_printing(A, x, b, Mr, os if os is not None else sys.stdout)
        its = ctypes.c_int(0)
        res = ctypes.c_double(0)
        check(lib().te_bicgstab_solve(A.h, x.ncomp, x.ptr, b.ptr, Mr.h if Mr is not None else None,
                                      float(self.tolerance), int(self.max_iterations), int(self.flags),
                                      ctypes.byref(its), ctypes.byref(res)))
        self.final_residual = res.value
        return its.value

    def _solve_printing(self, A, x, b, Mr, os):
        """The same solve advanced one iteration at a time through the resumable batch
        (a batch of one), reading the residual after each iteration."""
        P = x.domain.getNumLocalPatches()
        offs = (ctypes.c_int * 2)(0, P)
        h = ctypes.c_void_p()
        check(lib().te_bicgstab_batch_create(A.h, x.ncomp, x.ptr, b.ptr, Mr.h if Mr is not None else None,
                                             float(self.tolerance), int(self.max_iterations), int(self.flags),
                                             1, offs, ctypes.byref(h)))
        try:
            its, res, st, run = (ctypes.c_int * 1)(), (ctypes.c_double * 1)(), (ctypes.c_int * 1)(), (ctypes.c_int * 1)()
            check(lib().te_bicgstab_batch_state(h, its, res, st, run))
            os.write("%5d %16.8e\n" % (its[0], res[0]))
            shown = its[0]
            n = ctypes.c_int(1)
            while n.value:
                check(lib().te_bicgstab_batch_step(h, 1, ctypes.byref(n)))
                check(lib().te_bicgstab_batch_state(h, its, res, st, run))
                if its[0] != shown:
                    os.write("%5d %16.8e\n" % (its[0], res[0]))
                    shown = its[0]
            self.final_residual = res[0]
            if st[0] == capi.TE_ERR_BREAKDOWN:
                raise BreakdownError(st[0], f"BiCGStab broke down on iteration {its[0]}")
            check(st[0])
            return its[0]
        finally:
            lib().te_bicgstab_batch_destroy(h)


class IterativeRefinement:
    """FP64 iterative refinement around a cycle (no reference counterpart; the
    Iterative::Solver interface, Iterative/Solver.h:64-69): x += Mr (b - A x)
    until the true FP64 residual ||b - A x|| / ||b|| <= tolerance."""

    def __init__(self, tolerance=1e-10, max_iterations=200):
        self.tolerance, self.max_iterations = tolerance, max_iterations
        self.final_residual = None

    def setTolerance(self, tol):
        self.tolerance = tol

    def setMaxIterations(self, n):
        self.max_iterations = n

    def getTolerance(self):
        return self.tolerance

    def getMaxIterations(self):
        return self.max_iterations

    def solve(self, A, x: Vector, b: Vector, Mr=None):
        if Mr is None:
            raise RuntimeError("IterativeRefinement needs a preconditioner (a cycle)")
        its = ctypes.c_int(0)
        res = ctypes.c_double(0)
        rc = lib().te_ir_solve(A.h, x.ncomp, x.ptr, b.ptr, Mr.h, float(self.tolerance), int(self.max_iterations),
                               ctypes.byref(its), ctypes.byref(res))
        self.final_residual = res.value
        check(rc)
        return its.value


class CG:
    """Iterative::CG (Iterative/CG.h:40-194) on the GPU, FP64 vectors; Mr is
    applied to each search direction before A, as in the reference."""

    def __init__(self, tolerance=1e-12, max_iterations=1000):
        self.tolerance, self.max_iterations = tolerance, max_iterations
        self.final_residual = None

    def setTolerance(self, tol):
        self.tolerance = tol

    def setMaxIterations(self, n):
        self.max_iterations = n

    def getTolerance(self):
        return self.tolerance

    def getMaxIterations(self):
        return self.max_iterations

    def solve(self, A, x: Vector, b: Vector, Mr=None):
        its = ctypes.c_int(0)
        res = ctypes.c_double(0)
        check(lib().te_cg_solve(A.h, x.ncomp, x.ptr, b.ptr, Mr.h if Mr is not None else None,
                                float(self.tolerance), int(self.max_iterations), ctypes.byref(its),
                                ctypes.byref(res)))
        self.final_residual = res.value
        return its.value
