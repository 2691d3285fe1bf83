"""TEST INFRASTRUCTURE ONLY: ctypes front end of the CPU oracle.

``Oracle("teo")`` wraps the restatement (oracle/_build/libte_oracle.so);
``Oracle("teref")`` wraps ThunderEgg itself compiled from its sources
(oracle/_ref/libteref.so, only where the reference sources exist).  Both take
the flat mesh tables of thunderegg_gb300.mesh.MeshLevel and numpy level
vectors in ThunderEgg's layout.  Only tests/, __graft_entry__.smoke() and the
CPU legs of bench.py use this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from thunderegg_gb300.capi import TeLevelDesc  # noqa: E402

# The ThunderEgg source tree that the reference build (target "ref") compiles
# and the mesh-input tests read; THUNDEREGG_REF overrides the default location.
REF_ROOT = os.environ.get("THUNDEREGG_REF", "/root/reference")
REF_SRC = os.path.join(REF_ROOT, "src", "ThunderEgg")
REF_MESH_INPUTS = os.path.join(REF_ROOT, "test", "mesh_inputs")

ORACLE_LIB = os.path.join(HERE, "_build", "libte_oracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libteref.so")

_dp = ctypes.POINTER(ctypes.c_double)


class GmgConfig(ctypes.Structure):
    _fields_ = [("scheme", ctypes.c_int), ("fill_type", ctypes.c_int), ("op_kind", ctypes.c_int),
                ("neumann", ctypes.c_int), ("smoother", ctypes.c_int),
                ("dft_neumann_mask", ctypes.c_int), ("inner_tol", ctypes.c_double),
                ("inner_max_it", ctypes.c_int), ("inner_continue_on_breakdown", ctypes.c_int),
                ("pre_sweeps", ctypes.c_int), ("post_sweeps", ctypes.c_int),
                ("coarse_sweeps", ctypes.c_int), ("extrapolate_boundary_ghosts", ctypes.c_int),
                ("tol", ctypes.c_double), ("max_it", ctypes.c_int), ("use_precond", ctypes.c_int),
                ("mid_sweeps", ctypes.c_int), ("cycle_type", ctypes.c_int), ("krylov", ctypes.c_int),
                ("precond_exit", ctypes.c_int)]


CYCLE_TYPES = {"V": 0, "W": 1, "F": 2}  # CycleOpts::cycle_type strings (CycleBuilder.h:176-191)


def gmg_config(scheme=0, fill_type=0, op_kind=0, neumann=0, smoother=0, dft_neumann_mask=0,
               inner_tol=1e-12, inner_max_it=1000, inner_continue_on_breakdown=1, pre_sweeps=1,
               post_sweeps=1, coarse_sweeps=1, extrapolate_boundary_ghosts=0, tol=1e-10,
               max_it=1000, use_precond=1, mid_sweeps=1, cycle_type="V", krylov="bicgstab",
               precond_exit=0):
    """precond_exit=1: the BiCGStab early exit adds alpha * M p (the GPU's
    TE_BICGSTAB_PRECONDITIONED_EXIT, flags=1); 0 is the reference's update.  Only the
    restatement ("teo") honours it; the compiled reference always runs its own rule."""
    return GmgConfig(scheme, fill_type, op_kind, neumann, smoother, dft_neumann_mask, inner_tol,
                     inner_max_it, inner_continue_on_breakdown, pre_sweeps, post_sweeps,
                     coarse_sweeps, extrapolate_boundary_ghosts, tol, max_it, use_precond,
                     mid_sweeps, CYCLE_TYPES[cycle_type], {"bicgstab": 0, "cg": 1}[krylov], precond_exit)


def build(ref: bool = False):
    """Compile the oracle (and, if asked and the sources exist, the reference)."""
    targets = ["oracle"] + (["ref"] if ref else [])
    subprocess.run(["make", "-s", "-C", HERE, f"-j{os.cpu_count() or 4}", f"REF_ROOT={REF_ROOT}"] + targets,
                   check=True)


def ref_sources_present():
    """True where the ThunderEgg source tree exists (the CPU machine, not the GPU machine)."""
    return os.path.isdir(REF_SRC)


def ref_available():
    return os.path.exists(REF_LIB)


def _ptr(a):
    return a.ctypes.data_as(_dp) if a is not None else None


class Oracle:
    def __init__(self, prefix="teo"):
        self.prefix = prefix
        path = ORACLE_LIB if prefix == "teo" else REF_LIB
        if not os.path.exists(path):
            if prefix == "teo":
                build()
            else:
                raise FileNotFoundError(path)
        self.L = ctypes.CDLL(path)
        self.L[f"{prefix}_last_error"].restype = ctypes.c_char_p

    def _f(self, name):
        return self.L[f"{self.prefix}_{name}"]

    def _check(self, rc):
        if rc != 0:
            msg = self._f("last_error")()
            raise RuntimeError(f"{self.prefix} error {rc}: {msg.decode() if msg else ''}")

    # -- ghost filling --------------------------------------------------------
    def ghost_fill(self, lvl, u, scheme, fill_type=0, ncomp=1):
        u = np.ascontiguousarray(u, dtype=np.float64)
        d = lvl.to_desc()
        self._check(self._f("ghost_fill")(ctypes.byref(d), scheme, fill_type, ncomp, _ptr(u)))
        return u

    def ghost_calls(self, lvl, fill_type=0):
        d = lvl.to_desc()
        n = self._f("ghost_num_calls")(ctypes.byref(d), fill_type)
        rows = np.zeros((max(n, 1), 6), np.int32)
        self._check(self._f("ghost_calls")(ctypes.byref(d), fill_type,
                                           rows.ctypes.data_as(ctypes.POINTER(ctypes.c_int))))
        return rows[:n]

    # -- operators ----------------------------------------------------------------
    def apply(self, lvl, u, scheme, fill_type=0, kind=0, neumann=0, coeffs=None, ncomp=1):
        u = np.ascontiguousarray(u, dtype=np.float64)
        f = np.zeros_like(u)
        d = lvl.to_desc()
        c = None if coeffs is None else np.ascontiguousarray(coeffs, dtype=np.float64)
        self._check(self._f("operator_apply")(ctypes.byref(d), scheme, fill_type, kind, neumann,
                                              _ptr(c), ncomp, _ptr(u), _ptr(f)))
        return u, f

    def modify_rhs(self, lvl, u, f, scheme=0, fill_type=0, kind=0, coeffs=None, ncomp=1):
        u = np.ascontiguousarray(u, dtype=np.float64)
        f = np.ascontiguousarray(f, dtype=np.float64).copy()
        d = lvl.to_desc()
        c = None if coeffs is None else np.ascontiguousarray(coeffs, dtype=np.float64)
        self._check(self._f("modify_rhs")(ctypes.byref(d), scheme, fill_type, kind, _ptr(c), ncomp,
                                          _ptr(u), _ptr(f)))
        return f

    def patch_solver(self, lvl, f, u, scheme, fill_type=0, kind=0, coeffs=None, smoother=0,
                     dft_neumann_mask=0, tol=1e-12, max_it=1000, cont=1, mode=0, ncomp=1):
        f = np.ascontiguousarray(f, dtype=np.float64)
        u = np.ascontiguousarray(u, dtype=np.float64).copy()
        d = lvl.to_desc()
        c = None if coeffs is None else np.ascontiguousarray(coeffs, dtype=np.float64)
        its = ctypes.c_longlong(0)
        self._check(self._f("patch_solver")(ctypes.byref(d), scheme, fill_type, kind, _ptr(c),
                                            smoother, dft_neumann_mask, ctypes.c_double(tol), max_it,
                                            cont, mode, ncomp, _ptr(f), _ptr(u), ctypes.byref(its)))
        return u, its.value

    # -- right-hand-side boundary helpers ---------------------------------------------
    _point_fn = ctypes.CFUNCTYPE(ctypes.c_double, ctypes.POINTER(ctypes.c_double))

    def add_bc_to_rhs(self, lvl, f, gfun=None, hfun=None, grad=None, kind=0, neumann=0):
        """addDrichletBCToRHS (kind 0 Poisson, 1 VarPoisson with coefficient hfun) or, with
        neumann=1, Poisson's addNeumannBCToRHS (grad: one function per axis).  Each function
        takes the point's coordinates x, y[, z] as floats."""
        D = lvl.dim
        f = np.ascontiguousarray(f, dtype=np.float64).copy()

        def wrap(fn):
            if fn is None:
                return self._point_fn(0)
            return self._point_fn(lambda x: float(fn(*[x[a] for a in range(D)])))

        keep = [wrap(gfun), wrap(hfun)] + [wrap(g) for g in (grad or [None] * D)]
        garr = (self._point_fn * D)(*keep[2:])
        d = lvl.to_desc()
        self._check(self._f("add_bc_to_rhs")(ctypes.byref(d), kind, neumann, keep[0], keep[1], garr, _ptr(f)))
        return f

    # -- transfers -------------------------------------------------------------
    def restrict(self, fine, coarse, vf, extrapolate=0, ncomp=1):
        vf = np.ascontiguousarray(vf, dtype=np.float64)
        vc = np.zeros(coarse.padded_shape(ncomp))
        df, dc = fine.to_desc(), coarse.to_desc()
        self._check(self._f("restrict")(ctypes.byref(df), ctypes.byref(dc), extrapolate, ncomp,
                                        _ptr(vf), _ptr(vc)))
        return vc

    def interpolate(self, coarse, fine, vc, vf, ncomp=1):
        vc = np.ascontiguousarray(vc, dtype=np.float64)
        vf = np.ascontiguousarray(vf, dtype=np.float64).copy()
        dc, df = coarse.to_desc(), fine.to_desc()
        self._check(self._f("interpolate")(ctypes.byref(dc), ctypes.byref(df), ncomp, _ptr(vc),
                                           _ptr(vf)))
        return vf

    # -- cycle and solve -------------------------------------------------------------
    def _levels(self, levels):
        arr = (TeLevelDesc * len(levels))()
        keep = []
        for k, lv in enumerate(levels):
            d = lv.to_desc()
            keep.append(lv._keep)
            arr[k] = d
        return arr, keep

    def _coeffs(self, coeffs, n):
        if coeffs is None:
            return None, []
        cs = [np.ascontiguousarray(c, dtype=np.float64) for c in coeffs]
        arr = (_dp * n)(*[c.ctypes.data_as(_dp) for c in cs])
        return arr, cs

    def vcycle(self, levels, f, cfg, coeffs=None, ncomp=1):
        arr, keep = self._levels(levels)
        carr, ckeep = self._coeffs(coeffs, len(levels))
        f = np.ascontiguousarray(f, dtype=np.float64)
        u = np.zeros_like(f)
        self._check(self._f("vcycle_apply")(arr, len(levels), ctypes.byref(cfg), carr, ncomp,
                                            _ptr(f), _ptr(u)))
        return u

    def solve(self, levels, f, cfg, u0=None, coeffs=None, ncomp=1):
        """BiCGStab(A, u, f, cycle), or CG with cfg.krylov = 1 -> (u, iterations, final relative
        residual, status)."""
        arr, keep = self._levels(levels)
        carr, ckeep = self._coeffs(coeffs, len(levels))
        f = np.ascontiguousarray(f, dtype=np.float64)
        u = np.zeros_like(f) if u0 is None else np.ascontiguousarray(u0, dtype=np.float64).copy()
        its = ctypes.c_int(0)
        res = ctypes.c_double(0)
        rc = self._f("gmg_solve")(arr, len(levels), ctypes.byref(cfg), carr, ncomp, _ptr(u),
                                  _ptr(f), ctypes.byref(its), ctypes.byref(res))
        if rc not in (0, 3):
            self._check(rc)
        return u, its.value, res.value, rc
