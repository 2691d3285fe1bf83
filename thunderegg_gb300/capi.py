"""ctypes binding of the C ABI declared in include/te_gpu.h.

The shared library ``thunderegg_gb300/_build/libte_gpu.so`` is built in-tree
by :func:`thunderegg_gb300.build.build`.  Loading fails loudly when it is
missing: there is no fallback path.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libte_gpu.so")

TE_OK, TE_ERR_INVALID, TE_ERR_CUDA, TE_ERR_BREAKDOWN = 0, 1, 2, 3
TE_ERR_UNSUPPORTED, TE_ERR_BUDGET, TE_ERR_TIMEOUT, TE_ERR_NOT_CONVERGED = 4, 5, 6, 7
TE_F64, TE_F32 = 0, 1
TE_GHOST_BILINEAR, TE_GHOST_BIQUADRATIC, TE_GHOST_TRILINEAR = 0, 1, 2
TE_FILL_FACES, TE_FILL_EDGES, TE_FILL_CORNERS = 0, 1, 2
TE_NOALLOC_MAX_PARTIALS = 65536
TE_CYCLE_V, TE_CYCLE_W, TE_CYCLE_FMG = 0, 1, 2
TE_BICGSTAB_PRECONDITIONED_EXIT, TE_BICGSTAB_FP64_OUTER, TE_BICGSTAB_SLOTS = 1, 2, 4
TE_TC_TF32X3, TE_TC_BF16 = 0, 1
TE_PENDING = 8

_ip = ctypes.POINTER(ctypes.c_int)
_dp = ctypes.POINTER(ctypes.c_double)


class TeLevelDesc(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int), ("ns", ctypes.c_int * 3), ("num_ghost", ctypes.c_int),
        ("num_patches", ctypes.c_int),
        ("id", _ip), ("refine_level", _ip), ("parent_id", _ip), ("orth_on_parent", _ip),
        ("child_ids", _ip), ("starts", _dp), ("spacings", _dp),
        ("nbr_type", _ip), ("nbr_ids", _ip), ("nbr_orth", _ip),
    ]


class TeCycleLevel(ctypes.Structure):
    _fields_ = [("op", ctypes.c_void_p), ("smoother", ctypes.c_void_p),
                ("restrictor", ctypes.c_void_p), ("interpolator", ctypes.c_void_p)]


class TeCycleOpts(ctypes.Structure):
    _fields_ = [("pre_sweeps", ctypes.c_int), ("post_sweeps", ctypes.c_int),
                ("mid_sweeps", ctypes.c_int), ("coarse_sweeps", ctypes.c_int)]


class TeServeOpts(ctypes.Structure):
    _fields_ = [("budget_bytes", ctypes.c_double), ("steps_per_round", ctypes.c_int), ("max_batch", ctypes.c_int)]


class TeSolveOpts(ctypes.Structure):
    _fields_ = [("scheme", ctypes.c_int), ("fill_type", ctypes.c_int), ("smoother", ctypes.c_int),
                ("inner_tol", ctypes.c_double), ("inner_max_iterations", ctypes.c_int),
                ("inner_continue_on_breakdown", ctypes.c_int), ("pre_sweeps", ctypes.c_int),
                ("post_sweeps", ctypes.c_int), ("coarse_sweeps", ctypes.c_int), ("tol", ctypes.c_double),
                ("max_iterations", ctypes.c_int), ("cycle_dtype", ctypes.c_int), ("flags", ctypes.c_int),
                ("tc_precision", ctypes.c_int)]


class TeServeResult(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("iterations", ctypes.c_int), ("residual", ctypes.c_double),
                ("latency_s", ctypes.c_double), ("restarts", ctypes.c_int)]


class TeServeCounters(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_longlong), ("admitted", ctypes.c_longlong), ("completed", ctypes.c_longlong),
                ("rejected", ctypes.c_longlong), ("union_builds", ctypes.c_longlong),
                ("union_cache_hits", ctypes.c_longlong), ("slot_fills", ctypes.c_longlong),
                ("reforms", ctypes.c_longlong), ("rounds", ctypes.c_longlong), ("queued", ctypes.c_int),
                ("active", ctypes.c_int), ("classes", ctypes.c_int), ("bytes_in_use", ctypes.c_double),
                ("build_s", ctypes.c_double), ("step_s", ctypes.c_double), ("finish_s", ctypes.c_double),
                ("form_s", ctypes.c_double)]


class TeError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"te_gpu error {code}: {msg}")
        self.code = code


class BreakdownError(TeError):
    """Mirror of ThunderEgg::Iterative::BreakdownError (BreakdownError.h:35-44)."""


_V = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double
_SIGS = {
    "te_last_error_message": (ctypes.c_char_p, []),
    "te_set_stream": (_I, [_V]),
    "te_synchronize": (_I, []),
    "te_kernel_launch_count": (ctypes.c_longlong, []),
    "te_domain_create": (_I, [ctypes.POINTER(TeLevelDesc), ctypes.POINTER(_V)]),
    "te_domain_destroy": (_I, [_V]),
    "te_domain_patch_stride": (ctypes.c_longlong, [_V, _I]),
    "te_domain_num_patches": (_I, [_V]),
    "te_vec_set": (_I, [_V, _I, _I, _V, _D, _I]),
    "te_vec_scale": (_I, [_V, _I, _I, _V, _D]),
    "te_vec_shift": (_I, [_V, _I, _I, _V, _D]),
    "te_vec_copy": (_I, [_V, _I, _I, _V, _V, _I]),
    "te_vec_add": (_I, [_V, _I, _I, _V, _V]),
    "te_vec_add_scaled": (_I, [_V, _I, _I, _V, _D, _V]),
    "te_vec_add_scaled2": (_I, [_V, _I, _I, _V, _D, _V, _D, _V]),
    "te_vec_scale_then_add": (_I, [_V, _I, _I, _V, _D, _V]),
    "te_vec_scale_then_add_scaled": (_I, [_V, _I, _I, _V, _D, _D, _V]),
    "te_vec_scale_then_add_scaled2": (_I, [_V, _I, _I, _V, _D, _D, _V, _D, _V]),
    "te_vec_two_norm": (_I, [_V, _I, _I, _V, _dp]),
    "te_vec_inf_norm": (_I, [_V, _I, _I, _V, _dp]),
    "te_vec_dot": (_I, [_V, _I, _I, _V, _V, _dp]),
    "te_vec_convert": (_I, [_V, _I, _I, _V, _I, _V]),
    "te_ghost_filler_create": (_I, [_V, _I, _I, ctypes.POINTER(_V)]),
    "te_ghost_filler_destroy": (_I, [_V]),
    "te_ghost_fill": (_I, [_V, _I, _I, _V]),
    "te_ghost_filler_num_calls": (_I, [_V]),
    "te_ghost_filler_calls": (_I, [_V, _ip]),
    "te_poisson_operator_create": (_I, [_V, _V, _I, ctypes.POINTER(_V)]),
    "te_varpoisson_operator_create": (_I, [_V, _V, _V, ctypes.POINTER(_V)]),
    "te_operator_destroy": (_I, [_V]),
    "te_operator_apply": (_I, [_V, _I, _I, _V, _V]),
    "te_operator_modify_rhs": (_I, [_V, _I, _I, _V, _V]),
    "te_level_alloc": (_I, [_V, _I, _I, ctypes.POINTER(_V)]),
    "te_level_free": (_I, [_V]),
    "te_device_alloc": (_I, [ctypes.c_size_t, ctypes.POINTER(_V)]),
    "te_device_free": (_I, [_V]),
    "te_copy": (_I, [_V, _V, ctypes.c_size_t]),
    "te_tune_report": (_I, [ctypes.c_char_p, _I, ctypes.POINTER(_I)]),
    "te_tune_reset": (_I, []),
    "te_domain_face_stride": (ctypes.c_longlong, [_V]),
    "te_domain_boundary_points": (_I, [_V, _V]),
    "te_operator_add_dirichlet_bc_to_rhs": (_I, [_V, _I, _V, _V, _V]),
    "te_operator_add_neumann_bc_to_rhs": (_I, [_V, _I, _V, _V]),
    "te_dft_patch_solver_create": (_I, [_V, _I, ctypes.POINTER(_V)]),
    "te_bicgstab_patch_solver_create": (_I, [_V, _D, _I, _I, ctypes.POINTER(_V)]),
    "te_patch_solver_destroy": (_I, [_V]),
    "te_patch_solver_smooth": (_I, [_V, _I, _I, _V, _V]),
    "te_patch_solver_apply": (_I, [_V, _I, _I, _V, _V]),
    "te_patch_solver_uses_tensor_cores": (_I, [_V, _ip]),
    "te_dft_patch_solver_create_tc": (_I, [_V, _I, _I, ctypes.POINTER(_V)]),
    "te_bicgstab_batch_create": (_I, [_V, _I, _V, _V, _V, ctypes.c_double, _I, _I, _I, _ip, ctypes.POINTER(_V)]),
    "te_bicgstab_batch_step": (_I, [_V, _I, _ip]),
    "te_bicgstab_batch_state": (_I, [_V, _ip, _dp, _ip, _ip]),
    "te_bicgstab_batch_sync_x": (_I, [_V]),
    "te_bicgstab_batch_destroy": (_I, [_V]),
    "te_linear_restrictor_create": (_I, [_V, _V, _I, ctypes.POINTER(_V)]),
    "te_restrictor_destroy": (_I, [_V]),
    "te_restrict": (_I, [_V, _I, _I, _V, _V]),
    "te_direct_interpolator_create": (_I, [_V, _V, ctypes.POINTER(_V)]),
    "te_interpolator_destroy": (_I, [_V]),
    "te_interpolate": (_I, [_V, _I, _I, _V, _V]),
    "te_vcycle_create": (_I, [ctypes.POINTER(TeCycleLevel), _I, TeCycleOpts, _I, ctypes.POINTER(_V)]),
    "te_cycle_create": (_I, [ctypes.POINTER(TeCycleLevel), _I, TeCycleOpts, _I, _I, ctypes.POINTER(_V)]),
    "te_cg_solve": (_I, [_V, _I, _V, _V, _V, _D, _I, ctypes.POINTER(_I), ctypes.POINTER(_D)]),
    "te_ir_solve": (_I, [_V, _I, _V, _V, _V, _D, _I, ctypes.POINTER(_I), ctypes.POINTER(_D)]),
    "te_bicgstab_batch_finish_slots": (_I, [_V, _I, ctypes.POINTER(_I), ctypes.POINTER(_I)]),
    "te_bicgstab_batch_reset": (_I, [_V, _I]),
    "te_cycle_destroy": (_I, [_V]),
    "te_cycle_apply": (_I, [_V, _I, _V, _V]),
    "te_cycle_timings": (_I, [_V, _I, _V, _V, _I, ctypes.c_char_p, _dp, _ip]),
    "te_bicgstab_solve": (_I, [_V, _I, _V, _V, _V, _D, _I, _I, _ip, _dp]),
    "te_bicgstab_solve_batched": (_I, [_V, _I, _V, _V, _V, _D, _I, _I, _I, _ip, _ip, _dp, _ip]),
    "te_level_dot_noalloc": (_I, [_I, _ip, _I, _I, _I, _I, _V, _V, _dp, _V]),
    "te_serve_create": (_I, [ctypes.POINTER(TeServeOpts), ctypes.POINTER(_V)]),
    "te_serve_destroy": (_I, [_V]),
    "te_serve_submit": (_I, [_V, ctypes.POINTER(TeLevelDesc), _I, ctypes.POINTER(TeSolveOpts), _dp,
                             ctypes.POINTER(ctypes.c_longlong)]),
    "te_serve_step": (_I, [_V, _ip]),
    "te_serve_poll": (_I, [_V, ctypes.c_longlong, _dp, ctypes.POINTER(TeServeResult)]),
    "te_serve_stats": (_I, [_V, ctypes.POINTER(TeServeCounters)]),
}

_lib = None


def lib():
    """The loaded te_gpu library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(rc):
    if rc != TE_OK:
        msg = lib().te_last_error_message()
        msg = msg.decode() if msg else ""
        if rc == TE_ERR_BREAKDOWN:
            raise BreakdownError(rc, msg)
        raise TeError(rc, msg)
    return rc


def exported_symbols():
    return list(_SIGS)
