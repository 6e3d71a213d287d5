"""ctypes binding of libjja_gb300.so (C ABI declared in include/jja_gb300.h).

The library is built in-tree by ``pyjjasim_gb300.build``. Loading fails loudly when it is
missing or cannot be built: there is no CPU fallback for the time-stepping path.
"""
import ctypes
import os
import threading

from . import build as _build

_lock = threading.Lock()
_lib = None

c_int, c_int64, c_double, c_void_p = ctypes.c_int, ctypes.c_int64, ctypes.c_double, ctypes.c_void_p
P_i64, P_i32, P_f64 = ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_double)

NOISE_NONE, NOISE_BUFFER, NOISE_PHILOX = 0, 1, 2


class FactorOpts(ctypes.Structure):
    _fields_ = [("nd_leaf", c_int), ("max_supernode", c_int), ("keep_factor", c_int), ("relax_zeros", c_int),
                ("relax_frac", c_double)]


class FactorStats(ctypes.Structure):
    _fields_ = [("n", c_int), ("n_supernodes", c_int), ("n_levels", c_int), ("max_k", c_int), ("max_m", c_int),
                ("nnz_L", c_int64), ("f_values", c_int64), ("factor_flops", c_double)]


class SolveTuning(ctypes.Structure):
    _fields_ = [("rhs_block", c_int), ("rows_per_lane", c_int), ("target_warps", c_int), ("min_piece", c_int),
                ("schedule", c_int), ("rows_per_lane_fwd", c_int), ("pack_rows", c_int), ("pack_min_warps", c_int),
                ("pdl", c_int), ("groups", c_int), ("coop_blocks", c_int),
                ("dst_lines", c_int), ("pack_lanes", c_int),
                ("subtree_rows", c_int)]


class ScheduleStats(ctypes.Structure):
    _fields_ = [("n_levels", c_int), ("n_subtrees", c_int), ("n_subtree_members", c_int), ("max_subtree_rows", c_int),
                ("n_pack_items", c_int), ("n_pack_shapes", c_int), ("n_fwd_items", c_int64), ("n_bwd_items", c_int64)]


class PlanDesc(ctypes.Structure):
    _fields_ = [("Nj", c_int), ("Nf", c_int), ("W", c_int), ("stencil_width", c_int),
                ("a_rowptr", P_i64), ("a_col", P_i32), ("a_val", P_f64),
                ("Ic", P_f64), ("inv_c0", P_f64), ("coef", P_f64), ("Rv", P_f64),
                ("extrap", c_double * 4), ("dt", c_double), ("Ic_w", P_f64), ("tuning", SolveTuning)]


class View(ctypes.Structure):
    _fields_ = [("ptr", c_void_p), ("stride_n", c_int64), ("stride_w", c_int64), ("stride_t", c_int64)]


class State(ctypes.Structure):
    _fields_ = [("hist", c_void_p * 4), ("theta_s", c_void_p), ("Is", View), ("f", View), ("Vs", View), ("T", View),
                ("noise_mode", c_int), ("noise", c_void_p), ("seed", ctypes.c_uint64), ("step", c_int64),
                ("th_out", c_void_p), ("I_out", c_void_p), ("src_t0", c_int64), ("src_steps", c_int64),
                ("store_all", c_int)]


class AdjointArgs(ctypes.Structure):
    _fields_ = [("G", View), ("th_m1", c_void_p), ("th_m2", c_void_p), ("mu_p1", c_void_p), ("mu_p2", c_void_p),
                ("cos_p1", c_void_p), ("cos_p2", c_void_p), ("mu_out", c_void_p), ("cos_out", c_void_p),
                ("usum", c_void_p), ("musum", c_void_p), ("gIc", c_void_p)]


class AdjointSegmentArgs(ctypes.Structure):
    _fields_ = [("seg", c_void_p), ("s0", c_int64), ("L", c_int64), ("Nt", c_int64),
                ("G", ctypes.POINTER(c_void_p)), ("mu", c_void_p * 3), ("cos", c_void_p * 3),
                ("usum", c_void_p), ("musum", c_void_p), ("gIc", c_void_p), ("use_graph", c_int)]


class StaticDesc(ctypes.Structure):
    _fields_ = [("Nj", c_int), ("Nf", c_int), ("Nn", c_int), ("W", c_int),
                ("a_rowptr", P_i64), ("a_col", P_i32), ("a_val", P_f64),
                ("m_rowptr", P_i64), ("m_col", P_i32), ("m_val", P_f64),
                ("l_rowptr", P_i64), ("l_col", P_i32), ("l_val", P_f64),
                ("kl_colptr", P_i64), ("kl_rowind", P_i32), ("kl_val", P_f64),
                ("Ic", P_f64), ("A_norm", c_double), ("M_norm", c_double)]


class NewtonArgs(ctypes.Structure):
    _fields_ = [("theta", c_void_p), ("Is", c_void_p), ("f", c_void_p), ("n", c_void_p), ("tol", c_double),
                ("maxiter", c_int), ("stop_as_residual_increases", c_int), ("stop_if_not_target_n", c_int)]


class NewtonResult(ctypes.Structure):
    _fields_ = [("status", ctypes.POINTER(c_int)), ("iterations", ctypes.POINTER(c_int)), ("residuals", P_f64),
                ("is_target", ctypes.POINTER(c_int))]


# exported symbol -> (restype, argtypes); every symbol of include/jja_gb300.h
SIGNATURES = {
    "jja_factor_create": (c_int, [c_int, P_i64, P_i32, P_f64, P_f64, P_f64, P_i32, ctypes.POINTER(FactorOpts),
                                  ctypes.POINTER(c_void_p)]),
    "jja_factor_destroy": (None, [c_void_p]),
    "jja_factor_get_stats": (c_int, [c_void_p, ctypes.POINTER(FactorStats)]),
    "jja_factor_get_perm": (c_int, [c_void_p, P_i32]),
    "jja_factor_get_supernodes": (c_int, [c_void_p, P_i32, P_i32, P_i32, P_i32, P_i32]),
    "jja_factor_solve_host": (c_int, [c_void_p, P_f64, c_int]),
    "jja_factor_check_schedule": (c_int, [c_void_p, c_int, ctypes.POINTER(SolveTuning), P_i64, P_i64]),
    "jja_factor_schedule_stats": (c_int, [c_void_p, c_int, ctypes.POINTER(SolveTuning), ctypes.POINTER(ScheduleStats)]),
    "jja_plan_create": (c_int, [ctypes.POINTER(PlanDesc), c_void_p, ctypes.POINTER(c_void_p)]),
    "jja_plan_destroy": (None, [c_void_p]),
    "jja_plan_device_bytes": (c_int64, [c_void_p]),
    "jja_plan_set_fast_poisson": (c_int, [c_void_p, c_int, c_int, P_i32, c_double]),
    "jja_plan_check": (c_int, [c_void_p, ctypes.POINTER(c_int)]),
    "jja_plan_test_wait_limit": (c_int, [c_void_p, c_void_p]),
    "jja_run": (c_int, [c_void_p, ctypes.POINTER(State), c_int, P_i64, P_i64, c_int, c_void_p]),
    "jja_run_timed": (c_int, [c_void_p, ctypes.POINTER(State), c_int, P_f64, c_void_p]),
    "jja_solve": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "jja_solve_static": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "jja_adjoint_step": (c_int, [c_void_p, ctypes.POINTER(AdjointArgs), c_void_p]),
    "jja_adjoint_segment": (c_int, [c_void_p, ctypes.POINTER(AdjointSegmentArgs), c_void_p]),
    "jja_adjoint_flux": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "jja_static_create": (c_int, [ctypes.POINTER(StaticDesc), c_void_p, ctypes.POINTER(c_void_p)]),
    "jja_static_destroy": (None, [c_void_p]),
    "jja_static_device_bytes": (c_int64, [c_void_p]),
    "jja_static_solve": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, ctypes.POINTER(c_int), c_void_p]),
    "jja_static_london": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "jja_static_newton": (c_int, [c_void_p, ctypes.POINTER(NewtonArgs), ctypes.POINTER(NewtonResult), c_void_p]),
    "jja_vortex": (c_int, [c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_void_p]),
    "jja_eval_sin": (c_int, [c_void_p, c_void_p, c_void_p, c_int64, c_void_p]),
    "jja_sin_host": (c_int, [P_f64, P_f64, P_f64, c_int64]),
    "jja_last_error": (ctypes.c_char_p, []),
    "jja_launch_count": (c_int64, []),
}


class JJAError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"libjja_gb300 error {code}: {msg}")
        self.code = code


def lib():
    """Load (building first if needed) and return the ctypes library handle."""
    global _lib
    with _lock:
        if _lib is None:
            path = _build.LIB
            if not _build.up_to_date():
                path = _build.build()
            if not os.path.exists(path):
                raise RuntimeError(f"libjja_gb300.so not found at {path}")
            L = ctypes.CDLL(path)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def check(code):
    if code != 0:
        raise JJAError(code, lib().jja_last_error().decode())


def ptr(arr, ctype=c_double):
    """ctypes pointer to a contiguous numpy array (None -> NULL)."""
    if arr is None:
        return None
    return arr.ctypes.data_as(ctypes.POINTER(ctype))
