"""ctypes binding of the C ABI declared in include/bembel_gb300.h.

The shared library is built in-tree (bembel_gb300/_build). There is no CPU
fallback: every numerical entry point runs on the GPU and reports an error
when the library or the device is unavailable.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libbembel_gb300.so")

BG_OK, BG_INVALID_ARG, BG_OOM, BG_UNSUPPORTED, BG_DEVICE_ERROR, BG_TIMEOUT, BG_CANCELLED, BG_NOT_CONVERGED = range(8)
STATUS_NAMES = ["BG_OK", "BG_INVALID_ARG", "BG_OOM", "BG_UNSUPPORTED", "BG_DEVICE_ERROR", "BG_TIMEOUT",
                "BG_CANCELLED", "BG_NOT_CONVERGED"]
LAPLACE_SL, HELMHOLTZ_SL, MAXWELL_SL = 0, 1, 2
PREC_FP64, PREC_MIXED, PREC_FP32 = 0, 1, 2
PRECISIONS = {"fp64": PREC_FP64, "mixed": PREC_MIXED, "fp32": PREC_FP32}


class H2Params(ctypes.Structure):
    _fields_ = [("n_p", ctypes.c_int), ("eta", ctypes.c_double), ("min_cluster_level", ctypes.c_int),
                ("store_fp64_far", ctypes.c_int), ("keep_fp64_blocks", ctypes.c_int)]


class SolveParams(ctypes.Structure):
    _fields_ = [("tol", ctypes.c_double), ("restart", ctypes.c_int), ("max_iter", ctypes.c_int),
                ("inner_precision", ctypes.c_int), ("inner_tol", ctypes.c_double),
                ("max_refinements", ctypes.c_int)]


class SolveStats(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("refinements", ctypes.c_int), ("fp64_matvecs", ctypes.c_int),
                ("low_matvecs", ctypes.c_int), ("final_relres", ctypes.c_double)]


class LaunchPlan(ctypes.Structure):
    _fields_ = [("near_kernel", ctypes.c_int), ("split_k_batches", ctypes.c_int), ("far_order", ctypes.c_int),
                ("transforms", ctypes.c_int), ("far_ctas", ctypes.c_int),
                ("mixed_near", ctypes.c_int), ("far_tiles", ctypes.c_int)]


class TuneReport(ctypes.Structure):
    _fields_ = [("candidates", ctypes.c_int), ("builtin_ms", ctypes.c_double), ("tuned_ms", ctypes.c_double),
                ("plan", LaunchPlan)]


class Request(ctypes.Structure):
    _fields_ = [("geometry", ctypes.c_int), ("op_kind", ctypes.c_int), ("M", ctypes.c_int), ("P", ctypes.c_int),
                ("kre", ctypes.c_double), ("kim", ctypes.c_double), ("data_kind", ctypes.c_int),
                ("nrhs", ctypes.c_int), ("data", ctypes.POINTER(ctypes.c_double)), ("tol", ctypes.c_double),
                ("inner_precision", ctypes.c_int), ("x", ctypes.c_void_p), ("x_capacity", ctypes.c_long)]


class RequestResult(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("N", ctypes.c_int), ("t_submit", ctypes.c_double),
                ("t_start", ctypes.c_double), ("t_done", ctypes.c_double), ("cache_hit", ctypes.c_int),
                ("batch_nrhs", ctypes.c_int), ("stats", SolveStats), ("error", ctypes.c_char * 160)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_long), ("completed", ctypes.c_long), ("failed", ctypes.c_long),
                ("batches", ctypes.c_long), ("cache_hits", ctypes.c_long), ("cache_misses", ctypes.c_long),
                ("evictions", ctypes.c_long), ("bytes_in_use", ctypes.c_size_t), ("bytes_budget", ctypes.c_size_t),
                ("assembly_s", ctypes.c_double), ("solve_s", ctypes.c_double), ("cached_operators", ctypes.c_int)]


class BembelError(RuntimeError):
    def __init__(self, status, message):
        name = STATUS_NAMES[status] if 0 <= status < len(STATUS_NAMES) else str(status)
        super().__init__("%s: %s" % (name, message))
        self.status = status


_lib = None


def load(build_if_missing=True):
    """Load the in-tree library (building it with nvcc if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise RuntimeError("bembel_gb300 library not built: %s" % LIB_PATH)
        from . import build as _build
        _build.build()
    L = ctypes.CDLL(LIB_PATH)
    P, I, D, Lg = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_long
    dp, ip, lp = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_long)
    PP = ctypes.POINTER(ctypes.c_void_p)
    sig = {
        "bg_h2_params_default": (None, [ctypes.POINTER(H2Params)]),
        "bg_solve_params_default": (None, [ctypes.POINTER(SolveParams)]),
        "bg_context_create": (I, [I, PP]),
        "bg_context_destroy": (I, [P]),
        "bg_last_error_string": (ctypes.c_char_p, [P]),
        "bg_profile_classes": (I, [P, ctypes.c_uint]),
        "bg_geometry_load_dat": (I, [P, ctypes.c_char_p, PP]),
        "bg_geometry_load_igs": (I, [P, ctypes.c_char_p, PP]),
        "bg_geometry_cube_sphere": (I, [P, PP]),
        "bg_geometry_destroy": (I, [P]),
        "bg_geometry_surface_point": (I, [P, I, D, D, dp]),
        "bg_operator_create": (I, [P, P, I, I, I, ctypes.POINTER(H2Params), PP]),
        "bg_operator_set_wavenumber": (I, [P, D, D]),
        "bg_operator_assemble": (I, [P]),
        "bg_operator_destroy": (I, [P]),
        "bg_operator_info": (I, [P, lp]),
        "bg_operator_assembly_times": (I, [P, dp]),
        "bg_operator_prepare_wavenumbers": (I, [P, dp, dp, I]),
        "bg_operator_release_wavenumbers": (I, [P]),
        "bg_operator_assemble_wavenumbers": (I, [P]),
        "bg_operator_num_wavenumbers": (I, [P, ip, dp, dp]),
        "bg_operator_quadrature_counts": (I, [P, lp]),
        "bg_matvec": (I, [P, P, Lg, P, Lg, I, dp, dp, I, I]),
        "bg_load_vector": (I, [P, I, dp, I, P, I]),
        "bg_solve": (I, [P, P, P, I, ctypes.POINTER(SolveParams), ctypes.POINTER(SolveStats), I]),
        "bg_potential": (I, [P, P, I, dp, I, P]),
        "bg_operator_elements": (I, [P, ip, dp]),
        "bg_operator_leaves": (I, [P, ip]),
        "bg_operator_transform": (I, [P, ip, ip, dp]),
        "bg_operator_leaf_block": (I, [P, Lg, I, I, dp]),
        "bg_operator_memory": (I, [P, ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_size_t)]),
        "bg_watchdog_selftest": (I, [P, ctypes.c_longlong]),
        "bg_operator_set_plan": (I, [P, I, I, ctypes.POINTER(LaunchPlan)]),
        "bg_operator_get_plan": (I, [P, I, I, ctypes.POINTER(LaunchPlan)]),
        "bg_operator_autotune": (I, [P, I, I, I, ctypes.POINTER(TuneReport)]),
        "bg_geometry_num_patches": (I, [P, ip]),
        "bg_server_create": (I, [P, ctypes.c_size_t, I, PP]),
        "bg_server_destroy": (I, [P]),
        "bg_server_add_geometry": (I, [P, P, ip]),
        "bg_server_submit": (I, [P, ctypes.POINTER(Request), lp]),
        "bg_server_wait": (I, [P, Lg, D, ctypes.POINTER(RequestResult)]),
        "bg_server_stats_get": (I, [P, ctypes.POINTER(ServerStats)]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(status, ctx_handle=None):
    if status != BG_OK:
        msg = ""
        if ctx_handle:
            msg = load().bg_last_error_string(ctx_handle).decode()
        raise BembelError(status, msg)
