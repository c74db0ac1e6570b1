"""ctypes binding of libhodlrnd_gb300.so (the C ABI in include/hodlrnd.h).

There is no fallback: if the library is missing this raises, naming the
build command.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
# HODLRND_LIBRARY selects another build of the library (for example one
# compiled with different HODLR_TUNE_* ring shapes)
LIB_PATH = os.environ.get("HODLRND_LIBRARY") or os.path.join(HERE, "libhodlrnd_gb300.so")

HODLR_OK = 0
HODLR_ERR_INVALID = 1
HODLR_ERR_CUDA = 2
HODLR_ERR_OOM = 3
HODLR_ERR_BUDGET = 4
HODLR_ERR_NOT_CONVERGED = 5
HODLR_ERR_TREE = 6
HODLR_ERR_STATE = 7
HODLR_ERR_DEVICE = 8
HODLR_ERR_IO = 9
HODLR_ERR_TIMEOUT = 10

HODLR_KERNEL_INV_R = 1
HODLR_KERNEL_INV_R2 = 2
HODLR_KERNEL_LOG_R = 3
HODLR_KERNEL_EXP_NEG_R = 4

HODLR_PREC_FP64 = 0
HODLR_PREC_MIXED = 1
HODLR_PREC_FP32_FACTORS = 2
HODLR_PREC_BF16_FACTORS = 3

HODLR_ORTHO_AUTO = 0
HODLR_ORTHO_MGS = 1
HODLR_ORTHO_CGS2 = 2

HODLR_FP64_CHECK_AUTO = 0
HODLR_FP64_CHECK_OFF = 1

HODLR_RELAX_AUTO = 0
HODLR_RELAX_OFF = 1
HODLR_RELAX_ALWAYS = 2


def relax_code(relax):
    """True: relaxed products once the residual allows; False: never; "always": every product."""
    if isinstance(relax, str):
        if relax != "always":
            raise ValueError(f"relax: True, False or 'always', not {relax!r}")
        return HODLR_RELAX_ALWAYS
    return HODLR_RELAX_AUTO if relax else HODLR_RELAX_OFF


class HodlrParams(ctypes.Structure):
    _fields_ = [("ndim", ctypes.c_int32), ("nmax", ctypes.c_int32), ("dprime", ctypes.c_int32),
                ("restart", ctypes.c_int32), ("eps_aca", ctypes.c_double), ("tol", ctypes.c_double),
                ("max_iter", ctypes.c_int64), ("precision", ctypes.c_int32), ("device", ctypes.c_int32),
                ("device_budget_bytes", ctypes.c_uint64), ("rank_cap", ctypes.c_int32),
                ("max_outer", ctypes.c_int32), ("inner_tol", ctypes.c_double), ("ortho", ctypes.c_int32),
                ("relax", ctypes.c_int32), ("relax_below", ctypes.c_double),
                ("fp64_check", ctypes.c_int32), ("aca_workspace_mib", ctypes.c_int32),
                ("stored_margin", ctypes.c_double)]


class HodlrKernelDesc(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("reserved", ctypes.c_int32), ("scale", ctypes.c_double),
                ("diag", ctypes.c_double)]


class HodlrSolveInfo(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int64), ("outer_iterations", ctypes.c_int64),
                ("rel_residual", ctypes.c_double), ("converged", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("seconds", ctypes.c_double), ("stop_tol", ctypes.c_double),
                ("rel_residual_stored", ctypes.c_double)]


class HodlrStats(ctypes.Structure):
    _fields_ = [(k, ctypes.c_int64) for k in ("n", "depth", "n_leaves", "n_far_blocks", "n_dense_far_blocks",
                                              "n_near_blocks", "max_rank")] + \
               [(k, ctypes.c_double) for k in ("n_flop", "memory_gb", "compression_ratio")] + \
               [(k, ctypes.c_uint64) for k in ("near_bytes", "far_bytes", "device_bytes")] + \
               [(k, ctypes.c_double) for k in ("t_tree_s", "t_aca_s", "t_near_s", "t_build_s", "t_matvec_s",
                                               "far_entries", "dense_far_entries", "near_entries",
                                               "t_aca_kernel_s", "t_compact_s", "aca_entries")]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


TRACE_KINDS = 16
# kinds 0-3: launches with FP64 vectors (FP64 factors, or FP32 factors with
# compensated accumulation); 4-7: FP32 vectors (inner solve of iterative refinement);
# 8-11: the FP64 operator of a reduced-precision operator's refinement residuals
TRACE_NAMES = {0: "zgemv_x64", 1: "near_x64", 2: "far_x64", 3: "combine_x64", 4: "zgemv_x32", 5: "near_x32",
               6: "far_x32", 7: "combine_x32", 8: "zgemv_ref64", 9: "near_ref64", 10: "far_ref64",
               11: "combine_ref64"}


class HodlrTrace(ctypes.Structure):
    _fields_ = [("launches", ctypes.c_uint64 * TRACE_KINDS), ("total_ms", ctypes.c_double * TRACE_KINDS),
                ("bytes_per_launch", ctypes.c_double * TRACE_KINDS)]


class HodlrError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[hodlr error {code}] {msg}")
        self.code = code


_lib = None


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with `python -m hodlrnd_gb300.build` "
                          "(there is no CPU fallback)")
    L = ctypes.CDLL(LIB_PATH)
    P, D, I64, I32 = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int64), \
        ctypes.POINTER(ctypes.c_int32)
    L.hodlr_params_default.argtypes = [ctypes.POINTER(HodlrParams)]
    L.hodlr_params_default.restype = None
    L.hodlr_ctx_create.argtypes = [ctypes.POINTER(HodlrParams), ctypes.POINTER(P)]
    L.hodlr_ctx_destroy.argtypes = [P]
    L.hodlr_last_error.argtypes = [P]
    L.hodlr_last_error.restype = ctypes.c_char_p
    L.hodlr_build.argtypes = [P, D, ctypes.c_int64, D, D, ctypes.POINTER(HodlrKernelDesc), ctypes.POINTER(P)]
    L.hodlr_op_destroy.argtypes = [P]
    L.hodlr_matvec.argtypes = [P, D, D, ctypes.c_int64]
    L.hodlr_matvec_device.argtypes = [P, P, P, ctypes.c_int64, P]
    L.hodlr_solve.argtypes = [P, D, D, ctypes.c_int64, ctypes.POINTER(HodlrSolveInfo)]
    L.hodlr_solve_device.argtypes = [P, P, P, ctypes.c_int64, P, ctypes.POINTER(HodlrSolveInfo)]
    L.hodlr_stats_get.argtypes = [P, ctypes.POINTER(HodlrStats)]
    L.hodlr_get_permutation.argtypes = [P, I64]
    L.hodlr_get_blocks.argtypes = [P, I32, I64, I64, I32]
    L.hodlr_set_solver.argtypes = [P, ctypes.c_int32, ctypes.c_double, ctypes.c_int64, ctypes.c_double, ctypes.c_int32]
    L.hodlr_get_block.argtypes = [P, ctypes.c_int64, I32, I32, I32, I32, D, D]
    L.hodlr_trace_enable.argtypes = [P, ctypes.c_int]
    L.hodlr_trace_get.argtypes = [P, ctypes.POINTER(HodlrTrace)]
    L.hodlr_kernel_launches.argtypes = []
    L.hodlr_kernel_launches.restype = ctypes.c_uint64
    L.hodlr_tree_build.argtypes = [ctypes.POINTER(HodlrParams), D, ctypes.c_int64, D, D, ctypes.POINTER(P)]
    L.hodlr_tree_build_device.argtypes = [ctypes.POINTER(HodlrParams), D, ctypes.c_int64, D, D, ctypes.POINTER(P)]
    L.hodlr_tree_build_device.restype = ctypes.c_int
    L.hodlr_tree_sizes.argtypes = [P, I64]
    L.hodlr_tree_get.argtypes = [P, I64, I64, I64, I64, I64, I64, I64]
    L.hodlr_tree_destroy.argtypes = [P]
    L.hodlr_set_relax.argtypes = [P, ctypes.c_int32, ctypes.c_double]
    L.hodlr_op_save.argtypes = [P, D, ctypes.c_char_p]
    L.hodlr_op_load.argtypes = [P, ctypes.c_char_p, ctypes.POINTER(P)]
    L.hodlr_vec_load.argtypes = [ctypes.c_char_p, D, ctypes.c_int64, I64]
    L.hodlr_vec_save.argtypes = [ctypes.c_char_p, D, ctypes.c_int64]
    L.hodlr_matvec_tc_device.argtypes = [P, P, P, ctypes.c_int64, P]
    L.hodlr_matvec_tc_device.restype = ctypes.c_int
    L.hodlr_tc_selftest.argtypes = [P, P, ctypes.c_int32, ctypes.c_int32, P]
    L.hodlr_tc_selftest.restype = ctypes.c_int
    for f in ("hodlr_op_save", "hodlr_op_load", "hodlr_set_relax", "hodlr_vec_load", "hodlr_vec_save", "hodlr_ctx_create", "hodlr_ctx_destroy", "hodlr_build", "hodlr_op_destroy", "hodlr_matvec",
              "hodlr_matvec_device", "hodlr_solve", "hodlr_solve_device", "hodlr_stats_get",
              "hodlr_get_permutation", "hodlr_get_blocks", "hodlr_tree_build", "hodlr_tree_sizes",
              "hodlr_tree_get", "hodlr_tree_destroy", "hodlr_get_block", "hodlr_trace_enable", "hodlr_trace_get", "hodlr_set_solver"):
        getattr(L, f).restype = ctypes.c_int
    _lib = L
    return L


def last_error(ctx=None):
    return lib().hodlr_last_error(ctx).decode(errors="replace")


def check(code, ctx=None):
    if code != HODLR_OK:
        raise HodlrError(code, last_error(ctx))
