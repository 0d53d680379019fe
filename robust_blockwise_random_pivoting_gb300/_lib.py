"""ctypes binding of ``librbrp_gb300.so`` (the C ABI of ``include/rbrp_gb300.h``).

There is no fallback: if the shared library is missing, importing the
package's compute API raises, so a GPU run can never silently route around
the CUDA kernels.  Build it with ``python -m robust_blockwise_random_pivoting_gb300.build``.
"""
import ctypes
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "librbrp_gb300.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "rbrp_gb300.h")

c_int, c_double, c_uint64, c_int64, c_void_p = (ctypes.c_int, ctypes.c_double, ctypes.c_uint64,
                                                ctypes.c_int64, ctypes.c_void_p)

SAMPLERS = {"np": 0, "es": 1, "greedy": 2, "gp": 2}
PRECISIONS = {"f64": 0, "f32_mixed": 1}
STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "allocation failed",
          4: "no result computed", 5: "numerical failure", 6: "buffer too small", 7: "device wait timed out"}


class Params(ctypes.Structure):
    _fields_ = [("tol", c_double), ("b", c_int), ("kmax", c_int), ("seed", c_uint64),
                ("sampler", c_int), ("precision", c_int), ("tol_loc", c_double),
                ("compute_T", c_int), ("recompute", c_int)]


class Result(ctypes.Structure):
    _fields_ = [("k", c_int), ("nblocks", c_int), ("res0", c_double), ("err_est", c_double),
                ("draws", c_uint64), ("ms_total", c_double), ("ms_loop", c_double),
                ("ms_T", c_double), ("recomputes", c_int)]


NPHASES = 8
PHASES = ["norms", "sample", "cgs", "panel", "project", "finish", "tsolve", "update"]


class PhaseStats(ctypes.Structure):
    _fields_ = [("ms", c_double * NPHASES), ("bytes", c_double * NPHASES), ("flops", c_double * NPHASES),
                ("launches", c_int * NPHASES)]


BATCH_PHASES = ["norms", "sample", "gram", "pivot", "basis", "project", "update", "finish", "tsolve"]


class BatchProblem(ctypes.Structure):
    _fields_ = [("m", c_int), ("n", c_int), ("lda", c_int64), ("A", c_void_p), ("perm", c_void_p),
                ("T", c_void_p), ("T_cap", c_int64)]


class BatchResult(ctypes.Structure):
    _fields_ = [("k", c_int), ("nblocks", c_int), ("status", c_int), ("attempts", c_int),
                ("res0", c_double), ("err_est", c_double), ("draws", c_uint64), ("alg_bytes", c_double),
                ("alg_flops", c_double)]


class BatchInfo(ctypes.Structure):
    _fields_ = [("b", c_int), ("panel_cols", c_int), ("ctas", c_int), ("ctas_per_sm", c_int),
                ("ms_last", c_double), ("ms_autotune", c_double), ("workspace_bytes", ctypes.c_size_t)]


class RBRPError(RuntimeError):
    def __init__(self, status, detail=""):
        self.status = status
        super().__init__(f"RBRP {STATUS.get(status, status)}" + (f": {detail}" if detail else ""))


_lib = None

_SIGS = {
    "rbrp_params_default": (None, [ctypes.POINTER(Params)]),
    "rbrp_create": (c_int, [ctypes.POINTER(c_void_p), c_int]),
    "rbrp_destroy": (c_int, [c_void_p]),
    "rbrp_set_stream": (c_int, [c_void_p, c_void_p]),
    "rbrp_status_string": (ctypes.c_char_p, [c_int]),
    "rbrp_last_error": (ctypes.c_char_p, [c_void_p]),
    "rbrp_abi_version": (c_int, []),
    "rbrp_id_f64": (c_int, [c_void_p, c_int, c_int, c_void_p, c_int64, ctypes.POINTER(Params), c_void_p,
                            ctypes.POINTER(Result)]),
    "rbrp_id_f32": (c_int, [c_void_p, c_int, c_int, c_void_p, c_int64, ctypes.POINTER(Params), c_void_p,
                            ctypes.POINTER(Result)]),
    "rbrp_copy_T": (c_int, [c_void_p, c_void_p, c_int64]),
    "rbrp_copy_L": (c_int, [c_void_p, c_void_p, c_int64]),
    "rbrp_T_device": (c_int, [c_void_p, ctypes.POINTER(c_void_p), ctypes.POINTER(c_int)]),
    "rbrp_get_trace": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_int, ctypes.POINTER(c_int)]),
    "rbrp_id_error_f64": (c_int, [c_void_p, c_int, c_int, c_void_p, c_int64, ctypes.POINTER(c_double)]),
    "rbrp_id_error_f32": (c_int, [c_void_p, c_int, c_int, c_void_p, c_int64, ctypes.POINTER(c_double)]),
    "rbrp_id_f64_host": (c_int, [c_void_p, c_int, c_int, c_void_p, c_int64, ctypes.POINTER(Params), c_void_p,
                                 c_void_p, c_int64, c_int64, ctypes.POINTER(Result)]),
    "rbrp_id_f32_host": (c_int, [c_void_p, c_int, c_int, c_void_p, c_int64, ctypes.POINTER(Params), c_void_p,
                                 c_void_p, c_int64, c_int64, ctypes.POINTER(Result)]),
    "rbrp_RBRP": (c_int, [c_int, c_int, c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_int,
                          ctypes.POINTER(c_int), ctypes.POINTER(c_double), ctypes.POINTER(c_double)]),
    "rbrp_RandAdapRBRP": (c_int, [c_void_p, c_int, c_int, ctypes.POINTER(c_void_p), ctypes.POINTER(c_void_p),
                                  ctypes.POINTER(c_void_p), ctypes.POINTER(c_int), ctypes.POINTER(c_double),
                                  c_double, c_int]),
    "rbrp_free": (c_int, [c_void_p]),
    "rbrp_set_profiling": (c_int, [c_void_p, c_int]),
    "rbrp_get_phase_stats": (c_int, [c_void_p, ctypes.POINTER(PhaseStats)]),
    "rbrp_reset_phase_stats": (c_int, [c_void_p]),
    "rbrp_set_variant": (c_int, [c_void_p, c_int]),
    "rbrp_set_tsolve_fp64": (c_int, [c_void_p, c_int]),
    "rbrp_set_wait_budget": (c_int, [c_void_p, ctypes.c_longlong]),
    "rbrp_matdivide_f64": (c_int, [c_void_p, c_int, c_int, c_int, c_void_p, c_int64, c_void_p, c_int64, c_double,
                                   c_void_p, c_int64, ctypes.POINTER(c_int)]),
    "rbrp_T_matdivide": (c_int, [c_void_p, c_double, ctypes.POINTER(c_int)]),
    "rbrp_refine_T_f64": (c_int, [c_void_p, c_int, c_int, c_void_p, c_int64, c_int, c_double,
                                  ctypes.POINTER(c_double)]),
    "rbrp_refine_T_f32": (c_int, [c_void_p, c_int, c_int, c_void_p, c_int64, c_int, c_double,
                                  ctypes.POINTER(c_double)]),
    "rbrp_id_error_f64_noalloc": (c_int, [c_int, c_int, c_void_p, c_int64, c_void_p, c_int, c_void_p, c_int64,
                                          c_double, c_void_p, c_void_p]),
    "rbrp_fixed_id_f32": (c_int, [c_void_p, c_int, c_int, c_void_p, c_int64, c_void_p, c_int, c_int, c_void_p,
                                  ctypes.POINTER(Result)]),
    "rbrp_fixed_id_f64": (c_int, [c_void_p, c_int, c_int, c_void_p, c_int64, c_void_p, c_int, c_int, c_void_p,
                                  ctypes.POINTER(Result)]),
    "rbrp_fixed_id_adjoint_f32": (c_int, [c_void_p, c_int, c_int, c_void_p, c_int64, c_void_p, ctypes.c_float,
                                          c_void_p, c_int64, ctypes.POINTER(c_double)]),
    "rbrp_sketch_gaussian_f32": (c_int, [c_void_p, c_int, c_int, c_int, c_void_p, c_int64, c_uint64,
                                         ctypes.c_float, c_void_p, c_int64]),
    "rbrp_lupp_pivots_f64": (c_int, [c_void_p, c_int, c_int, c_void_p, c_int64, c_void_p, c_void_p]),
    "rbrp_RandLUPP_OS": (c_int, [c_void_p, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_uint64]),
    "rbrp_RandCPQR_OS": (c_int, [c_void_p, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_uint64]),
    "rbrp_CPQR": (c_int, [c_int, c_int, c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_void_p]),
    "rbrp_batch_plan": (c_int, [c_void_p, c_int, ctypes.POINTER(BatchProblem), ctypes.POINTER(Params)]),
    "rbrp_batch_run": (c_int, [c_void_p]),
    "rbrp_batch_results": (c_int, [c_void_p, ctypes.POINTER(BatchResult), c_int]),
    "rbrp_batch_get_info": (c_int, [c_void_p, ctypes.POINTER(BatchInfo)]),
    "rbrp_batch_set_order": (c_int, [c_void_p, ctypes.POINTER(c_int), c_int]),
    "rbrp_batch_set_profiling": (c_int, [c_void_p, c_int]),
    "rbrp_batch_get_phase_cycles": (c_int, [c_void_p, ctypes.POINTER(c_double), c_int]),
    "rbrp_id_batched_f32": (c_int, [c_void_p, c_int, ctypes.POINTER(BatchProblem), ctypes.POINTER(Params),
                                    ctypes.POINTER(BatchResult)]),
}


def header_symbols(paths=None):
    """Function names declared in the C headers (include/*.h)."""
    import glob
    paths = paths or sorted(glob.glob(os.path.join(os.path.dirname(HEADER), "*.h")))
    names = set()
    for path in paths:
        txt = open(path).read()
        names.update(re.findall(r"^\s*(?:rbrp_status|void|int|const char\s*\*)\s*(rbrp_\w+)\s*\(", txt, re.M))
    return sorted(names)


def load():
    """Load the shared library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with "
                          "`python -m robust_blockwise_random_pivoting_gb300.build` (no CPU fallback exists)")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status, handle=None):
    if status != 0:
        detail = ""
        if handle is not None:
            detail = load().rbrp_last_error(handle).decode(errors="replace")
        raise RBRPError(status, detail)
