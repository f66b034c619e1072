"""ctypes binding of libgrns_gb300.so (the C ABI declared in include/grns/grns.h).

The library is built in-tree by grns_gb300/build.py.  There is no CPU or
pure-PyTorch fallback: if the library is missing or fails to load, every
entry point raises.
"""
import ctypes
import os

from . import build as _build

_lib = None

c_int, c_int64, c_size_t, c_void_p, c_uint32 = ctypes.c_int, ctypes.c_int64, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_uint32

# name -> (restype, argtypes)
SIGNATURES = {
    "grns_status_string": (ctypes.c_char_p, [c_int]),
    "grns_version": (ctypes.c_char_p, []),
    "grns_ctx_create": (c_int, [c_void_p, c_int, ctypes.POINTER(c_void_p)]),
    "grns_ctx_destroy": (c_int, [c_void_p]),
    "grns_params_parse": (c_int, [ctypes.c_char_p, c_void_p, c_int, c_void_p, c_void_p]),
    "grns_ctx_create_from_params": (c_int, [ctypes.c_char_p, ctypes.POINTER(c_void_p)]),
    "grns_ctx_n": (c_int, [c_void_p]),
    "grns_ctx_log2": (c_int, [c_void_p]),
    "grns_ctx_get_table": (c_int, [c_void_p, c_int, c_void_p, c_size_t]),
    "grns_ctx_set_path": (c_int, [c_void_p, c_int]),
    "grns_ctx_set_eval_split": (c_int, [c_void_p, c_int]),
    "grns_ctx_get_eval_split": (c_int, [c_void_p]),
    "grns_device_ceil_log2": (c_int, [c_void_p, c_void_p, c_int64, c_void_p]),
    "grns_eval": (c_int, [c_void_p, c_void_p, c_int64, c_int, c_void_p, c_void_p, c_void_p]),
    "grns_eval_tight": (c_int, [c_void_p, c_void_p, c_int64, c_int, c_void_p, c_void_p, c_void_p]),
    "grns_cmp": (c_int, [c_void_p, c_void_p, c_void_p, c_int64, c_int, c_void_p, c_void_p, c_void_p]),
    "grns_div": (c_int, [c_void_p, c_void_p, c_void_p, c_int64, c_int, c_void_p, c_void_p, c_void_p, c_void_p]),
    "grns_scale2pow": (c_int, [c_void_p, c_void_p, c_void_p, c_uint32, c_int64, c_int, c_void_p, c_void_p, c_void_p]),
    "grns_mpint_add": (c_int, [c_void_p, c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_void_p]),
    "grns_mpint_sub": (c_int, [c_void_p, c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_void_p]),
    "grns_mpint_mul": (c_int, [c_void_p, c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_void_p]),
    "grns_mpint_div": (c_int, [c_void_p, c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_void_p]),
    "grns_ctx_binary_limbs": (c_int, [c_void_p]),
    "grns_mrc": (c_int, [c_void_p, c_void_p, c_int64, c_int, c_void_p, c_void_p, c_void_p]),
    "grns_eval_fast": (c_int, [c_void_p, c_void_p, c_int64, c_int, c_void_p, c_void_p, c_void_p]),
    "grns_div_host": (c_int, [c_void_p, c_void_p, c_void_p, c_int64, c_int, c_void_p, c_void_p, c_void_p, c_int,
                              c_void_p]),
    "grns_scale2pow_host": (c_int, [c_void_p, c_void_p, c_void_p, ctypes.c_uint32, c_int64, c_int, c_void_p, c_void_p,
                                    c_int, c_void_p]),
    "grns_from_binary": (c_int, [c_void_p, c_void_p, c_int, c_int64, c_int, c_void_p, c_void_p]),
    "grns_to_binary": (c_int, [c_void_p, c_void_p, c_int64, c_int, c_void_p, c_int, c_void_p, c_void_p]),
    "grns_mpint_from_binary": (c_int, [c_void_p, c_void_p, c_int, c_void_p, c_int64, c_void_p, c_void_p]),
    "grns_mpint_to_binary": (c_int, [c_void_p, c_void_p, c_int64, c_void_p, c_int, c_void_p, c_void_p, c_void_p]),
    "grns_max_scratch_size": (c_int, [c_void_p, c_int64, ctypes.POINTER(c_size_t)]),
    "grns_max": (c_int, [c_void_p, c_void_p, c_int64, c_int, c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    "grns_max_noalloc": (c_int, [c_void_p, c_void_p, c_int64, c_int, c_void_p, c_void_p, c_void_p]),
    "grns_batch_create": (c_int, [c_void_p, c_void_p, c_int, c_int, ctypes.POINTER(c_void_p)]),
    "grns_batch_update": (c_int, [c_void_p, c_void_p, c_int]),
    "grns_batch_launch": (c_int, [c_void_p, c_void_p]),
    "grns_batch_destroy": (c_int, [c_void_p]),
    "grns_batch_chunks": (c_int64, [c_void_p]),
    "grns_batch_grid": (c_int, [c_void_p]),
    "grns_ctx_get_schedule": (c_int, [c_void_p, c_int, c_void_p]),
    "grns_ctx_set_schedule": (c_int, [c_void_p, c_int, c_void_p]),
    "grns_autotune": (c_int, [c_void_p, c_int, c_int64, ctypes.c_char_p, c_void_p, ctypes.POINTER(ctypes.c_double)]),
    "grns_autotune_load": (c_int, [c_void_p, ctypes.c_char_p, ctypes.POINTER(c_int)]),
    "grns_server_create": (c_int, [c_void_p, ctypes.POINTER(c_void_p)]),
    "grns_server_destroy": (c_int, [c_void_p]),
    "grns_server_add_context": (c_int, [c_void_p, c_void_p, ctypes.POINTER(c_int)]),
    "grns_server_put": (c_int, [c_void_p, c_int, c_int, c_void_p, c_int, c_int64, c_int, ctypes.POINTER(ctypes.c_uint64)]),
    "grns_server_get": (c_int, [c_void_p, ctypes.c_uint64, c_void_p, c_size_t]),
    "grns_server_array_info": (c_int, [c_void_p, ctypes.c_uint64, ctypes.POINTER(c_int64), ctypes.POINTER(c_size_t),
                                       ctypes.POINTER(c_void_p)]),
    "grns_server_free": (c_int, [c_void_p, ctypes.c_uint64]),
    "grns_server_submit": (c_int, [c_void_p, c_void_p, ctypes.POINTER(ctypes.c_uint64)]),
    "grns_server_poll": (c_int, [c_void_p, ctypes.c_uint64, ctypes.POINTER(c_int), ctypes.POINTER(ctypes.c_int32),
                                 ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]),
    "grns_server_wait": (c_int, [c_void_p, ctypes.c_uint64, c_int64, ctypes.POINTER(ctypes.c_int32),
                                 ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]),
    "grns_server_stats_get": (c_int, [c_void_p, c_void_p]),
    "grns_server_cancel": (c_int, [c_void_p, ctypes.c_uint64]),
    "grns_server_reset_stats": (c_int, [c_void_p]),
    "grns_server_set_gather_us": (c_int, [c_void_p, ctypes.c_int32]),
    "grns_gen_uniform": (c_int, [c_void_p, ctypes.c_uint64, c_uint32, c_int64, c_int, c_void_p, c_void_p]),
    "grns_gen_divisors": (c_int, [c_void_p, ctypes.c_uint64, c_int64, c_int, c_void_p, c_void_p]),
    "grns_gen_shifts": (c_int, [ctypes.c_uint64, c_int64, c_uint32, c_void_p, c_void_p]),
    "grns_gen_mpint": (c_int, [c_void_p, ctypes.c_uint64, c_int64, c_int, c_void_p, c_void_p]),
}


class Job(ctypes.Structure):
    """grns_job (include/grns/grns.h)"""
    _fields_ = [("op", ctypes.c_int32), ("layout", ctypes.c_int32), ("count", ctypes.c_int64),
                ("ld", ctypes.c_int64), ("a", c_void_p), ("b", c_void_p), ("out0", c_void_p),
                ("out1", c_void_p), ("flags", c_void_p), ("eval_a", c_void_p), ("eval_b", c_void_p),
                ("D_uniform", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


class Schedule(ctypes.Structure):
    _fields_ = [("coop", ctypes.c_int32), ("chunk", ctypes.c_int32)]


class ServerOptions(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", c_size_t), ("launch_slots", ctypes.c_int32),
                ("max_jobs_per_launch", ctypes.c_int32), ("admission_timeout_ms", ctypes.c_int32),
                ("direct_min_count", ctypes.c_int32), ("alloc_cap_bytes", c_size_t),
                ("gather_us", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class Request(ctypes.Structure):
    _fields_ = [("op", ctypes.c_int32), ("ctx_index", ctypes.c_int32), ("count", ctypes.c_int64),
                ("a", ctypes.c_uint64), ("b", ctypes.c_uint64), ("D_uniform", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32)]


class ServerStats(ctypes.Structure):
    _fields_ = [("completed", ctypes.c_uint64), ("rejected", ctypes.c_uint64), ("pending", ctypes.c_uint64),
                ("inflight", ctypes.c_uint64), ("launches", ctypes.c_uint64), ("p50_us", ctypes.c_double),
                ("p99_us", ctypes.c_double), ("mean_us", ctypes.c_double), ("numbers_per_s", ctypes.c_double),
                ("mean_jobs_per_launch", ctypes.c_double), ("bytes_in_use", c_size_t), ("budget", c_size_t)]


ARRAY_RNS, ARRAY_U32, ARRAY_MPINT, ARRAY_INTERVAL, ARRAY_MAXOUT = range(5)

OP_EVAL, OP_CMP, OP_DIV, OP_SCALE2POW, OP_MAX, OP_MPINT_ADD, OP_MPINT_SUB, OP_MPINT_MUL, OP_MPINT_DIV = range(9)


class GrnsError(RuntimeError):
    def __init__(self, status, what=""):
        self.status = status
        msg = lib().grns_status_string(status).decode()
        super().__init__(f"{what}: {msg} (status {status})" if what else f"{msg} (status {status})")


def lib_path():
    return _build.LIB


def lib(build_if_missing=False):
    """Load the native library (building it first only when asked)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if build_if_missing:
            _build.build()
        else:
            raise RuntimeError(f"grns_gb300 native library not built ({path}); run grns_gb300/build.py")
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(status, what=""):
    if status != 0:
        raise GrnsError(status, what)
