"""ctypes binding of libksvd_gb300.so (the C ABI in include/ksvd_gb300.h).

The library is the only compute path: if it is missing this module raises instead of falling
back to anything else.  Build it with ``ksvd_gb300.build.build()`` (or ``__graft_entry__.build()``).
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import build as _build

_lock = threading.Lock()
_lib = None

KSVD_OK = 0
STATUS_NAMES = {
    0: "KSVD_OK", 1: "KSVD_ERR_INVALID_ARGUMENT", 2: "KSVD_ERR_UNSUPPORTED",
    3: "KSVD_ERR_OUT_OF_MEMORY", 4: "KSVD_ERR_CUDA", 5: "KSVD_ERR_NUMERIC",
    6: "KSVD_ERR_TIMEOUT", 7: "KSVD_ERR_STATE",
}
PREC_FP32 = 0
PREC_MIXED = 1

# Every entry point declared in include/ksvd_gb300.h.
EXPORTS = (
    "ksvd_default_params", "ksvd_create", "ksvd_destroy", "ksvd_status_string",
    "ksvd_last_error", "ksvd_abi_version", "ksvd_workspace_bytes", "ksvd_random_permutation",
    "ksvd_normcols", "ksvd_gram", "ksvd_dtx", "ksvd_omp_gram", "ksvd_omp",
    "ksvd_update_dictionary", "ksvd_error", "ksvd_clear_dict", "ksvd_iterate",
    "ksvd_iterate_host", "ksvd_dense_gamma", "ksvd_synchronize", "ksvd_read_stage_times",
    "ksvd_rmse_noalloc", "ksvd_code_fixed", "ksvd_code_backward",
    "ksvd_refine_coefs", "ksvd_batched_omp", "ksvd_graph_replays",
    "ksvd_batched_iterate", "ksvd_remove_row_mean", "ksvd_perm_draws", "ksvd_set_perm_draws",
    "ksvd_autotune", "ksvd_autotune_batched", "ksvd_get_tuning", "ksvd_set_tuning",
    "ksvd_iterate_eps",
)

FLAG_PROFILE = 1
FLAG_REFINE_FINAL = 2
FLAG_GRAPH = 4
STAGES = ("gram", "dtx", "omp", "lists", "sweep", "error", "clear")


class StageTimes(C.Structure):
    _fields_ = [("ms", C.c_double * 8), ("calls", C.c_int64 * 8)]


class Params(C.Structure):
    _fields_ = [
        ("n", C.c_int32), ("K", C.c_int32), ("T", C.c_int32), ("precision", C.c_int32),
        ("mu_thresh", C.c_float), ("use_thresh", C.c_int32),
        ("max_replace_signals", C.c_int32), ("flags", C.c_int32), ("seed", C.c_uint64),
    ]


class Tuning(C.Structure):
    """ksvd_tuning: launch shapes chosen per handle."""
    _fields_ = [("omp_grid_mult", C.c_int32), ("sweep_ctas", C.c_int32),
                ("batch_chunk", C.c_int32), ("batch_concurrent", C.c_int32),
                ("tuned", C.c_int32), ("omp_fp16", C.c_int32)]

    def as_dict(self):
        return {k: int(getattr(self, k)) for k, _ in self._fields_}


class Problem(C.Structure):
    """ksvd_problem: one problem of a batched call (device pointers)."""
    _fields_ = [("n", C.c_int32), ("K", C.c_int32), ("T", C.c_int32), ("reserved", C.c_int32),
                ("N", C.c_int64), ("D", C.c_void_p), ("X", C.c_void_p), ("eps2", C.c_void_p),
                ("idx", C.c_void_p), ("coef", C.c_void_p), ("nnz", C.c_void_p)]


class KsvdError(RuntimeError):
    """A non-OK ksvd_status, with the library's message."""

    def __init__(self, status: int, message: str):
        self.status = status
        self.status_name = STATUS_NAMES.get(status, str(status))
        super().__init__("%s: %s" % (self.status_name, message))


def library_path() -> str:
    return _build.LIB_PATH


def _declare(lib):
    vp, i32, i64, u64 = C.c_void_p, C.c_int32, C.c_int64, C.c_uint64
    st = C.c_int
    sig = {
        "ksvd_default_params": (None, [C.POINTER(Params)]),
        "ksvd_create": (st, [C.POINTER(vp), C.POINTER(Params), vp]),
        "ksvd_destroy": (None, [vp]),
        "ksvd_status_string": (C.c_char_p, [st]),
        "ksvd_last_error": (C.c_char_p, [vp]),
        "ksvd_abi_version": (i32, []),
        "ksvd_workspace_bytes": (i64, [vp]),
        "ksvd_random_permutation": (st, [u64, i64, i32, vp]),
        "ksvd_normcols": (st, [vp, vp]),
        "ksvd_gram": (st, [vp, vp, vp]),
        "ksvd_dtx": (st, [vp, vp, vp, i64, vp]),
        "ksvd_omp_gram": (st, [vp, vp, vp, i64, vp, vp, vp, vp, vp]),
        "ksvd_omp": (st, [vp, vp, vp, i64, vp, vp, vp, vp]),
        "ksvd_update_dictionary": (st, [vp, vp, vp, i64, vp, vp, vp, vp]),
        "ksvd_error": (st, [vp, vp, vp, i64, vp, vp, vp, vp, vp]),
        "ksvd_clear_dict": (st, [vp, vp, vp, i64, vp, vp, vp, vp]),
        "ksvd_iterate": (st, [vp, vp, vp, i64, i32, vp, vp, vp, vp, vp]),
        "ksvd_iterate_host": (st, [vp, vp, vp, i64, i32, vp, vp, vp, vp, vp]),
        "ksvd_dense_gamma": (st, [vp, i64, vp, vp, vp, vp]),
        "ksvd_synchronize": (st, [vp]),
        "ksvd_read_stage_times": (st, [vp, C.POINTER(StageTimes), i32]),
        "ksvd_rmse_noalloc": (st, [i32, i32, i32, vp, vp, i64, vp, vp, vp, C.POINTER(C.c_double),
                                   vp]),
        "ksvd_code_fixed": (st, [vp, vp, vp, i64, vp, vp, vp, vp]),
        "ksvd_code_backward": (st, [vp, vp, vp, i64, vp, vp, vp, vp, vp, vp, vp]),
        "ksvd_refine_coefs": (st, [vp, vp, vp, i64, vp, vp, vp, vp]),
        "ksvd_batched_omp": (st, [vp, vp, i32]),
        "ksvd_graph_replays": (i64, [vp]),
        "ksvd_batched_iterate": (st, [vp, vp, i32, i32, vp]),
        "ksvd_remove_row_mean": (st, [vp, vp, i64, vp]),
        "ksvd_perm_draws": (i64, [vp]),
        "ksvd_set_perm_draws": (st, [vp, i64]),
        "ksvd_autotune": (st, [vp, vp, vp, i64, vp]),
        "ksvd_autotune_batched": (st, [vp, vp, i32, vp]),
        "ksvd_get_tuning": (st, [vp, vp]),
        "ksvd_set_tuning": (st, [vp, vp]),
        "ksvd_iterate_eps": (st, [vp, vp, vp, i64, i32, vp, vp, vp, vp, vp, vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args


def load(path: str | None = None):
    """Load the shared library (never builds it; a missing library is an error)."""
    global _lib
    with _lock:
        if _lib is None:
            p = path or library_path()
            if not os.path.exists(p):
                raise RuntimeError(
                    "libksvd_gb300.so not found at %s; build it with "
                    "`python -c 'import ksvd_gb300.build as b; b.build()'`" % p)
            lib = C.CDLL(p)
            _declare(lib)
            _lib = lib
    return _lib


def check(status: int, handle=None):
    if status != KSVD_OK:
        lib = load()
        msg = lib.ksvd_last_error(handle).decode() if handle else ""
        if not msg:
            msg = lib.ksvd_status_string(status).decode()
        raise KsvdError(status, msg)
