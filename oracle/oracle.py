"""ctypes wrapper over ``ksvd_oracle.cpp`` -- TEST INFRASTRUCTURE ONLY.

The C++ restatement of the reference's K-SVD path (patschris/KSVD, K-SVD/K-SVD/{KSVD,OMP,
DictionaryUpdate,Reduction,ReductionKernels,Multiplication}.cu) is compiled by ``build()`` into
``oracle/_build/libksvd_oracle.so`` with g++ and OpenMP.  Every function takes and returns numpy
arrays in the reference's layouts: column-major ``X`` (n x N), ``D`` (n x K), ``G`` (K x K),
``alpha0`` (K x N), and the sparse code as ``idx``/``coef`` (T slots per signal, selection order,
-1/0 padding) plus ``nnz`` (atoms per signal).

Parity status: unpinned against the reference's own numbers (the reference cannot run here);
pinned against its recorded output structure and first-principles known answers.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "ksvd_oracle.cpp")
_OUT_DIR = os.path.join(_HERE, "_build")
_LIB_PATH = os.path.join(_OUT_DIR, "libksvd_oracle.so")
_lock = threading.Lock()
_lib = None

__all__ = [
    "build", "load", "num_threads", "normcols", "gram", "dtx", "omp", "update", "error",
    "cleardict", "ksvd", "dense_gamma",
]


def build(force: bool = False) -> str:
    """Compile the oracle (portable flags: no -march=native, same results on x86 and Arm)."""
    os.makedirs(_OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(_LIB_PATH)
            and os.path.getmtime(_LIB_PATH) >= os.path.getmtime(_SRC)):
        return _LIB_PATH
    tmp = _LIB_PATH + ".tmp%d" % os.getpid()
    cmd = ["g++", "-O3", "-fopenmp", "-std=c++17", "-shared", "-fPIC", _SRC, "-o", tmp]
    subprocess.run(cmd, check=True)
    os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


def _sig(lib):
    i32, i64, vp, dbl = C.c_int, C.c_int64, C.c_void_p, C.c_double
    for suf, real in (("f32", C.c_float), ("f64", C.c_double)):
        getattr(lib, "oracle_normcols_" + suf).argtypes = [i32, i32, vp]
        getattr(lib, "oracle_gram_" + suf).argtypes = [i32, i32, vp, vp]
        getattr(lib, "oracle_dtx_" + suf).argtypes = [i32, i32, i64, vp, vp, vp]
        getattr(lib, "oracle_omp_" + suf).argtypes = [i32, i64, i32, vp, vp, vp, vp, vp, vp, vp]
        getattr(lib, "oracle_update_" + suf).argtypes = [
            i32, i32, i64, i32, vp, vp, vp, vp, vp, vp, i32, vp, vp, vp, vp]
        f = getattr(lib, "oracle_error_" + suf)
        f.argtypes = [i32, i64, i32, vp, vp, vp, vp, vp, vp, vp]
        f.restype = dbl
        f = getattr(lib, "oracle_cleardict_" + suf)
        f.argtypes = [i32, i32, i64, i32, vp, vp, vp, vp, vp, vp, vp, real, i32]
        f.restype = i32
        f = getattr(lib, "oracle_ksvd_" + suf)
        f.argtypes = [i32, i32, i64, i32, vp, vp, i32, vp, real, i32, i32, vp, vp, vp, vp]
        f.restype = i32
    lib.oracle_num_threads.restype = i32


def load():
    global _lib
    with _lock:
        if _lib is None:
            path = build()
            lib = C.CDLL(path)
            _sig(lib)
            _lib = lib
    return _lib


def num_threads() -> int:
    return int(load().oracle_num_threads())


def _suf(dtype) -> str:
    dtype = np.dtype(dtype)
    if dtype == np.float32:
        return "f32"
    if dtype == np.float64:
        return "f64"
    raise TypeError("oracle works in float32 or float64, got %s" % dtype)


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _fortran(a, dtype):
    """Column-major (MATLAB layout) contiguous copy of a 2-D array."""
    return np.asfortranarray(np.asarray(a, dtype=dtype))


def normcols(D):
    D = _fortran(D, D.dtype).copy(order="F")
    n, K = D.shape
    getattr(load(), "oracle_normcols_" + _suf(D.dtype))(n, K, _p(D))
    return D


def gram(D):
    D = _fortran(D, D.dtype)
    n, K = D.shape
    G = np.empty((K, K), dtype=D.dtype, order="F")
    getattr(load(), "oracle_gram_" + _suf(D.dtype))(n, K, _p(D), _p(G))
    return G


def dtx(D, X):
    D = _fortran(D, D.dtype)
    X = _fortran(X, D.dtype)
    n, K = D.shape
    N = X.shape[1]
    A0 = np.empty((K, N), dtype=D.dtype, order="F")
    getattr(load(), "oracle_dtx_" + _suf(D.dtype))(n, K, N, _p(D), _p(X), _p(A0))
    return A0


def omp(G, A0, T, xnorm2=None, eps2=None):
    """Batch-OMP on precomputed G = D'D and alpha0 = D'X.  Returns (idx, coef, nnz) with idx and
    coef shaped (N, T) in selection order."""
    G = _fortran(G, G.dtype)
    A0 = _fortran(A0, G.dtype)
    K, N = A0.shape
    idx = np.empty((N, T), dtype=np.int32)
    coef = np.empty((N, T), dtype=G.dtype)
    nnz = np.empty(N, dtype=np.int32)
    if eps2 is not None:
        eps2 = np.ascontiguousarray(np.broadcast_to(np.asarray(eps2, G.dtype), (N,)))
        xnorm2 = np.ascontiguousarray(np.asarray(xnorm2, G.dtype))
    getattr(load(), "oracle_omp_" + _suf(G.dtype))(
        K, N, T, _p(G), _p(A0), _p(xnorm2), _p(eps2), _p(idx), _p(coef), _p(nnz))
    return idx, coef, nnz


def update(X, D, idx, coef, nnz, perm, max_signals=5000):
    """One dictionary sweep.  Returns (D, coef, state) with state holding bitmap, replaced,
    unused and counter after the sweep."""
    D = _fortran(D, D.dtype).copy(order="F")
    X = _fortran(X, D.dtype)
    n, K = D.shape
    N, T = idx.shape
    idx = np.ascontiguousarray(idx, dtype=np.int32)
    coef = np.ascontiguousarray(coef, dtype=D.dtype).copy()
    nnz = np.ascontiguousarray(nnz, dtype=np.int32)
    perm = np.ascontiguousarray(perm, dtype=np.int32)
    bitmap = np.empty(N, np.int32)
    replaced = np.empty(K, np.int32)
    unused = np.empty(N, np.int32)
    counter = np.zeros(1, np.int64)
    getattr(load(), "oracle_update_" + _suf(D.dtype))(
        n, K, N, T, _p(X), _p(D), _p(idx), _p(coef), _p(nnz), _p(perm), int(max_signals),
        _p(bitmap), _p(replaced), _p(unused), _p(counter))
    return D, coef, dict(bitmap=bitmap, replaced=replaced, unused=unused, counter=int(counter[0]))


def error(X, D, idx, coef, nnz, bitmap=None):
    """Returns (rmse, err_masked)."""
    D = _fortran(D, D.dtype)
    X = _fortran(X, D.dtype)
    n, K = D.shape
    N, T = idx.shape
    idx = np.ascontiguousarray(idx, dtype=np.int32)
    coef = np.ascontiguousarray(coef, dtype=D.dtype)
    nnz = np.ascontiguousarray(nnz, dtype=np.int32)
    if bitmap is not None:
        bitmap = np.ascontiguousarray(bitmap, dtype=np.int32)
    err = np.empty(N, dtype=D.dtype)
    r = getattr(load(), "oracle_error_" + _suf(D.dtype))(
        n, N, T, _p(X), _p(D), _p(idx), _p(coef), _p(nnz), _p(bitmap), _p(err))
    return float(r), err


def cleardict(X, D, idx, coef, nnz, replaced, err_masked, mu_thresh=0.8, use_thresh=4):
    """Returns (D, err_masked, cleared)."""
    D = _fortran(D, D.dtype).copy(order="F")
    X = _fortran(X, D.dtype)
    n, K = D.shape
    N, T = idx.shape
    err = np.ascontiguousarray(err_masked, dtype=D.dtype).copy()
    c = getattr(load(), "oracle_cleardict_" + _suf(D.dtype))(
        n, K, N, T, _p(X), _p(D), _p(np.ascontiguousarray(idx, np.int32)),
        _p(np.ascontiguousarray(coef, D.dtype)), _p(np.ascontiguousarray(nnz, np.int32)),
        _p(np.ascontiguousarray(replaced, np.int32)), _p(err), float(mu_thresh), int(use_thresh))
    return D, err, int(c)


def ksvd(X, D, T, iters, perms, mu_thresh=0.8, use_thresh=4, max_signals=5000):
    """Full ExecuteIterations (normcols once, then iters x {G, D'X, OMP, update, error,
    clearDict}).  Returns (D, idx, coef, nnz, rmse[iters])."""
    D = _fortran(D, D.dtype).copy(order="F")
    X = _fortran(X, D.dtype)
    n, K = D.shape
    N = X.shape[1]
    perms = np.ascontiguousarray(perms, dtype=np.int32)
    assert perms.shape == (iters, K)
    idx = np.empty((N, T), np.int32)
    coef = np.empty((N, T), D.dtype)
    nnz = np.empty(N, np.int32)
    rmse = np.empty(iters, np.float64)
    getattr(load(), "oracle_ksvd_" + _suf(D.dtype))(
        n, K, N, T, _p(X), _p(D), int(iters), _p(perms), float(mu_thresh), int(use_thresh),
        int(max_signals), _p(idx), _p(coef), _p(nnz), _p(rmse))
    return D, idx, coef, nnz, rmse


def dense_gamma(idx, coef, nnz, K):
    """Dense K x N coefficient matrix (the reference's CUDA_Gamma layout, main.cu:133-142)."""
    N, T = idx.shape
    G = np.zeros((K, N), dtype=coef.dtype)
    for t in range(T):
        m = t < nnz
        G[idx[m, t], np.nonzero(m)[0]] = coef[m, t]
    return G
