"""ctypes wrapper over the reference's own kernels compiled for the host -- TEST INFRASTRUCTURE.

``oracle/ref_build.py`` compiles the reference's ``parOMP`` (K-SVD/K-SVD/OMP.cu:126-404) and its
per-atom update kernels (K-SVD/K-SVD/Multiplication.cu:177-224) unchanged into
``oracle/_ref/libref_kernels.so`` (FP64, the reference's default ``datatype``).  The functions
here run them on numpy arrays in the reference's column-major layouts, so tests can pin the
oracle to the reference's arithmetic.  They need a reference checkout at build time; without
one (and without an already built library) ``available()`` is False.
"""
from __future__ import annotations

import ctypes as C
import threading

import numpy as np

from . import ref_build

_lock = threading.Lock()
_lib = None
# sparsities the shim instantiates (Tdata is a compile-time constant in the reference)
SUPPORTED_T = (1, 2, 3, 4, 5, 6, 7, 8, 10, 12)


def load():
    global _lib
    with _lock:
        if _lib is None:
            path = ref_build.build()
            if path is None:
                return None
            lib = C.CDLL(path)
            vp, i32 = C.c_void_p, C.c_int
            lib.ref_paromp.argtypes = [i32, vp, vp, vp, vp, i32, i32]
            lib.ref_paromp.restype = i32
            lib.ref_a_times_x.argtypes = [vp, vp, vp, i32, i32, vp, vp, i32]
            lib.ref_normal_x_times_a.argtypes = [vp, vp, vp, i32, vp, vp, vp, vp, i32, i32, vp,
                                                 vp, i32, i32]
            _lib = lib
    return _lib


def available() -> bool:
    return load() is not None


def _f64(a):
    return np.asfortranarray(np.asarray(a, dtype=np.float64))


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def paromp(G, A0, T):
    """The reference's Batch-OMP on G = D'D (K x K) and alpha0 = D'X (K x N), K <= 32.

    Returns (idx, coef, nnz) in the oracle's layout -- T slots per signal in selection order,
    -1 / 0 padding -- converted from the reference's outputs: the K x N slot map (slot + 1 of
    every chosen atom, OMP.cu:313) and the T x N coefficients (OMP.cu:350-357).  Also returns
    the raw slot map."""
    lib = load()
    G = _f64(G).copy(order="F")
    A0 = _f64(A0).copy(order="F")
    K, N = A0.shape
    sel = np.zeros((K, N), np.float64, order="F")
    c = np.zeros((T, N), np.float64, order="F")
    if lib.ref_paromp(int(T), _p(A0), _p(sel), _p(G), _p(c), K, N) != 0:
        raise ValueError("reference parOMP supports K <= 32 and T in %s" % (SUPPORTED_T,))
    idx = np.full((N, T), -1, np.int32)
    coef = np.zeros((N, T), np.float64)
    nnz = np.zeros(N, np.int32)
    for s in range(N):
        atoms = np.nonzero(sel[:, s])[0]
        slots = sel[atoms, s].astype(np.int64) - 1
        nnz[s] = len(atoms)
        idx[s, slots] = atoms
        coef[s, slots] = c[slots, s]
    return idx, coef, nnz, sel


def a_times_x(D, v, Y_j, d_j, gn2, count):
    """a = Y_j - D v + d_j * gn2 with the reference's device_A_times_x_modified."""
    lib = load()
    D = _f64(D)
    n, K = D.shape
    out = np.array(Y_j, np.float64)
    v = np.array(v, np.float64)
    d = np.array(d_j, np.float64)
    g = np.array([gn2], np.float64)
    lib.ref_a_times_x(_p(D), _p(v), _p(out), n, K, _p(d), _p(g), int(count))
    return out


def normal_x_times_a(aD, Gamma, cols, gamma_j, rowlincomb, aDj, anorm, j, a, D_col_out=None):
    """New coefficients of atom j for the signals `cols` and the new atom a / ||a|| with the
    reference's device_normal_x_times_A_modified.  Gamma is the dense K x N code (modified in
    place on a copy and returned)."""
    lib = load()
    Gam = _f64(Gamma).copy(order="F")
    K = Gam.shape[0]
    cols_f = np.array(cols, np.float64)
    gj = np.array(gamma_j, np.float64)
    rl = np.array(rowlincomb, np.float64)
    const = np.array([aDj], np.float64)
    nrm = np.array([anorm], np.float64)
    a = np.array(a, np.float64)
    n = len(a)
    dcol = np.zeros(n, np.float64) if D_col_out is None else D_col_out
    aD = np.array(aD, np.float64)
    lib.ref_normal_x_times_a(_p(aD), _p(Gam), _p(cols_f), K, _p(gj), _p(rl), _p(const),
                             _p(nrm), int(j), len(cols), _p(dcol), _p(a), n, len(cols))
    return Gam, dcol
