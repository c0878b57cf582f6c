"""Host-side mirror of the reference's K-SVD interface over the C ABI.

The reference drives K-SVD through ``KSVD::ExecuteIterations(iternum)`` (KSVD.cu:55-131) with the
stages ``OMP::BatchOMP()`` (OMP.cu:42-59), ``DictionaryUpdate::updateDictionary(perm)``
(DictionaryUpdate.cu:45-203), ``KSVD::errorComputation`` (KSVD.cu:235-262), ``KSVD::clearDict``
(KSVD.cu:138-226) and ``KSVD::normcols`` (KSVD.cu:267-286), all on device buffers it owns
(DeviceMemory.cu:19-138).  ``KSVD`` below has the same stages and the same error behaviour as
the C ABI (a ``KsvdError`` carrying the ksvd_status instead of the reference's ``bool false``).

Tensor layouts (torch, row-major views of the reference's column-major arrays):
``X`` (N, n), ``D`` (K, n), ``G`` (K, K), ``alpha0`` (N, K), sparse code ``idx`` (N, T) int32,
``coef`` (N, T) float32, ``nnz`` (N,) int32.  All on the CUDA device, contiguous, float32.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native
from ._native import KsvdError, Params, check

__all__ = ["Handle", "KSVD", "KsvdError", "random_permutation", "PRECISIONS"]

PRECISIONS = {"fp32": _native.PREC_FP32, "mixed": _native.PREC_MIXED}


def _ptr(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _need(t, name, dtype, shape=None):
    import torch

    if not isinstance(t, torch.Tensor):
        raise TypeError("%s must be a torch tensor" % name)
    if t.device.type != "cuda":
        raise ValueError("%s must live on the CUDA device" % name)
    if t.dtype != dtype:
        raise TypeError("%s must be %s, got %s" % (name, dtype, t.dtype))
    if not t.is_contiguous():
        raise ValueError("%s must be contiguous" % name)
    if shape is not None and tuple(t.shape) != tuple(shape):
        raise ValueError("%s must have shape %s, got %s" % (name, shape, tuple(t.shape)))
    return t


def random_permutation(seed: int, iteration: int, K: int) -> np.ndarray:
    """The library's atom order for one sweep (host-only, no GPU needed)."""
    lib = _native.load()
    out = np.empty(K, np.int32)
    check(lib.ksvd_random_permutation(C.c_uint64(seed), iteration, K,
                                      out.ctypes.data_as(C.c_void_p)))
    return out


class Handle:
    """One ksvd_handle: problem sizes, parameters, stream and device workspace."""

    def __init__(self, n, K, T, precision="fp32", mu_thresh=0.8, use_thresh=4,
                 max_replace_signals=5000, seed=0x4B535644, stream=None, profile=False,
                 refine_final=False, graph=False):
        import torch

        self._lib = _native.load()
        p = Params()
        self._lib.ksvd_default_params(C.byref(p))
        p.n, p.K, p.T = int(n), int(K), int(T)
        p.precision = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        p.mu_thresh = float(mu_thresh)
        p.use_thresh = int(use_thresh)
        p.max_replace_signals = int(max_replace_signals)
        p.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
        p.flags = ((_native.FLAG_PROFILE if profile else 0)
                   | (_native.FLAG_REFINE_FINAL if refine_final else 0)
                   | (_native.FLAG_GRAPH if graph else 0))
        self.params = p
        self.n, self.K, self.T = p.n, p.K, p.T
        if stream is None:
            stream = torch.cuda.current_stream()
        self.stream = stream
        h = C.c_void_p()
        check(self._lib.ksvd_create(C.byref(h), C.byref(p), C.c_void_p(stream.cuda_stream)))
        self._h = h

    # -- lifecycle
    def close(self):
        if getattr(self, "_h", None):
            self._lib.ksvd_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, st):
        check(st, self._h)

    @property
    def workspace_bytes(self) -> int:
        return int(self._lib.ksvd_workspace_bytes(self._h))

    def synchronize(self):
        self._check(self._lib.ksvd_synchronize(self._h))

    def remove_row_mean(self, X):
        """X (N, n) device tensor: subtract each of the n rows' mean over the signals, in place.
        Returns the means (n,)."""
        import torch

        _need(X, "X", torch.float32, (X.shape[0], self.n))
        mean = torch.empty((self.n,), dtype=torch.float32, device=X.device)
        self._check(self._lib.ksvd_remove_row_mean(self._h, _ptr(X), X.shape[0], _ptr(mean)))
        return mean

    @property
    def perm_draws(self) -> int:
        """Atom orders drawn so far (saved with D for checkpoint/resume)."""
        return int(self._lib.ksvd_perm_draws(self._h))

    @perm_draws.setter
    def perm_draws(self, v):
        self._check(self._lib.ksvd_set_perm_draws(self._h, int(v)))

    def autotune(self, D, X):
        """Time launch shapes on this problem and keep the fastest; returns the choice."""
        t = _native.Tuning()
        self._check(self._lib.ksvd_autotune(self._h, _ptr(D), _ptr(X), X.shape[0], C.byref(t)))
        return t.as_dict()

    def autotune_batched(self, problems):
        arr, _ = self._problems(problems)
        t = _native.Tuning()
        self._check(self._lib.ksvd_autotune_batched(self._h, arr, len(problems), C.byref(t)))
        return t.as_dict()

    @property
    def tuning(self):
        t = _native.Tuning()
        self._check(self._lib.ksvd_get_tuning(self._h, C.byref(t)))
        return t.as_dict()

    @tuning.setter
    def tuning(self, d):
        cur = self.tuning                  # keys left out keep their current values
        cur.update({k: int(v) for k, v in d.items()})
        t = _native.Tuning(**cur)
        self._check(self._lib.ksvd_set_tuning(self._h, C.byref(t)))

    def graph_replays(self) -> int:
        """Iterations ksvd_iterate / ksvd_batched_iterate ran as CUDA-graph replays."""
        return int(self._lib.ksvd_graph_replays(self._h))

    def stage_times(self, reset=False):
        """{stage: (milliseconds, calls)} accumulated while profiling (profile=True)."""
        t = _native.StageTimes()
        self._check(self._lib.ksvd_read_stage_times(self._h, C.byref(t), int(bool(reset))))
        return {name: (t.ms[i], int(t.calls[i])) for i, name in enumerate(_native.STAGES)}

    # -- stages
    def normcols(self, D):
        import torch

        _need(D, "D", torch.float32, (self.K, self.n))
        self._check(self._lib.ksvd_normcols(self._h, _ptr(D)))
        return D

    def gram(self, D):
        import torch

        _need(D, "D", torch.float32, (self.K, self.n))
        G = torch.empty((self.K, self.K), dtype=torch.float32, device=D.device)
        self._check(self._lib.ksvd_gram(self._h, _ptr(D), _ptr(G)))
        return G

    def dtx(self, D, X):
        import torch

        _need(D, "D", torch.float32, (self.K, self.n))
        _need(X, "X", torch.float32)
        N = X.shape[0]
        A0 = torch.empty((N, self.K), dtype=torch.float32, device=X.device)
        self._check(self._lib.ksvd_dtx(self._h, _ptr(D), _ptr(X), N, _ptr(A0)))
        return A0

    def _code(self, N, device):
        import torch

        idx = torch.empty((N, self.T), dtype=torch.int32, device=device)
        coef = torch.empty((N, self.T), dtype=torch.float32, device=device)
        nnz = torch.empty((N,), dtype=torch.int32, device=device)
        return idx, coef, nnz

    def omp_gram(self, G, A0, xnorm2=None, eps2=None):
        import torch

        _need(G, "G", torch.float32, (self.K, self.K))
        _need(A0, "alpha0", torch.float32)
        N = A0.shape[0]
        idx, coef, nnz = self._code(N, A0.device)
        self._check(self._lib.ksvd_omp_gram(self._h, _ptr(G), _ptr(A0), N, _ptr(xnorm2),
                                            _ptr(eps2), _ptr(idx), _ptr(coef), _ptr(nnz)))
        return idx, coef, nnz

    def omp(self, D, X, eps2=None, out=None):
        import torch

        _need(D, "D", torch.float32, (self.K, self.n))
        _need(X, "X", torch.float32)
        N = X.shape[0]
        if eps2 is not None:
            _need(eps2, "eps2", torch.float32, (N,))
        idx, coef, nnz = out if out is not None else self._code(N, X.device)
        self._check(self._lib.ksvd_omp(self._h, _ptr(D), _ptr(X), N, _ptr(eps2), _ptr(idx),
                                       _ptr(coef), _ptr(nnz)))
        return idx, coef, nnz

    def update_dictionary(self, D, X, idx, coef, nnz, perm=None):
        import torch

        _need(D, "D", torch.float32, (self.K, self.n))
        N = X.shape[0]
        if perm is not None:
            perm = torch.as_tensor(np.asarray(perm, np.int32)).to(D.device)
        self._check(self._lib.ksvd_update_dictionary(self._h, _ptr(D), _ptr(X), N, _ptr(idx),
                                                     _ptr(coef), _ptr(nnz), _ptr(perm)))
        return D, coef

    def error(self, D, X, idx, coef, nnz, want_err=False):
        import torch

        N = X.shape[0]
        err = torch.empty((N,), dtype=torch.float32, device=X.device) if want_err else None
        r = C.c_double()
        self._check(self._lib.ksvd_error(self._h, _ptr(D), _ptr(X), N, _ptr(idx), _ptr(coef),
                                         _ptr(nnz), _ptr(err), C.byref(r)))
        return (r.value, err) if want_err else r.value

    def clear_dict(self, D, X, idx, coef, nnz):
        N = X.shape[0]
        c = C.c_int32()
        self._check(self._lib.ksvd_clear_dict(self._h, _ptr(D), _ptr(X), N, _ptr(idx),
                                              _ptr(coef), _ptr(nnz), C.byref(c)))
        return int(c.value)

    def iterate(self, D, X, iters, perms=None, out=None, eps2=None):
        """iters K-SVD iterations on device tensors; D is updated in place.  eps2 (N,) float32
        device tensor: error-constrained coding (||x - D gamma||^2 <= eps2, at most T atoms).
        Returns (idx, coef, nnz, rmse[iters])."""
        import torch

        _need(D, "D", torch.float32, (self.K, self.n))
        _need(X, "X", torch.float32)
        N = X.shape[0]
        idx, coef, nnz = out if out is not None else self._code(N, X.device)
        rmse = np.zeros(max(iters, 1), np.float64)
        pp = None
        if perms is not None:
            perms = np.ascontiguousarray(perms, dtype=np.int32)
            if perms.shape != (iters, self.K):
                raise ValueError("perms must be (iters, K)")
            pp = perms.ctypes.data_as(C.c_void_p)
        if eps2 is not None:
            _need(eps2, "eps2", torch.float32, (N,))
            self._check(self._lib.ksvd_iterate_eps(self._h, _ptr(D), _ptr(X), N, int(iters), pp,
                                                   _ptr(eps2), _ptr(idx), _ptr(coef), _ptr(nnz),
                                                   rmse.ctypes.data_as(C.c_void_p)))
        else:
            self._check(self._lib.ksvd_iterate(self._h, _ptr(D), _ptr(X), N, int(iters), pp,
                                               _ptr(idx), _ptr(coef), _ptr(nnz),
                                               rmse.ctypes.data_as(C.c_void_p)))
        return idx, coef, nnz, rmse[:iters]

    def iterate_host(self, D, X, iters, perms=None, out=None):
        """Whole-program call with HOST numpy arrays: D (n, K) and X (n, N) column-major
        float32.  D is updated in place when it already is a float32 column-major array (a copy
        is made otherwise).  ``out`` = (idx, coef, nnz) host arrays to fill (e.g. pinned).
        Returns (D, idx, coef, nnz, rmse)."""
        if not (isinstance(D, np.ndarray) and D.dtype == np.float32 and D.flags.f_contiguous
                and D.flags.writeable):
            D = np.asfortranarray(D, dtype=np.float32).copy(order="F")
        X = np.asfortranarray(X, dtype=np.float32)
        N = X.shape[1]
        if out is None:
            out = (np.empty((N, self.T), np.int32), np.empty((N, self.T), np.float32),
                   np.empty(N, np.int32))
        idx, coef, nnz = out
        rmse = np.zeros(max(iters, 1), np.float64)
        pp = None
        if perms is not None:
            perms = np.ascontiguousarray(perms, dtype=np.int32)
            pp = perms.ctypes.data_as(C.c_void_p)
        vp = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
        self._check(self._lib.ksvd_iterate_host(self._h, vp(D), vp(X), N, int(iters), pp,
                                                vp(idx), vp(coef), vp(nnz), vp(rmse)))
        return D, idx, coef, nnz, rmse[:iters]

    def code_fixed(self, D, X, idx, nnz, save_chol=True):
        """Least-squares coefficients on fixed supports; returns (coef, chol)."""
        import torch

        N = X.shape[0]
        coef = torch.empty((N, self.T), dtype=torch.float32, device=X.device)
        chol = (torch.empty((N, self.T * (self.T + 1) // 2), dtype=torch.float32,
                            device=X.device) if save_chol else None)
        self._check(self._lib.ksvd_code_fixed(self._h, _ptr(D), _ptr(X), N, _ptr(idx), _ptr(nnz),
                                              _ptr(coef), _ptr(chol)))
        return coef, chol

    def refine_coefs(self, D, X, idx, nnz, coef, want_fp64=True):
        """One FP64-residual refinement step of ``coef`` (in place); returns the FP64 values."""
        import torch

        N = X.shape[0]
        c64 = (torch.empty((N, self.T), dtype=torch.float64, device=X.device)
               if want_fp64 else None)
        self._check(self._lib.ksvd_refine_coefs(self._h, _ptr(D), _ptr(X), N, _ptr(idx), _ptr(nnz),
                                                _ptr(coef), _ptr(c64)))
        return c64

    def code_backward(self, D, X, idx, nnz, coef, chol, dcoef, dD=None, want_dX=True):
        """Gradient through fixed-support coding: returns (dD, dX); dD accumulates."""
        import torch

        N = X.shape[0]
        if dD is None:
            dD = torch.zeros((self.K, self.n), dtype=torch.float32, device=X.device)
        dX = torch.empty_like(X) if want_dX else None
        self._check(self._lib.ksvd_code_backward(self._h, _ptr(D), _ptr(X), N, _ptr(idx),
                                                 _ptr(nnz), _ptr(coef), _ptr(chol), _ptr(dcoef),
                                                 _ptr(dD), _ptr(dX)))
        return dD, dX

    def _problems(self, problems, out=None):
        import torch

        arr = (_native.Problem * max(len(problems), 1))()
        outs = []
        for i, q in enumerate(problems):
            D, X, T = q["D"], q["X"], int(q["T"])
            K, n = D.shape
            N = X.shape[0]
            _need(D, "D", torch.float32, (K, n))
            _need(X, "X", torch.float32, (N, n))
            if out is not None:
                idx, coef, nnz = out[i]
            else:
                idx = torch.empty((N, T), dtype=torch.int32, device=X.device)
                coef = torch.empty((N, T), dtype=torch.float32, device=X.device)
                nnz = torch.empty((N,), dtype=torch.int32, device=X.device)
            e = q.get("eps2")
            if e is not None:
                _need(e, "eps2", torch.float32, (N,))
            arr[i] = _native.Problem(n, K, T, 0, N, D.data_ptr(), X.data_ptr(),
                                     e.data_ptr() if e is not None else None, idx.data_ptr(),
                                     coef.data_ptr(), nnz.data_ptr())
            outs.append((idx, coef, nnz))
        return arr, outs

    def batched_omp(self, problems, out=None):
        """Batch-OMP of many independent problems in one persistent launch.

        ``problems``: sequence of dicts with D (K, n) and X (N, n) float32 device tensors, T, and
        optional eps2 (N,) float32 (error targets).  Returns [(idx, coef, nnz), ...]."""
        arr, outs = self._problems(problems, out)
        self._check(self._lib.ksvd_batched_omp(self._h, arr, len(problems)))
        return outs

    def batched_iterate(self, problems, iters, out=None):
        """K-SVD on many independent problems (dicts as for batched_omp; each D is normalised
        and updated in place).  Returns ([(idx, coef, nnz), ...], rmse (nprob, iters))."""
        arr, outs = self._problems(problems, out)
        rmse = np.zeros((max(len(problems), 1), max(iters, 1)), np.float64)
        self._check(self._lib.ksvd_batched_iterate(self._h, arr, len(problems), int(iters),
                                                   rmse.ctypes.data_as(C.c_void_p)))
        return outs, rmse[:len(problems), :iters]

    def dense_gamma(self, idx, coef, nnz):
        import torch

        N = idx.shape[0]
        g = torch.empty((N, self.K), dtype=torch.float32, device=idx.device)
        self._check(self._lib.ksvd_dense_gamma(self._h, N, _ptr(idx), _ptr(coef), _ptr(nnz),
                                               _ptr(g)))
        return g


class KSVD:
    """The reference's KSVD object (KSVD.cuh:21-27) over device tensors it holds, like the
    reference's DeviceMemory pool: ``X`` (N, n), working dictionary ``D`` (K, n), sparse code."""

    def __init__(self, X, D, T, precision="fp32", mu_thresh=0.8, use_thresh=4,
                 max_replace_signals=5000, seed=0x4B535644):
        import torch

        self.X = _need(X, "X", torch.float32)
        self.D = D.clone().contiguous()
        self.N, n = X.shape
        K = self.D.shape[0]
        self.h = Handle(n, K, T, precision, mu_thresh, use_thresh, max_replace_signals, seed)
        self.idx, self.coef, self.nnz = self.h._code(self.N, X.device)
        self.rmse = []

    def normcols(self):                       # KSVD.cu:267-286
        self.h.normcols(self.D)

    def batch_omp(self):                      # OMP.cu:42-59
        self.h.omp(self.D, self.X, out=(self.idx, self.coef, self.nnz))

    def update_dictionary(self, perm=None):   # DictionaryUpdate.cu:45-203
        self.h.update_dictionary(self.D, self.X, self.idx, self.coef, self.nnz, perm)

    def error_computation(self):              # KSVD.cu:235-262
        r = self.h.error(self.D, self.X, self.idx, self.coef, self.nnz)
        self.rmse.append(r)
        return r

    def clear_dict(self):                     # KSVD.cu:138-226
        return self.h.clear_dict(self.D, self.X, self.idx, self.coef, self.nnz)

    def execute_iterations(self, iternum, perms=None):   # KSVD.cu:55-131
        _, _, _, r = self.h.iterate(self.D, self.X, iternum, perms,
                                    out=(self.idx, self.coef, self.nnz))
        self.rmse.extend(r.tolist())
        return r

    def dense_gamma(self):                    # main.cu:133-142 (CUDA_Gamma, transposed view)
        return self.h.dense_gamma(self.idx, self.coef, self.nnz)
