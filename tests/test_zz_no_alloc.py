"""ksvd_rmse_noalloc: the RMSE entry point for callers that cannot allocate device memory (their
memory belongs to another allocator, or cudaMalloc's implicit synchronisation is not acceptable
on their path).  Called through the C ABI twice in a row, it must give the RMSE that ksvd_error
(the handle-based entry point, which uses its own workspace) gives, to 1e-6 relative -- tighter
than the 1e-4 the parity tests allow -- and the device's free memory must not change across the
two calls.  This file sorts last so a stop-at-first-failure run has already run every other test;
it also passes on its own in a fresh process."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev(a, cuda):
    import torch

    return torch.from_numpy(np.ascontiguousarray(np.asarray(a).T)).to(cuda)


def _call(lib, c, D, X, N, idx, coef, nnz, stream):
    r = C.c_double(-1.0)
    st = lib.ksvd_rmse_noalloc(c.n, c.K, c.T, C.c_void_p(D.data_ptr()), C.c_void_p(X.data_ptr()),
                               N, C.c_void_p(idx.data_ptr()), C.c_void_p(coef.data_ptr()),
                               C.c_void_p(nnz.data_ptr()), C.byref(r), stream)
    return st, r.value


def test_rmse_noalloc_matches_ksvd_error(cuda):
    import torch

    from ksvd_gb300 import Handle, _native, datagen

    lib = _native.load()
    p = datagen.make_problem("cfg0", N=5000, dict_from="extra")
    c = p["cfg"]
    X = _dev(p["X"], cuda)
    D = _dev(p["D"], cuda)
    h = Handle(c.n, c.K, c.T)
    idx, coef, nnz = h.omp(D, X)
    want = h.error(D, X, idx, coef, nnz)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    N = X.shape[0]
    # set-up call: the first call on a device may make the CUDA driver load the library's device
    # code (the static scratch array becomes resident then); nothing is allocated after it
    st, _ = _call(lib, c, D, X, N, idx, coef, nnz, stream)
    assert st == 0, lib.ksvd_last_error(None).decode()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    got = []
    for _ in range(2):
        st, v = _call(lib, c, D, X, N, idx, coef, nnz, stream)
        assert st == 0, lib.ksvd_last_error(None).decode()
        got.append(v)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)
    for g in got:
        assert abs(g - want) <= 1e-6 * want, (g, want)
    # the size limit is enforced before anything runs
    st, _ = _call(lib, c, D, X, 256 * 65536 + 1, idx, coef, nnz, stream)
    assert st == 2 and "16,777,216" in lib.ksvd_last_error(None).decode()
    # an unrelated call with a null handle replaces the message (no stale no-alloc text)
    assert lib.ksvd_synchronize(None) == 1
    assert "null handle" in lib.ksvd_last_error(None).decode()
    # an atom index outside [0, K) in a used slot is rejected, as ksvd_error rejects it
    bad = idx.clone()
    bad[7, 0] = c.K
    st, _ = _call(lib, c, D, X, N, bad, coef, nnz, stream)
    assert st == 1 and "outside [0, K)" in lib.ksvd_last_error(None).decode()
    st = lib.ksvd_error(h._h, C.c_void_p(D.data_ptr()), C.c_void_p(X.data_ptr()), N,
                        C.c_void_p(bad.data_ptr()), C.c_void_p(coef.data_ptr()),
                        C.c_void_p(nnz.data_ptr()), None, C.byref(C.c_double()))
    assert st == 1, lib.ksvd_last_error(h._h).decode()
    # and a good call afterwards still gives the same value
    st, v = _call(lib, c, D, X, N, idx, coef, nnz, stream)
    assert st == 0 and abs(v - want) <= 1e-6 * want
    h.close()
