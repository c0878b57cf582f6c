"""ksvd_rmse_noalloc: the RMSE entry point for callers that cannot allocate device memory (their
memory belongs to another allocator, or cudaMalloc's implicit synchronisation is not acceptable
on their path).  Called through the C ABI twice in a row, it must give the RMSE that ksvd_error
(the handle-based entry point, which uses its own workspace) gives, to 1e-6 relative -- tighter
than the 1e-4 the parity tests allow.  This file sorts last so a stop-at-first-failure run has
already run every other test; it also passes on its own in a fresh process."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev(a, cuda):
    import torch

    return torch.from_numpy(np.ascontiguousarray(np.asarray(a).T)).to(cuda)


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
    got = []
    for _ in range(2):
        r = C.c_double(-1.0)
        st = lib.ksvd_rmse_noalloc(c.n, c.K, c.T, C.c_void_p(D.data_ptr()), C.c_void_p(X.data_ptr()),
                                   X.shape[0], C.c_void_p(idx.data_ptr()),
                                   C.c_void_p(coef.data_ptr()), C.c_void_p(nnz.data_ptr()),
                                   C.byref(r), stream)
        assert st == 0, lib.ksvd_last_error(None).decode()
        got.append(r.value)
    for g in got:
        assert abs(g - want) <= 1e-6 * want, (g, want)
    # the size limit is enforced before anything runs
    r = C.c_double()
    st = lib.ksvd_rmse_noalloc(c.n, c.K, c.T, C.c_void_p(D.data_ptr()), C.c_void_p(X.data_ptr()),
                               256 * 65536 + 1, C.c_void_p(idx.data_ptr()),
                               C.c_void_p(coef.data_ptr()), C.c_void_p(nnz.data_ptr()),
                               C.byref(r), stream)
    assert st == 2 and "16,777,216" in lib.ksvd_last_error(None).decode()
    h.close()
