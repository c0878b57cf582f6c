"""Mixed precision (tcgen05 BF16 hi/lo GEMMs with FP32 accumulation) against the FP64 oracle.
Tolerances: D'X and D'D relative RMSE <= 2e-5 (three hi/lo passes keep ~16 mantissa bits of each
product); K-SVD RMSE per iteration within 1% of the FP64 oracle; Batch-OMP supports identical on
>= 99.9% of signals."""
import numpy as np
import pytest

from conftest import rel_rmse, support_match_vec
from test_gpu_ksvd import from_dev, problem, to_dev

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,K,N", [(256, 1024, 5000), (64, 256, 1000), (200, 100, 777),
                                   (300, 9, 3600), (16, 40, 300)])
def test_tc_gemms_match_fp64(oracle_mod, cuda, n, K, N):
    from ksvd_gb300 import Handle

    X, D = problem(n, K, N, min(4, K), 40)
    h = Handle(n, K, min(4, K), precision="mixed")
    Xd, Dd = to_dev(X, cuda), to_dev(D, cuda)
    A0 = from_dev(h.dtx(Dd, Xd))
    G = from_dev(h.gram(Dd))
    h.synchronize()
    X64, D64 = X.astype(np.float64), D.astype(np.float64)
    assert rel_rmse(A0, D64.T @ X64) < 2e-5
    assert rel_rmse(G, D64.T @ D64) < 2e-5
    h.close()


def test_mixed_omp_supports(oracle_mod, cuda):
    from ksvd_gb300 import Handle

    n, K, N, T = 256, 1024, 4000, 16
    X, D = problem(n, K, N, T, 41)
    h = Handle(n, K, T, precision="mixed")
    idx, coef, nnz = h.omp(to_dev(D, cuda), to_dev(X, cuda))
    h.synchronize()
    X64, D64 = X.astype(np.float64), D.astype(np.float64)
    ri, rc, rn = oracle_mod.omp(oracle_mod.gram(D64), oracle_mod.dtx(D64, X64), T)
    assert support_match_vec(idx.cpu().numpy(), nnz.cpu().numpy(), ri, rn) >= 0.999
    h.close()


@pytest.mark.parametrize("cfg,N,iters", [("cfg0", 4000, 3), ("cfg2", 20000, 2)])
def test_mixed_iterations_match_fp64_rmse(oracle_mod, cuda, cfg, N, iters):
    from ksvd_gb300 import Handle, datagen, random_permutation

    p = datagen.make_problem(cfg, N=N, dict_from="extra")
    c = p["cfg"]
    perms = np.stack([random_permutation(5, it, c.K) for it in range(iters)])
    Dr, ri, rc, rn, rr = oracle_mod.ksvd(p["X"].astype(np.float64), p["D"].astype(np.float64),
                                         c.T, iters, perms)
    h = Handle(c.n, c.K, c.T, precision="mixed")
    Dd = to_dev(p["D"], cuda)
    idx, coef, nnz, rmse = h.iterate(Dd, to_dev(p["X"], cuda), iters, perms)
    np.testing.assert_allclose(rmse, rr, rtol=1e-2)
    h.close()
