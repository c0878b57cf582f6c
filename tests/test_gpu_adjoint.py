"""Adjoint of fixed-support coding (ksvd_code_fixed / ksvd_code_backward through the C ABI) on
the adjoint workload's shape: n=128, K=512, N=100,000, T=12, supports from the library's OMP.

Loss L = ||X - D Gamma||_F^2 + 1/2 ||W Gamma||_F^2, W a seeded 10 x K Gaussian matrix.  The library
gives the part of dL/dD and dL/dX that flows through the coding step (from dL/dGamma and the
saved Cholesky factors); the direct terms -2 R Gamma' and 2 R are added here.  Checks:
  * coefficients vs FP64 least squares on the same supports: relative RMSE <= 1e-4;
  * the backward pass vs the FP64 adjoint (oracle/adjoint.py): relative RMSE <= 1e-4 for dD, dX;
  * the full gradient vs FP64 central differences (h=1e-3) on 1,000 sampled entries (500 of D,
    500 of X): max |error| <= 1e-3 x max |gradient| over the sample.
"""
import numpy as np
import pytest

from conftest import rel_rmse

pytestmark = pytest.mark.gpu


def test_adjoint_matches_fp64_and_finite_differences(cuda):
    import torch

    from ksvd_gb300 import Handle, datagen
    from oracle import adjoint as A

    p = datagen.make_problem("cfg4", dict_from="extra")
    c = p["cfg"]
    n, K, T = c.n, c.K, c.T
    X64 = np.asarray(p["X"], np.float64)
    D64 = np.asarray(p["D"], np.float64)
    D64 /= np.linalg.norm(D64, axis=0)
    N = X64.shape[1]
    Xd = torch.from_numpy(np.ascontiguousarray(X64.T.astype(np.float32))).to(cuda)
    Dd = torch.from_numpy(np.ascontiguousarray(D64.T.astype(np.float32))).to(cuda)
    D64 = Dd.double().cpu().numpy().T                         # the FP32 values the GPU sees
    X64 = Xd.double().cpu().numpy().T
    h = Handle(n, K, T)
    idx_d, _, nnz_d = h.omp(Dd, Xd)
    coef_d, chol_d = h.code_fixed(Dd, Xd, idx_d, nnz_d)
    h.synchronize()
    idx = idx_d.cpu().numpy()
    nnz = nnz_d.cpu().numpy()
    assert nnz.min() >= 1
    coef_ref = A.code_fixed(D64, X64, idx, nnz)
    assert rel_rmse(coef_d.cpu().numpy(), coef_ref) <= 1e-4

    W = np.random.default_rng(0x4B535644 + 4).standard_normal((10, K))
    dcoef = A.dcoef_w(D64, X64, idx, nnz, coef_ref, W)
    dD_d, dX_d = h.code_backward(Dd, Xd, idx_d, nnz_d, coef_d, chol_d,
                                 torch.from_numpy(dcoef.astype(np.float32)).to(cuda))
    h.synchronize()
    dD_ref, dX_ref = A.code_backward(D64, X64, idx, nnz, coef_ref, dcoef)
    dD_g = dD_d.double().cpu().numpy().T
    dX_g = dX_d.double().cpu().numpy().T
    assert rel_rmse(dD_g, dD_ref) <= 1e-4
    assert rel_rmse(dX_g, dX_ref) <= 1e-4

    # full gradient = direct terms + the library's adjoint, against central differences
    gD, gX, _, _ = A.grad_w(D64, X64, idx, nnz, W)
    full_D = gD - dD_ref + dD_g
    full_X = gX - dX_ref + dX_g
    rng = np.random.default_rng(4)
    used = np.unique(idx[idx >= 0])
    entD = [(int(rng.integers(n)), int(rng.choice(used))) for _ in range(500)]
    entX = [(int(rng.integers(n)), int(rng.integers(N))) for _ in range(500)]
    fdD = A.fd_grad_D(D64, X64, idx, nnz, W, entD)
    fdX = A.fd_grad_X(D64, X64, idx, nnz, W, entX)
    gd = np.array([full_D[i, j] for i, j in entD])
    gx = np.array([full_X[i, s] for i, s in entX])
    assert np.abs(gd - fdD).max() <= 1e-3 * np.abs(fdD).max()
    assert np.abs(gx - fdX).max() <= 1e-3 * np.abs(fdX).max()
    h.close()


def test_adjoint_ragged_and_empty_supports(cuda):
    """Supports of 0..T atoms (signals with none give zero coefficients and zero gradient)."""
    import torch

    from ksvd_gb300 import Handle
    from oracle import adjoint as A

    rng = np.random.default_rng(5)
    n, K, N, T = 40, 64, 3000, 9
    D = rng.standard_normal((n, K))
    D /= np.linalg.norm(D, axis=0)
    X = rng.standard_normal((n, N))
    nnz = rng.integers(0, T + 1, N).astype(np.int32)
    idx = np.full((N, T), -1, np.int32)
    for s in range(N):
        idx[s, : nnz[s]] = rng.choice(K, nnz[s], replace=False)
    D = D.astype(np.float32).astype(np.float64)
    X = X.astype(np.float32).astype(np.float64)
    Dd = torch.from_numpy(np.ascontiguousarray(D.T.astype(np.float32))).to(cuda)
    Xd = torch.from_numpy(np.ascontiguousarray(X.T.astype(np.float32))).to(cuda)
    idx_d = torch.from_numpy(idx).to(cuda)
    nnz_d = torch.from_numpy(nnz).to(cuda)
    h = Handle(n, K, T)
    coef_d, chol_d = h.code_fixed(Dd, Xd, idx_d, nnz_d)
    coef_ref = A.code_fixed(D, X, idx, nnz)
    assert rel_rmse(coef_d.cpu().numpy(), coef_ref) <= 1e-4
    dcoef = rng.standard_normal((N, T)) * (np.arange(T)[None, :] < nnz[:, None])
    dD_d, dX_d = h.code_backward(Dd, Xd, idx_d, nnz_d, coef_d, chol_d,
                                 torch.from_numpy(dcoef.astype(np.float32)).to(cuda))
    dD_ref, dX_ref = A.code_backward(D, X, idx, nnz, coef_ref, dcoef)
    assert rel_rmse(dD_d.double().cpu().numpy().T, dD_ref) <= 1e-4
    assert rel_rmse(dX_d.double().cpu().numpy().T, dX_ref) <= 1e-4
    zero = nnz == 0
    assert np.all(dX_d.cpu().numpy()[zero] == 0) and np.all(coef_d.cpu().numpy()[zero] == 0)
    h.close()


@pytest.mark.parametrize("precision", ["fp32", "mixed"])
def test_fp64_refinement_of_coefficients(cuda, precision):
    """One FP64-residual refinement step takes the OMP's FP32 (or BF16-mixed) least-squares
    coefficients to the FP64 least-squares solution on the same supports: relative RMSE <= 1e-10
    (the unrefined coefficients sit near 1e-7..1e-3)."""
    import torch

    from ksvd_gb300 import Handle, datagen
    from oracle import adjoint as A

    p = datagen.make_problem("cfg2", N=20000, dict_from="extra")
    c = p["cfg"]
    Xd = torch.from_numpy(np.ascontiguousarray(np.asarray(p["X"], np.float32).T)).to(cuda)
    D = np.asarray(p["D"], np.float64)
    Dd = torch.from_numpy(np.ascontiguousarray((D / np.linalg.norm(D, axis=0)).T
                                               .astype(np.float32))).to(cuda)
    h = Handle(c.n, c.K, c.T, precision=precision)
    idx_d, coef_d, nnz_d = h.omp(Dd, Xd)
    before = coef_d.double().cpu().numpy()
    c64 = h.refine_coefs(Dd, Xd, idx_d, nnz_d, coef_d)
    h.synchronize()
    D64 = Dd.double().cpu().numpy().T
    X64 = Xd.double().cpu().numpy().T
    idx, nnz = idx_d.cpu().numpy(), nnz_d.cpu().numpy()
    want = A.code_fixed(D64, X64, idx, nnz)
    e0 = rel_rmse(before, want)
    e1 = rel_rmse(c64.cpu().numpy(), want)
    assert e1 <= 1e-10, (e0, e1)
    assert e1 < 1e-3 * e0
    assert rel_rmse(coef_d.double().cpu().numpy(), want) <= 1e-7   # FP32 rounding of the result
    h.close()


def test_iterate_refine_final(cuda):
    """KSVD_FLAG_REFINE_FINAL: the coefficients ksvd_iterate returns are the least-squares ones on
    the final dictionary and supports, and reconstruct no worse than the sweep's."""
    import torch

    from ksvd_gb300 import Handle, datagen
    from oracle import adjoint as A

    p = datagen.make_problem("cfg0", N=4000, dict_from="extra")
    c = p["cfg"]
    X = torch.from_numpy(np.ascontiguousarray(np.asarray(p["X"], np.float32).T)).to(cuda)
    D0 = torch.from_numpy(np.ascontiguousarray(np.asarray(p["D"], np.float32).T)).to(cuda)
    outs = []
    for refine in (False, True):
        h = Handle(c.n, c.K, c.T, refine_final=refine)
        D = D0.clone()
        idx, coef, nnz, rmse = h.iterate(D, X, 3)
        h.synchronize()
        outs.append((D.double().cpu().numpy().T, idx.cpu().numpy(), coef.double().cpu().numpy(),
                     nnz.cpu().numpy(), rmse))
        h.close()
    (Da, ia, ca, na, ra), (Db, ib, cb, nb, rb) = outs
    np.testing.assert_allclose(ra, rb, rtol=1e-4)      # two runs: float atomics reorder sums
    X64 = X.double().cpu().numpy().T
    want = A.code_fixed(Db, X64, ib, nb)
    assert rel_rmse(cb, want) <= 1e-6

    def res(Dm, i, cf, nz):
        R = X64.copy()
        for s in range(len(nz)):
            R[:, s] -= Dm[:, i[s, : nz[s]]] @ cf[s, : nz[s]]
        return np.sum(R * R)

    assert res(Db, ib, cb, nb) <= res(Da, ia, ca, na) * (1 + 1e-4)
