"""Mixed precision (tcgen05 BF16 hi/lo GEMMs with FP32 accumulation) against the FP64 oracle.
Tolerances: D'X and D'D relative RMSE <= 2e-5 (three hi/lo passes keep ~16 mantissa bits of each
product); K-SVD RMSE per iteration within 1% of the FP64 oracle; Batch-OMP supports identical on
>= 99.9% of signals."""
import numpy as np
import pytest

from conftest import rel_rmse, support_match_vec, touched_atoms
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
    """The mixed path's whole iterations against the FP64 oracle.  After one iteration: supports
    identical on >= 99.9% of signals, the dictionary within 5e-4 relative RMSE over the atoms no
    differently coded signal touches (5e-3 over all when a signal is coded differently), the
    RMSE within 1e-4.  Over `iters` iterations: every iteration's RMSE within 1% (later supports
    drift apart as in any two implementations that round differently)."""
    from ksvd_gb300 import Handle, datagen, random_permutation

    p = datagen.make_problem(cfg, N=N, dict_from="extra")
    c = p["cfg"]
    perms = np.stack([random_permutation(5, it, c.K) for it in range(iters)])
    X64, D64 = p["X"].astype(np.float64), p["D"].astype(np.float64)
    D1, ri1, rc1, rn1, rr1 = oracle_mod.ksvd(X64, D64, c.T, 1, perms[:1])
    h1 = Handle(c.n, c.K, c.T, precision="mixed")
    Dd1 = to_dev(p["D"], cuda)
    i1, c1, n1, r1 = h1.iterate(Dd1, to_dev(p["X"], cuda), 1, perms[:1])
    gi, gn = i1.cpu().numpy(), n1.cpu().numpy()
    match = support_match_vec(gi, gn, ri1, rn1)
    flipped, touched = touched_atoms(gi, gn, ri1, rn1, c.K)
    Dg = from_dev(Dd1)
    e_all = rel_rmse(Dg, D1)
    e_unt = rel_rmse(Dg[:, ~touched], D1[:, ~touched]) if (~touched).any() else 0.0
    r_rel = float(np.max(np.abs(np.asarray(r1) - rr1) / rr1))
    print("%s mixed: supports %.5f, %d flipped, %d touched atoms, dictionary %.2e (untouched "
          "%.2e), RMSE rel %.2e" % (cfg, match, len(flipped), touched.sum(), e_all, e_unt, r_rel))
    assert match >= 0.999
    # G and alpha0 carry ~2^-16 relative error (BF16 hi/lo products): the coefficients differ at
    # ~1e-6, and the sweep's coupling of every atom to the earlier ones carries that to ~3e-4 in
    # the dictionary (measured: 2.7e-4 at cfg0, 2.9e-4 at cfg2 over the untouched atoms)
    assert e_unt <= 5e-4
    assert e_all <= (5e-4 if len(flipped) == 0 else 5e-3)
    assert r_rel <= 1e-4
    h1.close()
    Dr, ri, rc, rn, rr = oracle_mod.ksvd(p["X"].astype(np.float64), p["D"].astype(np.float64),
                                         c.T, iters, perms)
    h = Handle(c.n, c.K, c.T, precision="mixed")
    Dd = to_dev(p["D"], cuda)
    idx, coef, nnz, rmse = h.iterate(Dd, to_dev(p["X"], cuda), iters, perms)
    np.testing.assert_allclose(rmse, rr, rtol=1e-2)
    h.close()


def _coding_inputs(case):
    """(G, alpha0, T, eps2-or-None) for the FP16 alpha update's selection test."""
    rng = np.random.default_rng(77)
    if case == "incoherent":
        X, D = problem(256, 1024, 20000, 16, 42)
        T = 16
    elif case == "coherent":
        X, D = problem(64, 256, 5000, 8, 43)
        D[:, 128:] = D[:, :128] + 0.01 * rng.standard_normal((64, 128)).astype(np.float32)
        D /= np.linalg.norm(D, axis=0)
        T = 8
    elif case == "noiseless":
        D = rng.standard_normal((128, 512))
        D /= np.linalg.norm(D, axis=0)
        X = np.zeros((128, 5000))
        for s in range(5000):
            S = rng.choice(512, 6, replace=False)
            X[:, s] = D[:, S] @ rng.standard_normal(6)
        X, D = X.astype(np.float32), D.astype(np.float32)
        T = 12
    elif case == "ragged-K":
        X, D = problem(100, 200, 5000, 10, 44)
        T = 10
    elif case in ("scale-up", "scale-down"):
        X, D = problem(128, 512, 3000, 12, 49)
        X = X * np.float32(1e4 if case == "scale-up" else 1e-4)   # coefficients far from 1
        T = 16
    elif case == "small-K":
        X, D = problem(64, 100, 3000, 10, 48)
        T = 16
    elif case == "t32":
        X, D = problem(128, 512, 3000, 24, 45)
        T = 32
    else:  # error targets
        X, D = problem(256, 1024, 10000, 16, 46)
        T = 16
    D64, X64 = D.astype(np.float64), X.astype(np.float64)
    G = (D64.T @ D64).astype(np.float32)
    A0 = (D64.T @ X64).astype(np.float32)
    eps2 = None
    if case == "eps":
        xn = np.sum(X64 * X64, axis=0)
        eps2 = (xn * rng.uniform(0.002, 0.05, X.shape[1])).astype(np.float32)
    return X, G, A0, T, eps2


@pytest.mark.parametrize("case", ["incoherent", "coherent", "noiseless", "ragged-K", "small-K",
                                  "scale-up", "scale-down", "t32", "eps"])
def test_fp16_alpha_update_selects_like_fp32(cuda, case):
    """The mixed path's Batch-OMP forms alpha from an FP16 copy of G and re-evaluates every atom
    within its rigorous error bound of the maximum in FP32 with the FP32 path's operations.  Given
    the same G and alpha0 its supports, coefficients and support sizes are bit-identical to the
    FP32 Batch-OMP's: on incoherent dictionaries (few near ties), on nearly duplicated atoms (many
    candidates: the whole-alpha FP32 fallback), on noiseless signals (the stop tests at
    exhaustion), at K not a multiple of 128 (also K <= 128: four rows per lane and group), with
    signals scaled by 1e4 and 1e-4 (the coefficients' power-of-two scaling into FP16 range), at
    T = 32 and with error targets."""
    import torch

    from ksvd_gb300 import Handle

    X, G, A0, T, eps2 = _coding_inputs(case)
    K = G.shape[0]
    Gd, Ad = to_dev(G, cuda), to_dev(A0, cuda)
    xn2 = e2 = None
    if eps2 is not None:
        xn2 = torch.from_numpy(np.sum(X.astype(np.float32) ** 2, axis=0)).to(cuda)
        e2 = torch.from_numpy(eps2).to(cuda)
    outs = []
    for prec in ("fp32", "mixed"):
        h = Handle(X.shape[0], K, T, precision=prec)
        if prec == "mixed":
            h.tuning = dict(h.tuning, omp_fp16=1)     # the FP16 update at every T
        outs.append(h.omp_gram(Gd, Ad, xn2, e2))
        h.synchronize()
        h.close()
    (ia, ca, na), (ib, cb, nb) = outs
    assert torch.equal(na, nb)
    assert torch.equal(ia, ib)
    assert torch.equal(ca, cb)


def test_fp16_update_identical_at_full_cfg2_size(cuda):
    """The FP16 alpha update against the FP32 kernel on the whole cfg2 workload (n=256, K=1024,
    1,000,000 signals, T=16) given the same G and alpha0: identical supports, coefficients and
    support sizes on every signal (the error bound is rigorous, so no mismatch is allowed)."""
    import torch

    from ksvd_gb300 import Handle, datagen

    c = datagen.CONFIGS["cfg2"]
    p = datagen.make_problem("cfg2", device="cuda")
    D = p["D"] / p["D"].norm(dim=1, keepdim=True)
    G = (D @ D.T).contiguous()
    A0 = (p["X"] @ D.T).contiguous()
    del p
    outs = []
    for prec in ("fp32", "mixed"):
        h = Handle(c.n, c.K, c.T, precision=prec)
        if prec == "mixed":
            h.tuning = dict(h.tuning, omp_fp16=1)
        outs.append(h.omp_gram(G, A0))
        h.synchronize()
        h.close()
    (ia, ca, na), (ib, cb, nb) = outs
    assert A0.shape[0] == 1_000_000
    bad = int(((ia != ib).any(1) | (ca != cb).any(1) | (na != nb)).sum())
    assert bad == 0, "%d of %d signals differ" % (bad, A0.shape[0])
