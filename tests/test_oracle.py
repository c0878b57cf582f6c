"""The CPU oracle pinned against the reference's recorded fixtures, first-principles known
answers and an independent numpy restatement of the reference's arithmetic (CPU only)."""
import os

import numpy as np
import pytest

from conftest import rel_rmse, support_match

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


# ---------------------------------------------------------------- independent numpy restatement

def np_omp(G, a0, T):
    """Batch-OMP of one signal, written from the algorithm (not from the C++ oracle)."""
    K = len(a0)
    I, gam = [], np.zeros(0)
    alpha = a0.copy()
    while len(I) < T:
        p = int(np.argmax(alpha * alpha))
        if p in I or alpha[p] ** 2 < 1e-14:
            break
        if I:
            GI = G[np.ix_(I, I)]
            w = np.linalg.solve(np.linalg.cholesky(GI), G[I, p])
            if 1.0 - w @ w <= 1e-14:
                break
        I.append(p)
        gam = np.linalg.solve(G[np.ix_(I, I)], a0[I])
        alpha = a0 - G[:, I] @ gam
    return I, gam


def np_update(X, D, Gam, perm, max_signals=5000):
    """Approximate K-SVD sweep on a dense Gamma (K x N), reference order of operations."""
    D = D.copy()
    Gam = Gam.copy()
    n, K = D.shape
    N = X.shape[1]
    lists = [np.nonzero(Gam[j])[0] for j in range(K)]
    gn2 = np.array([np.sum(Gam[j, lists[j]] ** 2) for j in range(K)])
    Y = np.stack([X[:, lists[j]] @ Gam[j, lists[j]] for j in range(K)], 1)
    unused = list(range(N))
    counter = 0
    replaced = np.zeros(K, np.int32)
    bitmap = np.ones(N, np.int32)
    for j in perm:
        I = lists[j]
        if len(I) == 0:
            ncand = min(max_signals, N - counter)
            cand = unused[:ncand]
            E = np.sum((X[:, cand] - D @ Gam[:, cand]) ** 2, 0)
            b = int(np.argmax(E))
            s = cand[b]
            D[:, j] = X[:, s] / np.linalg.norm(X[:, s])
            unused[b] = unused[N - counter - 1]
            counter += 1
            replaced[j] = 1
            bitmap[s] = 0
            continue
        gj = Gam[j, I]
        v = Gam[:, I] @ gj
        v[j] = gn2[j]
        a = Y[:, j] - D @ v + D[:, j] * gn2[j]
        an = np.linalg.norm(a)
        aD = a @ D
        Gam[j, I] = (a @ X[:, I] - aD @ Gam[:, I] + aD[j] * gj) / an
        D[:, j] = a / an
    return D, Gam, replaced, bitmap


def np_cleardict(X, D, Gam, replaced, err, mu=0.8, use_thresh=4):
    D = D.copy()
    err = err.copy()
    use = np.sum(Gam ** 2 > 1e-7, 1)
    out = []
    for j in range(D.shape[1]):
        g = D.T @ D[:, j]
        g[j] = 0
        if (np.max(g ** 2) > mu * mu or use[j] < use_thresh) and not replaced[j]:
            s = int(np.argmax(err))
            D[:, j] = X[:, s] / np.linalg.norm(X[:, s])
            err[s] = 0
            out.append((j, s))
    return D, err, out


def dense(idx, coef, nnz, K):
    N, T = idx.shape
    out = np.zeros((K, N))
    for t in range(T):
        m = t < nnz
        out[idx[m, t], np.nonzero(m)[0]] = coef[m, t]
    return out


def small_problem(seed=0, n=24, K=40, N=400, T=4, noise=0.05):
    rng = np.random.default_rng(seed)
    D0 = rng.standard_normal((n, K))
    D0 /= np.linalg.norm(D0, axis=0)
    Gm = np.zeros((K, N))
    for s in range(N):
        Gm[rng.choice(K, T, replace=False), s] = rng.standard_normal(T)
    X = D0 @ Gm + noise * rng.standard_normal((n, N))
    return np.asfortranarray(X), D0, Gm


# ---------------------------------------------------------------- golden fixtures

def test_reference_initial_dictionary_fixture(oracle_mod):
    """The reference's D.mat: 300 x 9, unnormalised, normcols gives unit columns."""
    D = np.load(os.path.join(GOLD, "ref_D_300x9.npy"))
    assert D.shape == (300, 9)
    nrm = np.linalg.norm(D, axis=0)
    assert np.all((nrm > 15) & (nrm < 19))
    Dn = oracle_mod.normcols(np.asfortranarray(D))
    np.testing.assert_allclose(np.linalg.norm(Dn, axis=0), 1.0, rtol=0, atol=1e-14)
    np.testing.assert_allclose(Dn, D / nrm, rtol=1e-14, atol=0)


def test_reference_gamma_structure(oracle_mod):
    """The reference's recorded CUDA_Gamma (K=9 x N=3600, T=6): every column holds exactly T
    nonzeros.  Running the oracle at the reference's own shape from the reference's own initial
    D gives the same structure (K x N layout, T distinct atoms per signal)."""
    z = np.load(os.path.join(GOLD, "ref_gamma_structure.npz"))
    for tag in ("a", "b"):
        K, N = z["shape_" + tag]
        assert (K, N) == (9, 3600)
        assert np.all(z["nnz_" + tag] == 6)
        sup = z["support_" + tag]
        assert np.all(np.diff(sup.astype(int), axis=1) > 0)      # distinct atoms per signal
    D = np.load(os.path.join(GOLD, "ref_D_300x9.npy"))
    from ksvd_gb300 import datagen

    p = datagen.make_problem("ref", dtype=np.float64)
    X = p["X"]
    perms = np.stack([np.random.default_rng(i).permutation(9) for i in range(3)]).astype(np.int32)
    Dn, idx, coef, nnz, rmse = oracle_mod.ksvd(X, np.asfortranarray(D), 6, 3, perms)
    g = oracle_mod.dense_gamma(idx, coef, nnz, 9)
    assert g.shape == (9, 3600)
    assert np.all((g != 0).sum(0) == 6)
    assert np.all(np.diff(rmse) <= 1e-12)                        # K-SVD never increases RMSE here


def test_oracle_small_regression(oracle_mod):
    """The oracle's FP64 output on a fixed tiny problem is stable across builds and platforms."""
    import importlib.util

    spec = importlib.util.spec_from_file_location("mg", os.path.join(GOLD, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    X, D, T, perms = mg.oracle_small_problem()
    Dn, idx, coef, nnz, rmse = oracle_mod.ksvd(X, D, T, perms.shape[0], perms)
    ref = np.load(os.path.join(GOLD, "oracle_small.npz"))
    assert support_match(idx, nnz, ref["idx"], ref["nnz"]) == 1.0
    np.testing.assert_allclose(rmse, ref["rmse"], rtol=1e-9)
    assert rel_rmse(Dn, ref["D"]) < 1e-9
    assert rel_rmse(coef, ref["coef"]) < 1e-9


# ---------------------------------------------------------------- known answers

def test_normcols_gram_dtx(oracle_mod):
    X, D0, _ = small_problem()
    D = np.asfortranarray(D0 * 3.0)
    Dn = oracle_mod.normcols(D)
    np.testing.assert_allclose(Dn, D0, atol=1e-14)
    np.testing.assert_allclose(oracle_mod.gram(Dn), Dn.T @ Dn, atol=1e-13)
    np.testing.assert_allclose(oracle_mod.dtx(Dn, X), Dn.T @ X, atol=1e-12)


def test_omp_orthonormal_exact(oracle_mod):
    """Orthonormal D: the support is recovered exactly and gamma = D'x; once x is explained the
    residual test stops early (nnz < T)."""
    rng = np.random.default_rng(1)
    Q, _ = np.linalg.qr(rng.standard_normal((16, 16)))
    N, T = 50, 5
    X = np.zeros((16, N))
    truth = []
    for s in range(N):
        S = rng.choice(16, 3, replace=False)
        g = rng.choice([-1, 1], 3) * (1 + rng.random(3))
        X[:, s] = Q[:, S] @ g
        truth.append(set(S.tolist()))
    G = oracle_mod.gram(np.asfortranarray(Q))
    A0 = oracle_mod.dtx(np.asfortranarray(Q), np.asfortranarray(X))
    idx, coef, nnz = oracle_mod.omp(G, A0, T)
    assert np.all(nnz == 3)
    for s in range(N):
        assert set(idx[s, :3].tolist()) == truth[s]
        np.testing.assert_allclose(coef[s, :3], (Q.T @ X[:, s])[idx[s, :3]], atol=1e-12)
        assert np.all(idx[s, 3:] == -1) and np.all(coef[s, 3:] == 0)


def test_omp_noiseless_recovery(oracle_mod):
    rng = np.random.default_rng(2)
    n, K, N, T = 128, 256, 300, 4
    D = rng.standard_normal((n, K))
    D /= np.linalg.norm(D, axis=0)
    X = np.zeros((n, N))
    truth = []
    for s in range(N):
        S = rng.choice(K, T, replace=False)
        X[:, s] = D[:, S] @ (rng.choice([-1, 1], T) * (0.5 + rng.random(T)))
        truth.append(set(S.tolist()))
    D = np.asfortranarray(D)
    idx, coef, nnz = oracle_mod.omp(oracle_mod.gram(D), oracle_mod.dtx(D, np.asfortranarray(X)), T)
    ok = np.mean([set(idx[s, : nnz[s]].tolist()) == truth[s] for s in range(N)])
    assert ok >= 0.99


def test_omp_one_atom_dictionary(oracle_mod):
    rng = np.random.default_rng(3)
    d = rng.standard_normal((10, 1))
    d /= np.linalg.norm(d)
    X = rng.standard_normal((10, 20))
    idx, coef, nnz = oracle_mod.omp(oracle_mod.gram(d), oracle_mod.dtx(d, X), 1)
    assert np.all(nnz == 1) and np.all(idx[:, 0] == 0)
    np.testing.assert_allclose(coef[:, 0], d[:, 0] @ X, atol=1e-13)


def test_omp_zero_signal_and_repeated_atom(oracle_mod):
    """A zero signal takes no atom; a dictionary with a repeated atom never uses both copies."""
    rng = np.random.default_rng(4)
    D = rng.standard_normal((12, 8))
    D /= np.linalg.norm(D, axis=0)
    D[:, 5] = D[:, 2]
    X = rng.standard_normal((12, 30))
    X[:, 0] = 0
    D = np.asfortranarray(D)
    idx, coef, nnz = oracle_mod.omp(oracle_mod.gram(D), oracle_mod.dtx(D, X), 6)
    assert nnz[0] == 0
    for s in range(1, 30):
        sup = idx[s, : nnz[s]].tolist()
        assert len(set(sup)) == len(sup)
        assert not (2 in sup and 5 in sup)


def test_omp_matches_numpy(oracle_mod):
    X, D0, _ = small_problem(seed=5)
    D = np.asfortranarray(D0)
    G, A0 = oracle_mod.gram(D), oracle_mod.dtx(D, X)
    idx, coef, nnz = oracle_mod.omp(G, A0, 6)
    for s in range(X.shape[1]):
        I, gam = np_omp(G, A0[:, s], 6)
        assert nnz[s] == len(I)
        assert idx[s, : nnz[s]].tolist() == I                     # same selection order
        np.testing.assert_allclose(coef[s, : nnz[s]], gam, rtol=1e-9, atol=1e-12)


def test_omp_error_target(oracle_mod):
    X, D0, _ = small_problem(seed=6, noise=0.01)
    D = np.asfortranarray(D0)
    G, A0 = oracle_mod.gram(D), oracle_mod.dtx(D, X)
    xn2 = np.sum(X * X, 0)
    eps2 = 0.05 * xn2
    idx, coef, nnz = oracle_mod.omp(G, A0, 20, xnorm2=xn2, eps2=eps2)
    for s in range(X.shape[1]):
        S = idx[s, : nnz[s]]
        r = X[:, s] - D[:, S] @ coef[s, : nnz[s]]
        assert r @ r <= eps2[s] * (1 + 1e-9) or nnz[s] == 20
        if nnz[s] > 0:   # one atom fewer would not have met the target
            S1 = S[:-1]
            g1 = np.linalg.lstsq(D[:, S1], X[:, s], rcond=None)[0] if len(S1) else np.zeros(0)
            r1 = X[:, s] - D[:, S1] @ g1
            assert r1 @ r1 > eps2[s] * (1 - 1e-9)


# ---------------------------------------------------------------- dictionary update

def test_update_matches_numpy(oracle_mod):
    X, D0, _ = small_problem(seed=7)
    rng = np.random.default_rng(7)
    D = np.asfortranarray(D0 + 0.1 * rng.standard_normal(D0.shape))
    D = oracle_mod.normcols(D)
    G, A0 = oracle_mod.gram(D), oracle_mod.dtx(D, X)
    idx, coef, nnz = oracle_mod.omp(G, A0, 4)
    perm = rng.permutation(D.shape[1]).astype(np.int32)
    D1, coef1, st = oracle_mod.update(X, D, idx, coef, nnz, perm)
    D2, Gam2, rep2, bm2 = np_update(X, D, dense(idx, coef, nnz, D.shape[1]), perm)
    np.testing.assert_allclose(D1, D2, rtol=1e-9, atol=1e-11)
    np.testing.assert_allclose(dense(idx, coef1, nnz, D.shape[1]), Gam2, rtol=1e-9, atol=1e-11)
    assert np.array_equal(st["replaced"], rep2) and np.array_equal(st["bitmap"], bm2)


def test_update_special_case_unused_atom(oracle_mod):
    """An atom no signal uses is replaced by the worst-represented candidate signal."""
    X, D0, _ = small_problem(seed=8, n=24, K=30, N=200, T=3)
    D = D0.copy()
    # atom 7: orthogonal to every signal, so OMP never selects it
    Q, _ = np.linalg.qr(np.concatenate([X, np.eye(24)], 1)[:, :25])
    D[:, 7] = 0
    X = X - np.outer(X.mean(1) * 0, np.ones(X.shape[1]))
    P = np.linalg.svd(X, full_matrices=True)[0]
    D[:, 7] = P[:, -1]                         # least-energy direction of the data
    X = X - np.outer(P[:, -1], P[:, -1] @ X)   # remove it from the data entirely
    D = oracle_mod.normcols(np.asfortranarray(D))
    X = np.asfortranarray(X)
    idx, coef, nnz = oracle_mod.omp(oracle_mod.gram(D), oracle_mod.dtx(D, X), 3)
    assert not np.any((idx == 7) & (np.arange(3)[None, :] < nnz[:, None]))
    perm = np.arange(30, dtype=np.int32)
    D1, coef1, st = oracle_mod.update(X, D, idx, coef, nnz, perm)
    D2, Gam2, rep2, bm2 = np_update(X, D, dense(idx, coef, nnz, 30), perm)
    assert st["replaced"][7] == 1 and st["counter"] == 1
    s = int(np.nonzero(st["bitmap"] == 0)[0][0])
    np.testing.assert_allclose(D1[:, 7], X[:, s] / np.linalg.norm(X[:, s]), atol=1e-12)
    np.testing.assert_allclose(D1, D2, rtol=1e-9, atol=1e-11)


def test_error_and_cleardict(oracle_mod):
    """errorComputation and clearDict: a coherent atom pair loses its first member to the
    worst-represented signal; the second member then survives."""
    X, D0, _ = small_problem(seed=9, n=24, K=30, N=300, T=3)
    rng = np.random.default_rng(9)
    D = D0.copy()
    D[:, 12] = D[:, 4] + 0.05 * rng.standard_normal(24)
    D = oracle_mod.normcols(np.asfortranarray(D))
    assert (D[:, 4] @ D[:, 12]) ** 2 > 0.64
    idx, coef, nnz = oracle_mod.omp(oracle_mod.gram(D), oracle_mod.dtx(D, X), 3)
    rmse, err = oracle_mod.error(X, D, idx, coef, nnz)
    r = X - D @ dense(idx, coef, nnz, 30)
    np.testing.assert_allclose(err, np.sum(r * r, 0), rtol=1e-12)
    assert abs(rmse - np.sqrt(np.sum(r * r) / r.size)) < 1e-14
    D1, err1, cleared = oracle_mod.cleardict(X, D, idx, coef, nnz, np.zeros(30, np.int32), err)
    D2, err2, repl = np_cleardict(X, D, dense(idx, coef, nnz, 30), np.zeros(30), err)
    s = int(np.argmax(err))
    assert repl[0] == (4, s)                   # the coherent pair's first member goes first
    np.testing.assert_allclose(D1[:, 4], X[:, s] / np.linalg.norm(X[:, s]), atol=1e-12)
    np.testing.assert_allclose(D1, D2, atol=1e-12)
    np.testing.assert_array_equal(err1, err2)
    assert cleared == len(repl) and err1[s] == 0


def test_ksvd_reduces_error(oracle_mod):
    from ksvd_gb300 import datagen

    p = datagen.make_problem("cfg0", N=3000, dtype=np.float64)
    perms = np.stack([np.random.default_rng(i).permutation(256) for i in range(4)]).astype(np.int32)
    Dn, idx, coef, nnz, rmse = oracle_mod.ksvd(p["X"], p["D"], 8, 4, perms)
    assert np.all(np.diff(rmse) < 0)
    np.testing.assert_allclose(np.linalg.norm(Dn, axis=0), 1.0, atol=1e-12)


def test_adjoint_formula_matches_finite_differences():
    """The FP64 adjoint of fixed-support coding (oracle/adjoint.py) against central differences
    (h=1e-3) of L = ||X - D Gamma||^2 + 1/2 ||W Gamma||^2, with ragged supports (0..T atoms)."""
    from oracle import adjoint as A

    rng = np.random.default_rng(11)
    n, K, N, T = 16, 40, 200, 5
    D = rng.standard_normal((n, K))
    D /= np.linalg.norm(D, axis=0)
    X = rng.standard_normal((n, N))
    nnz = rng.integers(0, T + 1, N).astype(np.int32)
    idx = np.full((N, T), -1, np.int32)
    for s in range(N):
        idx[s, : nnz[s]] = rng.choice(K, nnz[s], replace=False)
    W = rng.standard_normal((10, K))
    dD, dX, coef, _ = A.grad_w(D, X, idx, nnz, W)
    # coefficients: least squares on the support
    s = int(np.argmax(nnz))
    want = np.linalg.lstsq(D[:, idx[s, : nnz[s]]], X[:, s], rcond=None)[0]
    np.testing.assert_allclose(coef[s, : nnz[s]], want, rtol=1e-10, atol=1e-12)
    ent = [(int(rng.integers(n)), int(rng.integers(K))) for _ in range(60)]
    fd = A.fd_grad_D(D, X, idx, nnz, W, ent)
    an = np.array([dD[i, j] for i, j in ent])
    assert np.abs(fd - an).max() <= 1e-5 * np.abs(an).max()
    ent = [(int(rng.integers(n)), int(rng.integers(N))) for _ in range(60)]
    fd = A.fd_grad_X(D, X, idx, nnz, W, ent)
    an = np.array([dX[i, s] for i, s in ent])
    assert np.abs(fd - an).max() <= 1e-8 * np.abs(an).max()
