"""The oracle pinned to the reference's own arithmetic (CPU only).

oracle/ref_build.py compiles the reference's parOMP (K-SVD/K-SVD/OMP.cu:126-404) and its
per-atom update kernels (K-SVD/K-SVD/Multiplication.cu:177-224) unchanged for the host; these
tests run them beside the oracle on the same seeded FP64 inputs.  The reference's kernels need
K <= 32 (parOMP's alpha[32]) and a compile-time T, so the cases are small.  Required: identical
supports in identical selection order and coefficients / atoms equal to 1e-12 relative (the two
differ only in the order of floating-point sums).  The tests skip where no reference checkout is
available to build from (the compiled library is not committed)."""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def ref():
    from oracle import reference

    if not reference.available():
        pytest.skip("no reference checkout to compile the reference kernels from")
    return reference


def _unit(D):
    return D / np.linalg.norm(D, axis=0)


def _signals(rng, D, N, T, snr_db=None, scale=1.0):
    n, K = D.shape
    X = np.zeros((n, N))
    for s in range(N):
        S = rng.choice(K, T, replace=False)
        X[:, s] = D[:, S] @ rng.standard_normal(T)
    if snr_db is not None:
        sig = np.linalg.norm(X, axis=0) / np.sqrt(n) * 10 ** (-snr_db / 20)
        X += rng.standard_normal((n, N)) * sig
    return X * scale


def _compare_omp(oracle_mod, ref, D, X, T):
    G = D.T @ D
    A0 = D.T @ X
    ri, rc, rn, _ = ref.paromp(G, A0, T)
    oi, oc, on = oracle_mod.omp(np.asfortranarray(G), np.asfortranarray(A0), T)
    assert np.array_equal(rn, on), np.nonzero(rn != on)[0][:10]
    assert np.array_equal(ri, oi), np.nonzero(np.any(ri != oi, 1))[0][:10]
    scale = np.maximum(np.abs(rc), 1e-300)
    used = np.arange(T)[None, :] < on[:, None]
    rel = np.abs(rc - oc)[used] / scale[used]
    assert rel.max(initial=0.0) <= 1e-12, rel.max()
    return on


def test_paromp_reference_shape(oracle_mod, ref):
    """The reference's own workload shape: its recorded 300 x 9 initial dictionary (input/D.mat),
    normalised as KSVD.cu:57 does, T = 6 (ProgramParameters.cuh:20), 3,600 signals."""
    rng = np.random.default_rng(11)
    D = oracle_mod.normcols(np.load(os.path.join(GOLD, "ref_D_300x9.npy")).astype(np.float64))
    X = _signals(rng, D, 3600, 6, snr_db=20)
    nnz = _compare_omp(oracle_mod, ref, D, X, 6)
    assert np.all(nnz == 6)


@pytest.mark.parametrize("n,K,T,snr", [(16, 8, 1, 20), (16, 8, 3, None), (64, 16, 5, 30),
                                       (64, 32, 8, 20), (32, 32, 12, 10), (128, 32, 10, None),
                                       (20, 24, 7, 15)])
def test_paromp_random(oracle_mod, ref, n, K, T, snr):
    rng = np.random.default_rng(1000 + n + K + T)
    D = _unit(rng.standard_normal((n, K)))
    X = _signals(rng, D, 400, min(T, K), snr_db=snr)
    _compare_omp(oracle_mod, ref, D, X, T)


def test_paromp_early_stops(oracle_mod, ref):
    """Signals that stop early: exact atoms (the residual vanishes after one atom: alpha_p^2 <
    1e-14, OMP.cu:304), zero signals (stop at once), and sparse signals with T above their true
    support (noiseless: the residual vanishes after the true atoms)."""
    rng = np.random.default_rng(5)
    D = _unit(rng.standard_normal((48, 24)))
    X = np.concatenate([D[:, :6] * 3.0, np.zeros((48, 3)), _signals(rng, D, 40, 3)], 1)
    nnz = _compare_omp(oracle_mod, ref, D, X, 8)
    assert np.all(nnz[:6] == 1) and np.all(nnz[6:9] == 0) and np.all(nnz[9:] <= 8)


def test_paromp_scaled_signals(oracle_mod, ref):
    rng = np.random.default_rng(9)
    D = _unit(rng.standard_normal((64, 32)))
    for scale in (1e4, 1e-4):
        X = _signals(rng, D, 200, 5, snr_db=25, scale=scale)
        _compare_omp(oracle_mod, ref, D, X, 6)


def test_atom_update_kernels_match_oracle_sweep(oracle_mod, ref):
    """The first atom of an oracle sweep (DictionaryUpdate.cu:99-197) against the reference's
    per-atom kernels: a = Y_j - D v + d_j ||gamma_j||^2 (device_A_times_x_modified,
    Multiplication.cu:177-193), then the new coefficients (a'x_s - Gamma_s'(a'D) + (a'd_j)
    gamma_j(s)) / ||a|| and the new atom a / ||a|| (device_normal_x_times_A_modified,
    Multiplication.cu:198-224).  The kernels' inputs (Y_j, v, a'D, a'x_s, ||a||) are formed in
    numpy as the reference's reduction kernels define them."""
    rng = np.random.default_rng(21)
    n, K, N, T = 24, 16, 300, 4
    D = _unit(rng.standard_normal((n, K)))
    X = _signals(rng, D, N, T, snr_db=20)
    G, A0 = D.T @ D, D.T @ X
    idx, coef, nnz = oracle_mod.omp(np.asfortranarray(G), np.asfortranarray(A0), T)
    Gam = oracle_mod.dense_gamma(idx, coef, nnz, K)
    for j in (0, 5, 11):
        I = np.nonzero(Gam[j])[0]
        assert len(I) > 0
        perm = np.array([j] + [k for k in range(K) if k != j], np.int32)
        D1, coef1, _ = oracle_mod.update(np.asfortranarray(X), np.asfortranarray(D), idx, coef,
                                         nnz, perm)
        gam_j = Gam[j, I]
        gn2 = float(gam_j @ gam_j)
        Y_j = X[:, I] @ gam_j
        v = Gam[:, I] @ gam_j
        v[j] = gn2
        a = ref.a_times_x(D, v, Y_j, D[:, j], gn2, len(I))
        anorm = float(np.sqrt(a @ a))
        aD = D.T @ a
        rowlin = a @ X[:, I]
        Gnew, dnew = ref.normal_x_times_a(aD, Gam, I, gam_j, rowlin, aD[j], anorm, j, a)
        # oracle: new atom j and the new coefficients of atom j's entries
        np.testing.assert_allclose(D1[:, j], dnew, rtol=1e-12, atol=1e-14)
        Gam1 = oracle_mod.dense_gamma(idx, coef1, nnz, K)
        np.testing.assert_allclose(Gam1[j, I], Gnew[j, I], rtol=1e-12, atol=1e-14)
