"""Regenerate the golden fixtures in this folder.

Inputs (read only here, where the reference checkout exists):
  K-SVD/K-SVD/input/D.mat            D (300 x 9, FP64): the reference's initial dictionary
  K-SVD/K-SVD/output/temp.mat         CUDA_Gamma (9 x 3600, FP64): a recorded final Gamma
  K-SVD/x64/Release/output/temp.mat   CUDA_Gamma (9 x 3600, FP64): a second recorded run
The X.mat that produced the recorded Gamma is not in the reference (.MISSING_LARGE_BLOBS), so
only D and the *structure* of Gamma are kept: the support (row indices of the nonzeros) of every
column, in ascending atom order, and the nonzero count per column.

Also writes ``oracle_small.npz``: the oracle's FP64 outputs on one fixed tiny problem, so a
change of the oracle (or a platform difference) is caught by tests/test_oracle.py.

Usage: python tests/golden/make_golden.py [REFERENCE_ROOT]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def main(ref_root):
    import scipy.io as sio

    D = sio.loadmat(os.path.join(ref_root, "K-SVD/K-SVD/input/D.mat"))["D"]
    np.save(os.path.join(HERE, "ref_D_300x9.npy"), np.asarray(D, np.float64))
    sups = {}
    for tag, rel in (("a", "K-SVD/K-SVD/output/temp.mat"),
                     ("b", "K-SVD/x64/Release/output/temp.mat")):
        g = sio.loadmat(os.path.join(ref_root, rel))["CUDA_Gamma"]
        K, N = g.shape
        nz = (g != 0)
        counts = nz.sum(0).astype(np.int16)
        T = int(counts.max())
        sup = np.full((N, T), 255, np.uint8)
        for s in range(N):
            r = np.nonzero(nz[:, s])[0]
            sup[s, : len(r)] = r
        sups["support_" + tag] = sup
        sups["nnz_" + tag] = counts
        sups["shape_" + tag] = np.array([K, N])
    np.savez_compressed(os.path.join(HERE, "ref_gamma_structure.npz"), **sups)
    make_oracle_small()


def oracle_small_problem():
    rng = np.random.default_rng(20241203)
    n, K, N, T = 16, 24, 300, 4
    D0 = rng.standard_normal((n, K))
    D0 /= np.linalg.norm(D0, axis=0)
    G = np.zeros((K, N))
    for s in range(N):
        G[rng.choice(K, T, replace=False), s] = rng.standard_normal(T)
    X = D0 @ G + 0.05 * rng.standard_normal((n, N))
    Dinit = X[:, rng.choice(N, K, replace=False)]
    perms = np.stack([rng.permutation(K) for _ in range(3)]).astype(np.int32)
    return np.asfortranarray(X), np.asfortranarray(Dinit), T, perms


def make_oracle_small():
    sys.path.insert(0, ROOT)
    import oracle

    X, D, T, perms = oracle_small_problem()
    Dn, idx, coef, nnz, rmse = oracle.ksvd(X, D, T, perms.shape[0], perms)
    np.savez_compressed(os.path.join(HERE, "oracle_small.npz"), D=Dn, idx=idx, coef=coef,
                        nnz=nnz, rmse=rmse)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py REFERENCE_CHECKOUT")
    main(sys.argv[1])
