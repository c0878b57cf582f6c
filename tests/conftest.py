import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle

    oracle.build()
    oracle.load()
    return oracle


@pytest.fixture(scope="session")
def native_lib():
    """The product library (built from source if needed; nvcc cross-compiles without a GPU)."""
    from ksvd_gb300 import build, _native

    build.build()
    return _native.load()


@pytest.fixture(scope="session")
def cuda(native_lib):
    """GPU tests fail (they do not skip) when no CUDA device is visible."""
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test selected but torch.cuda.is_available() is False")
    torch.cuda.init()
    return torch.device("cuda", 0)


def rel_rmse(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.sqrt(np.mean((a - b) ** 2)) / max(np.sqrt(np.mean(b ** 2)), 1e-300))


def support_match(idx_a, nnz_a, idx_b, nnz_b):
    """Fraction of signals whose support SETS agree."""
    N = len(nnz_a)
    ok = 0
    for s in range(N):
        if nnz_a[s] != nnz_b[s]:
            continue
        if set(idx_a[s, : nnz_a[s]].tolist()) == set(idx_b[s, : nnz_b[s]].tolist()):
            ok += 1
    return ok / max(N, 1)


def support_match_vec(idx_a, nnz_a, idx_b, nnz_b):
    """Vectorised support-set agreement (sorted slots with -1 padding)."""
    T = idx_a.shape[1]
    ar = np.arange(T)[None, :]
    a = np.where(ar < nnz_a[:, None], idx_a, np.iinfo(np.int32).max)
    b = np.where(ar < nnz_b[:, None], idx_b, np.iinfo(np.int32).max)
    return float(np.mean(np.all(np.sort(a, 1) == np.sort(b, 1), 1) & (nnz_a == nnz_b)))


def coef_by_atom(idx, coef, nnz, K):
    """Dense (N, K) coefficient matrix from a sparse code (for value comparisons)."""
    N, T = idx.shape
    out = np.zeros((N, K), np.float64)
    for t in range(T):
        m = t < nnz
        out[np.nonzero(m)[0], idx[m, t]] = coef[m, t]
    return out


def touched_atoms(idx_a, nnz_a, idx_b, nnz_b, K):
    """(signals whose support sets differ, boolean mask of the atoms in either of their supports)."""
    T = idx_a.shape[1]
    ar = np.arange(T)[None, :]
    sa = np.sort(np.where(ar < nnz_a[:, None], idx_a, -1), 1)
    sb = np.sort(np.where(ar < nnz_b[:, None], idx_b, -1), 1)
    flipped = np.nonzero(np.any(sa != sb, 1) | (nnz_a != nnz_b))[0]
    touched = np.zeros(K, bool)
    for s in flipped:
        touched[sa[s][sa[s] >= 0]] = True
        touched[sb[s][sb[s] >= 0]] = True
    return flipped, touched
