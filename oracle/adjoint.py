"""FP64 numpy reference for fixed-support coding and its adjoint -- TEST INFRASTRUCTURE ONLY.

The reference (patschris/KSVD) has no differentiable path; this restates the mathematics the
library's ``ksvd_code_fixed`` / ``ksvd_code_backward`` implement, so the tests can check the CUDA
kernels against an independent FP64 gradient and both against central finite differences.

Per signal s with support S (``idx[s, :nnz[s]]``), A = D[:, S]:
    gamma_S = (A'A)^-1 A'x                             (least squares on the support)
Given g = dL/dgamma_S, with u = (A'A)^-1 g and r = x - A gamma_S:
    dL/dx        = A u
    dL/dD[:, S]  = r u' - (A u) gamma_S'
The test loss of the adjoint workload (n=128, K=512, N=100,000, T=12):
    L(D, X) = ||X - D Gamma||_F^2 + 1/2 ||W Gamma||_F^2,  W a seeded 10 x K Gaussian matrix,
with Gamma = code(D, X) on fixed supports.

Layouts follow the reference: D is n x K, X is n x N (numpy arrays in any order), idx/coef are
N x T with -1 / 0 padding, nnz has N entries.
"""
from __future__ import annotations

import numpy as np

__all__ = ["code_fixed", "code_backward", "loss_w", "grad_w", "loss_w_signals", "fd_grad_D",
           "fd_grad_X"]


def _groups(nnz, chunk=8192):
    """(t, signal indices) pairs: signals grouped by support size, in chunks (batched solves)."""
    out = []
    for t in np.unique(nnz):
        if t > 0:
            rows = np.nonzero(nnz == t)[0]
            for c in range(0, len(rows), chunk):
                out.append((int(t), rows[c:c + chunk]))
    return out


def code_fixed(D, X, idx, nnz, cols=None):
    """gamma (N x T, FP64) for the signals ``cols`` (all when None) on their fixed supports."""
    D = np.asarray(D, np.float64)
    X = np.asarray(X, np.float64)
    T = idx.shape[1]
    sel = np.arange(X.shape[1]) if cols is None else np.asarray(cols)
    coef = np.zeros((len(sel), T))
    nz = nnz[sel]
    for t, rows in _groups(nz):
        s = sel[rows]
        A = D[:, idx[s, :t]].transpose(1, 0, 2)            # (m, n, t)
        M = np.einsum("mni,mnj->mij", A, A)
        b = np.einsum("mni,nm->mi", A, X[:, s])
        coef[rows, :t] = np.linalg.solve(M, b[..., None])[..., 0]
    return coef


def code_backward(D, X, idx, nnz, coef, dcoef):
    """(dD, dX) in FP64 through the fixed-support coding step, given dL/dgamma."""
    D = np.asarray(D, np.float64)
    X = np.asarray(X, np.float64)
    n, K = D.shape
    dD = np.zeros((n, K))
    dX = np.zeros_like(X)
    for t, s in _groups(nnz):
        S = idx[s, :t]
        A = D[:, S].transpose(1, 0, 2)                      # (m, n, t)
        M = np.einsum("mni,mnj->mij", A, A)
        u = np.linalg.solve(M, np.asarray(dcoef, np.float64)[s, :t, None])[..., 0]
        g = np.asarray(coef, np.float64)[s, :t]
        r = X[:, s].T - np.einsum("mni,mi->mn", A, g)       # (m, n)
        Au = np.einsum("mni,mi->mn", A, u)
        dX[:, s] = Au.T
        contrib = np.einsum("mn,mi->min", r, u) - np.einsum("mn,mi->min", Au, g)  # (m, t, n)
        np.add.at(dD.T, S.reshape(-1), contrib.reshape(-1, n))
    return dD, dX


def loss_w_signals(D, X, idx, nnz, W, cols):
    """The loss restricted to the signals ``cols`` (the other signals' terms do not move)."""
    D = np.asarray(D, np.float64)
    X = np.asarray(X, np.float64)
    cols = np.asarray(cols)
    coef = code_fixed(D, X, idx, nnz, cols)
    total = float(np.sum(X[:, cols] ** 2 * (nnz[cols] == 0)[None, :]))
    for t, rows in _groups(nnz[cols]):
        s = cols[rows]
        S = idx[s, :t]
        g = coef[rows, :t]
        r = X[:, s].T - np.einsum("mni,mi->mn", D[:, S].transpose(1, 0, 2), g)
        wg = np.einsum("kmi,mi->mk", W[:, S], g)
        total += float(np.sum(r * r) + 0.5 * np.sum(wg * wg))
    return total


def loss_w(D, X, idx, nnz, W):
    return loss_w_signals(D, X, idx, nnz, W, np.arange(np.asarray(X).shape[1]))


def dcoef_w(D, X, idx, nnz, coef, W):
    """dL/dgamma_S for L = ||X - D Gamma||^2 + 1/2 ||W Gamma||^2 (FP64)."""
    D = np.asarray(D, np.float64)
    X = np.asarray(X, np.float64)
    T = idx.shape[1]
    out = np.zeros((X.shape[1], T))
    WtW = W.T @ W
    for t, s in _groups(nnz):
        S = idx[s, :t]
        A = D[:, S].transpose(1, 0, 2)
        g = np.asarray(coef, np.float64)[s, :t]
        r = X[:, s].T - np.einsum("mni,mi->mn", A, g)
        out[s, :t] = -2.0 * np.einsum("mni,mn->mi", A, r) + np.einsum(
            "mij,mj->mi", WtW[S[:, :, None], S[:, None, :]], g)
    return out


def grad_w(D, X, idx, nnz, W):
    """Analytic (dL/dD, dL/dX) in FP64: the direct terms plus the adjoint of the coding step."""
    D = np.asarray(D, np.float64)
    X = np.asarray(X, np.float64)
    coef = code_fixed(D, X, idx, nnz)
    dc = dcoef_w(D, X, idx, nnz, coef, W)
    dD, dX = code_backward(D, X, idx, nnz, coef, dc)
    R = X.copy()
    for t, s in _groups(nnz):
        S = idx[s, :t]
        R[:, s] -= np.einsum("mni,mi->nm", D[:, S].transpose(1, 0, 2), coef[s, :t])
    # direct terms of ||X - D Gamma||^2 with Gamma held fixed
    for t, s in _groups(nnz):
        S = idx[s, :t]
        contrib = -2.0 * np.einsum("nm,mi->min", R[:, s], coef[s, :t])
        np.add.at(dD.T, S.reshape(-1), contrib.reshape(-1, D.shape[0]))
    dX += 2.0 * R
    return dD, dX, coef, dc


def _users(idx, nnz, j):
    T = idx.shape[1]
    live = np.arange(T)[None, :] < nnz[:, None]
    return np.nonzero(((idx == j) & live).any(axis=1))[0]


def fd_grad_D(D, X, idx, nnz, W, entries, h=1e-3):
    """Central differences of the loss in FP64 at the (row, atom) entries of D."""
    D = np.array(D, np.float64)
    out = np.empty(len(entries))
    for e, (i, j) in enumerate(entries):
        cols = _users(idx, nnz, j)
        if len(cols) == 0:
            out[e] = 0.0
            continue
        old = D[i, j]
        D[i, j] = old + h
        lp = loss_w_signals(D, X, idx, nnz, W, cols)
        D[i, j] = old - h
        lm = loss_w_signals(D, X, idx, nnz, W, cols)
        D[i, j] = old
        out[e] = (lp - lm) / (2 * h)
    return out


def fd_grad_X(D, X, idx, nnz, W, entries, h=1e-3):
    """Central differences of the loss in FP64 at the (row, signal) entries of X."""
    X = np.array(X, np.float64)
    out = np.empty(len(entries))
    for e, (i, s) in enumerate(entries):
        old = X[i, s]
        X[i, s] = old + h
        lp = loss_w_signals(D, X, idx, nnz, W, [s])
        X[i, s] = old - h
        lm = loss_w_signals(D, X, idx, nnz, W, [s])
        X[i, s] = old
        out[e] = (lp - lm) / (2 * h)
    return out
