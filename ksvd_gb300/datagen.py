"""Seeded synthetic K-SVD workloads.

The reference's only workload is fMRI data (Matlab/fmriKSVD.m:9, ``300_3600.mat``) that is not
published; these generators stand in for it with the shapes and value distributions of the
named configurations:

* ``cfg0``  n=64,  K=256,  N=10,000,    T=8,  10 iterations, 20 dB (CPU-runnable case)
* ``cfg1``  n=200, K=512,  N=200,000,   T=10, 20 iterations, 10 dB, AR(1) rho=0.9 atoms,
  row means removed (Matlab/remmean.m:13-15)
* ``cfg2``  n=256, K=1024, N=1,000,000, T=16, 10 iterations, 25 dB (the headline workload)
* ``cfg3``  64 independent problems, n uniform in {32, 64, 128, 256}, K = 4n, N uniform in
  10k..200k each, error-constrained coding (``make_batched``)
* ``cfg4``  n=128, K=512,  N=100,000,   T=12 (fixed-support coding adjoint)
* ``ref``   n=300, K=9,    N=3,600,     T=6,  30 iterations (the reference's own shape)

Generation (per signal): T distinct atom indices uniform without replacement, coefficients
N(0,1), additive white Gaussian noise with sigma_s = ||D0 gamma_s|| / sqrt(n) * 10^(-SNR/20).
Ground-truth atoms are unit-norm N(0,1) columns (or unit-norm AR(1) random walks for cfg1).
The initial dictionary is K distinct random signals, normalised.

Two backends with the same distributions: numpy (``device='cpu'``, small and medium sizes,
platform-independent PCG64 stream) and torch (``device='cuda'``, the full-size bench inputs,
generated on the GPU in chunks).
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

SEED_BASE = 0x4B535644  # "KSVD"


@dataclasses.dataclass(frozen=True)
class Config:
    name: str
    n: int
    K: int
    N: int
    T: int
    iters: int
    snr_db: float
    atoms: str = "gauss"          # "gauss" | "ar1"
    rho: float = 0.9
    remove_row_mean: bool = False
    index: int = 0


CONFIGS = {
    "cfg0": Config("cfg0", 64, 256, 10_000, 8, 10, 20.0, index=0),
    "cfg1": Config("cfg1", 200, 512, 200_000, 10, 20, 10.0, atoms="ar1", remove_row_mean=True,
                   index=1),
    "cfg2": Config("cfg2", 256, 1024, 1_000_000, 16, 10, 25.0, index=2),
    "cfg4": Config("cfg4", 128, 512, 100_000, 12, 1, 20.0, index=4),
    "ref": Config("ref", 300, 9, 3600, 6, 30, 20.0, index=5),
}


def _unit_columns(A):
    return A / np.linalg.norm(A, axis=0, keepdims=True)


def ground_truth_dictionary(cfg: Config, rng: np.random.Generator) -> np.ndarray:
    if cfg.atoms == "ar1":
        e = rng.standard_normal((cfg.n, cfg.K))
        A = np.empty_like(e)
        A[0] = e[0]
        for r in range(1, cfg.n):
            A[r] = cfg.rho * A[r - 1] + e[r]
        return _unit_columns(A)
    return _unit_columns(rng.standard_normal((cfg.n, cfg.K)))


def _supports(rng, N, K, T, chunk=65536):
    out = np.empty((N, T), dtype=np.int64)
    for s0 in range(0, N, chunk):
        s1 = min(N, s0 + chunk)
        keys = rng.random((s1 - s0, K))
        out[s0:s1] = np.argpartition(keys, T - 1, axis=1)[:, :T]
    return out


def make_problem(cfg, N=None, seed=None, dtype=np.float32, device="cpu", dict_from="signals"):
    """Returns dict(X=(n,N) col-major, D=(n,K) initial dictionary, D0, support, gamma).

    ``dict_from="signals"`` takes the initial dictionary from K distinct signals of X (the
    MATLAB toolbox convention the reference's harness follows); ``"extra"`` draws K further
    signals from the same distribution that are not part of X, so that no signal starts out
    identical to an atom (used by the parity tests: such a signal's residual is rounding noise
    after its first atom, and an absolute stop threshold then depends on the arithmetic).

    With ``device='cuda'`` X and D are torch CUDA tensors shaped (N, n) and (K, n) row-major,
    i.e. the same column-major memory as the numpy (n, N) / (n, K) arrays."""
    if isinstance(cfg, str):
        cfg = CONFIGS[cfg]
    N = cfg.N if N is None else int(N)
    seed = SEED_BASE + cfg.index if seed is None else int(seed)
    if device != "cpu":
        return _make_problem_torch(cfg, N, seed, device)
    rng = np.random.default_rng(seed)
    D0 = ground_truth_dictionary(cfg, rng)
    Nx = N
    if dict_from == "extra":
        N = N + cfg.K
    sup = _supports(rng, N, cfg.K, cfg.T)
    gam = rng.standard_normal((N, cfg.T))
    X = np.empty((cfg.n, N), dtype=np.float64, order="F")
    chunk = 65536
    for s0 in range(0, N, chunk):
        s1 = min(N, s0 + chunk)
        clean = np.einsum("rst,st->rs", D0[:, sup[s0:s1]], gam[s0:s1])
        sig = np.linalg.norm(clean, axis=0) / math.sqrt(cfg.n) * 10 ** (-cfg.snr_db / 20)
        X[:, s0:s1] = clean + rng.standard_normal(clean.shape) * sig
    if cfg.remove_row_mean:
        X -= X.mean(axis=1, keepdims=True)
    if dict_from == "extra":
        D = _unit_columns(X[:, Nx:])
        X, sup, gam = X[:, :Nx], sup[:Nx], gam[:Nx]
    else:
        pick = rng.choice(N, size=cfg.K, replace=False)
        D = _unit_columns(X[:, pick])
    return dict(X=np.asfortranarray(X.astype(dtype)), D=np.asfortranarray(D.astype(dtype)),
                D0=D0, support=sup, gamma=gam, cfg=cfg)


def _make_problem_torch(cfg, N, seed, device):
    import torch

    g = torch.Generator(device=device)
    g.manual_seed(seed)
    rng = np.random.default_rng(seed)
    D0 = torch.from_numpy(ground_truth_dictionary(cfg, rng).T.astype(np.float32)).to(device)
    X = torch.empty((N, cfg.n), dtype=torch.float32, device=device)
    chunk = 1 << 17
    for s0 in range(0, N, chunk):
        s1 = min(N, s0 + chunk)
        m = s1 - s0
        keys = torch.rand((m, cfg.K), generator=g, device=device)
        sup = keys.topk(cfg.T, dim=1).indices                       # (m, T) distinct
        gam = torch.randn((m, cfg.T), generator=g, device=device)
        clean = torch.einsum("mtr,mt->mr", D0[sup], gam)              # (m, n)
        sig = clean.norm(dim=1, keepdim=True) / math.sqrt(cfg.n) * 10 ** (-cfg.snr_db / 20)
        X[s0:s1] = clean + torch.randn((m, cfg.n), generator=g, device=device) * sig
        del keys, sup, gam, clean
    if cfg.remove_row_mean:
        X -= X.mean(dim=0, keepdim=True)
    pick = torch.randperm(N, generator=g, device=device)[: cfg.K]
    D = X[pick].clone()
    D /= D.norm(dim=1, keepdim=True)
    return dict(X=X, D=D, cfg=cfg)


def make_batched(nprob=64, seed=SEED_BASE + 3, device="cuda", n_choices=(32, 64, 128, 256),
                 n_range=(10_000, 200_000), scale=1.0):
    """The batched workload: ``nprob`` independent problems with n uniform in ``n_choices``,
    K = 4n, N uniform in ``n_range`` (times ``scale``).  Each signal is a sparse combination of
    T_s ~ U[1, min(48, n/2)] unit-norm N(0,1) atoms with N(0,1) coefficients plus white noise at
    an SNR uniform in [15, 30] dB; its error target is eps^2 = 1.05 * n * sigma_s^2 (the
    expected noise energy), so the coded supports spread over 1..64 atoms.  The coefficient
    slots per signal are T = min(64, n).  The initial dictionary is K distinct signals,
    normalised.  Returns a list of dicts (D (K, n), X (N, n), eps2 (N,), T) of device tensors."""
    import torch

    rng = np.random.default_rng(seed)
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    out = []
    for _ in range(nprob):
        n = int(rng.choice(n_choices))
        K = 4 * n
        N_full = int(rng.integers(n_range[0], n_range[1] + 1))
        N = max(K, int(N_full * scale))
        tmax = min(48, n // 2)
        D0 = torch.from_numpy(_unit_columns(rng.standard_normal((n, K))).T.astype(np.float32))
        D0 = D0.to(device)
        X = torch.empty((N, n), dtype=torch.float32, device=device)
        eps2 = torch.empty((N,), dtype=torch.float32, device=device)
        chunk = 1 << 14
        for s0 in range(0, N, chunk):
            m = min(N, s0 + chunk) - s0
            t = torch.randint(1, tmax + 1, (m, 1), generator=g, device=device)
            keys = torch.rand((m, K), generator=g, device=device)
            top = keys.topk(tmax, dim=1).indices                      # (m, tmax) distinct
            live = torch.arange(tmax, device=device)[None, :] < t
            gam = torch.randn((m, tmax), generator=g, device=device) * live
            clean = torch.einsum("mtr,mt->mr", D0[top], gam)
            snr = 15 + 15 * torch.rand((m, 1), generator=g, device=device)
            sig = clean.norm(dim=1, keepdim=True) / math.sqrt(n) * 10 ** (-snr / 20)
            X[s0:s0 + m] = clean + torch.randn((m, n), generator=g, device=device) * sig
            eps2[s0:s0 + m] = (1.05 * n * sig * sig)[:, 0]
        pick = torch.randperm(N, generator=g, device=device)[:K]
        D = X[pick].clone()
        D /= D.norm(dim=1, keepdim=True)
        out.append(dict(D=D, X=X, eps2=eps2, T=min(64, n), n=n, K=K, N=N, N_full=N_full))
    return out
