"""Counter-based RNG and cross-entropy-method refit in FP64 (test infrastructure).

The reference has no CEM: its searches are Optuna TPE (scripts/mass_opt.py:216),
a grid (scripts/mass_landscape.py:153) and Optuna CMA-ES
(spigym/config/algo/active_sysid.yaml:20). This module restates the engine's
CEM so its device implementation can be checked.

RNG: Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
easy as 1, 2, 3", SC'11): 10 rounds of the 4x32 Philox S-box with multipliers
0xD2511F53 / 0xCD9E8D57 and Weyl key increments 0x9E3779B9 / 0xBB67AE85.
Uniforms u = (w + 0.5) * 2^-32 (open interval); normals by Box-Muller on word
pairs. Counter = (sample, iteration, block, job), key = (seed_lo, seed_hi).
"""
from __future__ import annotations

import numpy as np

M0, M1 = 0xD2511F53, 0xCD9E8D57
W0, W1 = 0x9E3779B9, 0xBB67AE85
MASK = 0xFFFFFFFF


def philox4x32_10(ctr, key):
    """ctr [..., 4], key [..., 2] (uint32-valued) -> [..., 4] uint32."""
    c = [np.asarray(ctr, dtype=np.uint64)[..., i] & MASK for i in range(4)]
    k0 = np.asarray(key, dtype=np.uint64)[..., 0] & MASK
    k1 = np.asarray(key, dtype=np.uint64)[..., 1] & MASK
    for r in range(10):
        if r:
            k0 = (k0 + W0) & MASK
            k1 = (k1 + W1) & MASK
        p0 = np.uint64(M0) * c[0]
        p1 = np.uint64(M1) * c[2]
        hi0, lo0 = p0 >> np.uint64(32), p0 & MASK
        hi1, lo1 = p1 >> np.uint64(32), p1 & MASK
        c = [hi1 ^ c[1] ^ k0, lo1, hi0 ^ c[3] ^ k1, lo0]
    return np.stack(c, -1).astype(np.uint32)


def _key(seed):
    seed = int(seed) & 0xFFFFFFFFFFFFFFFF
    return np.array([seed & MASK, seed >> 32], dtype=np.uint64)


def _words(seed, job, it, n_samples, n_dims):
    """[N, ceil(P/4)*4] Philox words for samples 0..N-1 of (job, iteration)."""
    nb = (n_dims + 3) // 4
    n = np.arange(n_samples, dtype=np.uint64)
    ctr = np.zeros((n_samples, nb, 4), dtype=np.uint64)
    ctr[..., 0] = n[:, None]
    ctr[..., 1] = it
    ctr[..., 2] = np.arange(nb, dtype=np.uint64)[None, :]
    ctr[..., 3] = job
    key = np.broadcast_to(_key(seed), (n_samples, nb, 2))
    return philox4x32_10(ctr, key).reshape(n_samples, nb * 4)


def uniforms(seed, job, it, n_samples, n_dims):
    w = _words(seed, job, it, n_samples, n_dims)[:, :n_dims]
    return (w.astype(np.float64) + 0.5) * 2.0 ** -32


def normals(seed, job, it, n_samples, n_dims):
    w = _words(seed, job, it, n_samples, n_dims)
    u = (w.astype(np.float64) + 0.5) * 2.0 ** -32
    u1, u2 = u[:, 0::2], u[:, 1::2]
    r = np.sqrt(-2.0 * np.log(u1))
    z = np.empty_like(u)
    z[:, 0::2] = r * np.cos(2.0 * np.pi * u2)
    z[:, 1::2] = r * np.sin(2.0 * np.pi * u2)
    return z[:, :n_dims]


def n_elite(n_samples, elite_frac=0.1):
    return max(2, int(np.floor(elite_frac * n_samples + 0.5)))


def elite_order(cost):
    """Indices sorted by (cost ascending, index ascending); NaN sorts after +inf."""
    c = np.asarray(cost, dtype=np.float64)
    nan = np.isnan(c)
    return np.lexsort((np.arange(c.shape[0]), np.where(nan, np.inf, c), nan))


def refit(theta, cost, ne, mu_prev, cov_prev, alpha, min_std):
    """Elite mean / covariance with smoothing alpha and a per-dimension std floor."""
    th = np.asarray(theta, dtype=np.float64)
    e = th[elite_order(cost)[:ne]]
    mu = e.mean(0)
    d = e - mu
    cov = d.T @ d / ne
    mu = alpha * mu + (1.0 - alpha) * mu_prev
    cov = alpha * cov + (1.0 - alpha) * cov_prev
    cov = cov + np.diag(np.asarray(min_std, dtype=np.float64) ** 2)
    return mu, cov


def sample(mu, cov, lo, hi, seed, job, it, n_samples):
    L = np.linalg.cholesky(cov)
    z = normals(seed, job, it, n_samples, mu.shape[0])
    return np.clip(mu + z @ L.T, lo, hi)


def init_samples(lo, hi, seed, job, n_samples):
    u = uniforms(seed, job, 0, n_samples, len(lo))
    return lo + (hi - lo) * u


def prior_moments(lo, hi):
    lo, hi = np.asarray(lo, np.float64), np.asarray(hi, np.float64)
    return 0.5 * (lo + hi), np.diag((hi - lo) ** 2 / 12.0)
