"""Candidate-command parametrisations (test infrastructure).

Restates spigym/agents/sysid/active_sysid.py:259-400. ``values`` is the flat
list of numbers an Optuna trial would return, in the order the reference asks
for them (constant: dim-major then update; polynomial: update, dim,
coefficient; bezier: update, dim, control point).
"""
from __future__ import annotations

from math import comb

import numpy as np


def constant(values, n_updates, n_dims, steps):
    v = np.asarray(values, dtype=np.float64).reshape(n_dims, n_updates).T
    return np.repeat(v, steps, axis=0)


def polynomial(values, ranges, idxs, n_updates, steps, degree):
    n_dims = len(idxs)
    c = np.asarray(values, dtype=np.float64).reshape(n_updates, n_dims, degree + 1)
    t = np.linspace(0.0, 1.0, steps)
    powers = t[None, :] ** np.arange(degree + 1)[:, None]
    poly = np.tanh(np.einsum("udk,ks->usd", c, powers))
    lo = np.asarray([ranges[i][0] for i in idxs])
    hi = np.asarray([ranges[i][1] for i in idxs])
    return (lo + (poly + 1.0) * 0.5 * (hi - lo)).reshape(n_updates * steps, n_dims)


def bezier(values, ranges, idxs, n_updates, steps, n_points):
    n_dims = len(idxs)
    cp = np.asarray(values, dtype=np.float64).reshape(n_updates, n_dims, n_points)
    t = np.linspace(0.0, 1.0, steps)
    n = n_points - 1
    basis = np.stack([comb(n, j) * t ** j * (1 - t) ** (n - j) for j in range(n_points)], 0)
    seg = np.einsum("udj,js->usd", cp, basis)
    lo = np.asarray([ranges[i][0] for i in idxs])
    hi = np.asarray([ranges[i][1] for i in idxs])
    return np.clip(seg, lo, hi).reshape(n_updates * steps, n_dims)


def expand(sampled, default_command, idxs):
    full = np.tile(np.asarray(default_command, dtype=np.float64), (sampled.shape[0], 1))
    full[:, idxs] = sampled
    return full
