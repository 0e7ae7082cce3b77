"""Candidate-excitation parametrisations of the reference's active-sysid search.

Same sampling rules as spigym/agents/sysid/active_sysid.py:259-400, with the Optuna trial
replaced by a flat vector of the values a trial would return (in the order the reference asks
for them):

* ``constant``   -- one value per (dimension, update), held for ``steps`` control steps (:295-316)
* ``polynomial`` -- per update and dimension a degree-d polynomial on t in [0, 1], squashed
  with tanh and mapped to the range (:318-358)
* ``bezier``     -- per update and dimension a Bezier curve through n control points,
  clipped to the range (:360-400)
* ``expand``     -- sampled dimensions over the default command (:286-292)

The reference feeds these commands to a trained omni policy (not available here); the engine
scores them open loop as joint-target offsets (``as_actions``) with the Fisher information of
its exact sensitivities (spi_gb300.sensitivity.score_excitations).
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
    poly = np.tanh(np.einsum("udk,ks->usd", c, t[None, :] ** np.arange(degree + 1)[:, None]))
    lo = np.asarray([ranges[i][0] for i in idxs], np.float64)
    hi = np.asarray([ranges[i][1] for i in idxs], np.float64)
    return (lo + (poly + 1.0) * 0.5 * (hi - lo)).reshape(n_updates * steps, n_dims)


def bezier(values, ranges, idxs, n_updates, steps, n_points):
    n_dims = len(idxs)
    cp = np.asarray(values, dtype=np.float64).reshape(n_updates, n_dims, n_points)
    t = np.linspace(0.0, 1.0, steps)
    n = n_points - 1
    basis = np.stack([comb(n, j) * t ** j * (1 - t) ** (n - j) for j in range(n_points)], 0)
    lo = np.asarray([ranges[i][0] for i in idxs], np.float64)
    hi = np.asarray([ranges[i][1] for i in idxs], np.float64)
    return np.clip(np.einsum("udj,js->usd", cp, basis), lo, hi).reshape(n_updates * steps, n_dims)


def expand(sampled, default_command, idxs):
    full = np.tile(np.asarray(default_command, dtype=np.float64), (sampled.shape[0], 1))
    full[:, list(idxs)] = sampled
    return full


def as_actions(joint_offsets_rad, action_scale):
    """Joint-target offsets [T, 12] (rad) as raw actions."""
    return (np.asarray(joint_offsets_rad, np.float64) / action_scale).astype(np.float32)
