"""Candidate-command parametrisations (test infrastructure).

Restates spigym/agents/sysid/active_sysid.py:259-400 in its own loop form, one update,
dimension and time step at a time, so that it checks the product's vectorised version
(spi_gb300.excitation) independently. ``values`` is the flat list of numbers an Optuna trial
would return, in the order the reference asks for them:

* constant (:295-316): dimension-major, then update;
* polynomial (:318-358): update, dimension, coefficient (degree + 1 of them);
* bezier (:360-400): update, dimension, control point.
"""
from __future__ import annotations

import math

import numpy as np


def constant(values, n_updates, n_dims, steps):
    """One value per (dimension, update), held for ``steps`` control steps (:295-316)."""
    it = iter(values)
    held = [[0.0] * n_dims for _ in range(n_updates)]
    for d in range(n_dims):
        for u in range(n_updates):
            held[u][d] = float(next(it))
    out = []
    for u in range(n_updates):
        for _ in range(steps):
            out.append(list(held[u]))
    return np.array(out)


def _t_grid(steps):
    """steps points from 0 to 1 inclusive (np.linspace(0, 1, steps))."""
    if steps == 1:
        return [0.0]
    return [i / (steps - 1) for i in range(steps)]


def polynomial(values, ranges, idxs, n_updates, steps, degree):
    """Per update and dimension: tanh of a degree-``degree`` polynomial in t, mapped from
    [-1, 1] onto the dimension's range (:318-358)."""
    it = iter(values)
    t = _t_grid(steps)
    n_dims = len(idxs)
    out = []
    for _ in range(n_updates):
        coeffs = [[float(next(it)) for _ in range(degree + 1)] for _ in range(n_dims)]
        seg = [[0.0] * n_dims for _ in range(steps)]
        for d in range(n_dims):
            vmin, vmax = ranges[idxs[d]]
            for s in range(steps):
                p = 0.0
                for i, c in enumerate(coeffs[d]):
                    p += c * t[s] ** i
                seg[s][d] = vmin + (math.tanh(p) + 1.0) * 0.5 * (vmax - vmin)
        out.extend(seg)
    return np.array(out)


def bezier(values, ranges, idxs, n_updates, steps, n_points):
    """Per update and dimension: the Bezier curve of ``n_points`` control points (Bernstein
    basis of degree n_points - 1), clipped to the dimension's range (:360-400)."""
    it = iter(values)
    t = _t_grid(steps)
    n_dims = len(idxs)
    n = n_points - 1
    out = []
    for _ in range(n_updates):
        cp = [[float(next(it)) for _ in range(n_points)] for _ in range(n_dims)]
        seg = [[0.0] * n_dims for _ in range(steps)]
        for d in range(n_dims):
            vmin, vmax = ranges[idxs[d]]
            for s in range(steps):
                v = 0.0
                for j in range(n_points):
                    v += math.comb(n, j) * t[s] ** j * (1.0 - t[s]) ** (n - j) * cp[d][j]
                seg[s][d] = min(max(v, vmin), vmax)
        out.extend(seg)
    return np.array(out)


def expand(sampled, default_command, idxs):
    """The default command on every step, the sampled dimensions written over it (:286-292)."""
    sampled = np.asarray(sampled, dtype=np.float64)
    out = []
    for s in range(sampled.shape[0]):
        row = [float(v) for v in default_command]
        for k, i in enumerate(idxs):
            row[int(i)] = float(sampled[s, k])
        out.append(row)
    return np.array(out)
