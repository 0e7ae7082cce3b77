"""Batched 6-D spatial algebra in FP64 (Featherstone conventions), test infrastructure.

Motion vectors are (angular; linear), force vectors (moment; force). Every
function takes leading batch dimensions. Plain dense 6x6 matrices are used on
purpose: the oracle favours obviously-correct algebra over speed.
"""
from __future__ import annotations

import numpy as np


def skew(v):
    """[..., 3] -> [..., 3, 3] with skew(a) @ b == cross(a, b)."""
    v = np.asarray(v, dtype=np.float64)
    z = np.zeros(v.shape[:-1])
    return np.stack([
        np.stack([z, -v[..., 2], v[..., 1]], -1),
        np.stack([v[..., 2], z, -v[..., 0]], -1),
        np.stack([-v[..., 1], v[..., 0], z], -1),
    ], -2)


def rot_axis(axis: int, q):
    """Active rotation matrix about the x (0) or y (1) axis by angle(s) q."""
    q = np.asarray(q, dtype=np.float64)
    c, s = np.cos(q), np.sin(q)
    o, z = np.ones_like(q), np.zeros_like(q)
    if axis == 0:
        rows = [[o, z, z], [z, c, -s], [z, s, c]]
    elif axis == 1:
        rows = [[c, z, s], [z, o, z], [-s, z, c]]
    else:
        rows = [[c, -s, z], [s, c, z], [z, z, o]]
    return np.stack([np.stack(r, -1) for r in rows], -2)


def plucker(E, r):
    """Motion transform B_X_A from A to B: E rotates A-coords to B-coords, r = B origin in A."""
    E = np.asarray(E, dtype=np.float64)
    r = np.broadcast_to(np.asarray(r, dtype=np.float64), E.shape[:-2] + (3,))
    X = np.zeros(E.shape[:-2] + (6, 6))
    X[..., :3, :3] = E
    X[..., 3:, 3:] = E
    X[..., 3:, :3] = -E @ skew(r)
    return X


def crm(v):
    """Motion cross-product operator v x (.) for motion vectors."""
    v = np.asarray(v, dtype=np.float64)
    M = np.zeros(v.shape[:-1] + (6, 6))
    w = skew(v[..., :3])
    M[..., :3, :3] = w
    M[..., 3:, 3:] = w
    M[..., 3:, :3] = skew(v[..., 3:])
    return M


def crf(v):
    """Force cross-product operator v x* (.) = -crm(v)^T."""
    return -np.swapaxes(crm(v), -1, -2)


def rigid_inertia(m, c, Ic):
    """Spatial inertia about the frame origin of a body with mass m, CoM c, inertia Ic about CoM."""
    m = np.asarray(m, dtype=np.float64)
    c = np.asarray(c, dtype=np.float64)
    Ic = np.asarray(Ic, dtype=np.float64)
    C = skew(c)
    I = np.zeros(np.broadcast_shapes(m.shape + (1, 1), Ic.shape[:-2] + (1, 1))[:-2] + (6, 6))
    mm = m[..., None, None]
    I[..., :3, :3] = Ic + mm * (C @ np.swapaxes(C, -1, -2))
    I[..., :3, 3:] = mm * C
    I[..., 3:, :3] = mm * np.swapaxes(C, -1, -2)
    I[..., 3:, 3:] = mm * np.eye(3)
    return I


def mv(M, v):
    return np.einsum("...ij,...j->...i", M, v)
