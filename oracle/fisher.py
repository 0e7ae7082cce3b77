"""Fisher-information objectives in FP64 (test infrastructure).

* ``fd_fisher_reward`` restates the reference's finite-difference proxy,
  spigym/envs/sysid/active_sysid_openloop.py:402-426: envs are laid out as
  groups of (1 main + P aux), aux k carries +delta on parameter k
  (:51-68); J = (s_main - s_aux)/delta over the 13 root-state entries
  (positions minus env origins) and the 12 joint positions; the reward is
  trace(J^T J), repeated to every env of the group.
* ``fisher_logdet`` is the adjoint-based objective: F = sum_w J_w^T diag(w) J_w
  over windows (J_w = d s_H / d theta, 37 x P), scored by log det(F + eps I).
"""
from __future__ import annotations

import numpy as np


def fd_fisher_reward(root, dof, origins, n_main, P, delta):
    root = np.asarray(root, dtype=np.float64).copy()
    dof = np.asarray(dof, dtype=np.float64)
    root[:, :3] -= np.asarray(origins, dtype=np.float64)
    root = root.reshape(n_main, P + 1, 13)
    dof = dof.reshape(n_main, P + 1, 12)
    g = np.concatenate([(root[:, :1] - root[:, 1:]) / delta, (dof[:, :1] - dof[:, 1:]) / delta], -1)
    tr = np.einsum("npk,npk->n", g, g)
    return np.repeat(tr, P + 1)


def fisher_matrix(J, weights=None):
    """J [..., W, 37, P] -> [..., P, P] summed over windows."""
    J = np.asarray(J, dtype=np.float64)
    if weights is None:
        return np.einsum("...wsp,...wsq->...pq", J, J)
    return np.einsum("...wsp,s,...wsq->...pq", J, np.asarray(weights, np.float64), J)


def fisher_logdet(F, eps=1e-6):
    F = np.asarray(F, dtype=np.float64)
    P = F.shape[-1]
    L = np.linalg.cholesky(F + eps * np.eye(P))
    return 2.0 * np.sum(np.log(np.diagonal(L, axis1=-2, axis2=-1)), -1)
