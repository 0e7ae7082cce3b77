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


def fd_fisher_episode(x0, actions, theta, param_ids, delta, ksync, sim, reset_step=True):
    """The reference's open-loop active-sysid episode for C candidates, step by step.

    Restates, in FP64 on the oracle's dynamics:
    * the env layout of active_sysid_openloop.py:51-80: every candidate is a group of 1 main
      + P aux envs, aux k with +delta on parameter param_ids[k];
    * reset_all (:116-131 over base_task.reset_all) running one zero-action step, with
      step_idx = 1 after it, before the policy loop (reset_step);
    * per step (_pre_physics_step :170-172 increments step_idx; _post_physics_step
      :209-252): the reward ``fd_fisher_reward`` of the new states, then, when
      step_idx % ksync == 1 (every step if 0 <= ksync <= 1, never if ksync < 0), the aux
      states set to the main's (_reset_envs_states_to_main_envs :316-330);
    * evaluate_policy (active_sysid.py:527-600): rewards of the loop steps summed and divided
      by the loop's step counter, which ends one above the number of steps.

    x0 [C, 37], actions [C, n, 12], theta [C, 13]. Returns (mean reward [C], per-step rewards
    [C, n] of the loop steps)."""
    from . import dynamics as dyn
    x0 = np.asarray(x0, dtype=np.float64)
    actions = np.asarray(actions, dtype=np.float64)
    C, n = actions.shape[:2]
    theta = np.broadcast_to(np.atleast_2d(np.asarray(theta, dtype=np.float64)), (C, 13))
    P = len(param_ids)
    G = P + 1
    th = np.repeat(theta, G, 0)
    for k, s in enumerate(param_ids):
        th[k + 1::G, s] += delta
    x = np.repeat(x0, G, 0)
    main = np.arange(C) * G
    origins = np.zeros((C * G, 3))

    def reward(xs):
        return fd_fisher_reward(xs[:, :13], xs[:, 13:25], origins, C, P, delta)[main]

    def resync(xs, step_idx):
        if ksync >= 0 and (ksync <= 1 or step_idx % ksync == 1):
            xs = xs.copy()
            for k in range(1, G):
                xs[main + k] = xs[main]
        return xs

    step_idx = 0
    if reset_step:
        x = dyn.control_step(x, np.zeros((C * G, 12)), th, sim)
        step_idx = 1
        x = resync(x, step_idx)
    per_step = np.zeros((C, n))
    step = 1
    for t in range(n):
        x = dyn.control_step(x, np.repeat(actions[:, t], G, 0), th, sim)
        step_idx += 1
        per_step[:, t] = reward(x)
        x = resync(x, step_idx)
        step += 1
    return per_step.sum(1) / step, per_step
