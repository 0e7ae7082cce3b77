"""Per-window errors and per-sample costs (test infrastructure).

* Reference cost (scripts/eval.py:287-310): final-step L2 norms of the base
  position error, the raw xyzw quaternion difference and the joint position
  error, masked, summed, divided by the number of non-end windows; weighted
  10 / 5 / 1 by ``compute_cost`` (scripts/mass_opt.py:28-32, 62-76).
* Weighted squared error (six blocks: position, quaternion, linear velocity,
  angular velocity, joint position, joint velocity) at the final step, mean
  over the valid windows.

Component order shared with the CUDA kernel:
  0 |dp|   1 |dquat|   2 |dq|                 (reference L2 norms)
  3 |dp|^2 4 |dquat|^2 5 |dv|^2 6 |dw|^2 7 |dq|^2 8 |dqd|^2
"""
from __future__ import annotations

import numpy as np

REF_COEFF = np.array([10.0, 5.0, 1.0])
BLOCKS = ((0, 3), (3, 7), (7, 10), (10, 13), (13, 25), (25, 37))
N_COMP = 9


def window_components(final, target):
    """final, target [..., 37] -> [..., 9] error components of each window."""
    d = np.asarray(final, dtype=np.float64) - np.asarray(target, dtype=np.float64)
    sq = np.stack([np.sum(d[..., a:b] ** 2, -1) for a, b in BLOCKS], -1)
    l2 = np.sqrt(np.stack([sq[..., 0], sq[..., 1], sq[..., 4]], -1))
    return np.concatenate([l2, sq], -1)


def reduce_components(comp, weight, n_valid):
    """Masked mean over windows. comp [..., W, 9], weight [W] -> [..., 9]."""
    return np.einsum("...wk,w->...k", comp, np.asarray(weight, dtype=np.float64)) / float(n_valid)


def compute_cost(costs):
    """Reference weighted cost of (base_pos, base_quat, joint_pos) means."""
    costs = np.asarray(costs, dtype=np.float64)
    return costs[..., 0] * REF_COEFF[0] + costs[..., 1] * REF_COEFF[1] + costs[..., 2] * REF_COEFF[2]


DEFAULT_SQ_WEIGHTS = np.array([10.0, 5.0, 0.1, 0.1, 1.0, 0.01])


def scalar_cost(mean_comp, mode="sq", sq_weights=DEFAULT_SQ_WEIGHTS):
    """mode 'ref': reference 10/5/1 weights of the L2 means; 'sq': weighted squared error."""
    mean_comp = np.asarray(mean_comp, dtype=np.float64)
    if mode == "ref":
        return compute_cost(mean_comp[..., 0:3])
    return mean_comp[..., 3:9] @ np.asarray(sq_weights, dtype=np.float64)
