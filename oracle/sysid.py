"""Ground-truth trajectories, reference evaluation and landscape in FP64 (test infrastructure).

* ``collect`` records frames the way scripts/data/sine.py:39-72 does: each
  frame holds the state *after* its action, plus the action itself; the dict
  keys follow scripts/data/common.py:format_data (:83-100).
* ``evaluate_reference`` restates scripts/eval.py:evaluate_batch (:217-310)
  for one theta: reset every window to its logged state, replay H actions,
  reference L2 errors at the final step, per-chunk mask, mean over non-end
  windows -> (base_pos, base_quat, joint_pos).
* ``landscape`` restates scripts/mass_landscape.py:mass_sweep (:111-128) over
  base-mass scales, and the weighted total / argmin of :160-167.
"""
from __future__ import annotations

import numpy as np

from . import cost as oc
from . import dynamics as dyn
from . import go2_model as gm
from . import windows as ow


def sine_actions(T, amp, freq, phase, control_dt, action_scale, settle=0):
    """Per-joint sine joint-target offsets amp*sin(2 pi f t + phase) as actions [B,T,12]."""
    t = (np.arange(T) - settle) * control_dt
    a = (np.asarray(amp)[:, None, :] / action_scale) * np.sin(
        2 * np.pi * np.asarray(freq)[:, None, :] * t[None, :, None] + np.asarray(phase)[:, None, :])
    a[:, :settle] = 0.0
    return a


def standing_state(B, z=0.33):
    x = np.zeros((B, gm.STATE_DIM))
    x[:, 2] = z
    x[:, 6] = 1.0
    x[:, 13:25] = gm.DEFAULT_DOF_POS
    return x


def collect(x0, actions, theta, sim: gm.SimParams):
    """Roll a batch and return one format_data-style dict per rollout."""
    tr = dyn.rollout(x0, actions, theta, sim, trace=True)
    out = []
    T = actions.shape[1]
    for b in range(tr.shape[0]):
        s = tr[b].astype(np.float32)
        out.append({
            "joint_positions": s[:, 13:25], "joint_velocities": s[:, 25:37],
            "actions": np.asarray(actions[b], dtype=np.float32),
            "base_positions": s[:, 0:3], "base_orientations": s[:, 3:7],
            "base_linear_velocities": s[:, 7:10], "base_angular_velocities": s[:, 10:13],
            "timestamps": np.arange(T) * sim.control_dt,
            "sim_duration": T * sim.control_dt,
            "data_frequency": int(round(1.0 / sim.control_dt)),
            "robot_type": "go2",
            "pd_gain_kp": np.asarray(sim.kp, dtype=np.float32).reshape(-1),
            "pd_gain_kd": np.asarray(sim.kd, dtype=np.float32).reshape(-1),
        })
    return out


def window_components(ds, theta, sim: gm.SimParams):
    """[N, W, 9] error components of every (theta, window) pair."""
    x0 = ow.init_states(ds).astype(np.float64)
    tgt = ow.target_states(ds).astype(np.float64)
    acts = ds["action_sequences"].astype(np.float64)
    theta = np.atleast_2d(np.asarray(theta, dtype=np.float64))
    N, W = theta.shape[0], x0.shape[0]
    th = np.repeat(theta, W, 0)
    fin = dyn.rollout(np.tile(x0, (N, 1)), np.tile(acts, (N, 1, 1)), th, sim)
    return oc.window_components(fin, np.tile(tgt, (N, 1))).reshape(N, W, oc.N_COMP)


def evaluate_reference(ds, theta, batch_size, sim: gm.SimParams):
    comp = window_components(ds, theta, sim)
    w = ow.eval_mask(ds["motion_ends"], batch_size)
    mean = oc.reduce_components(comp, w, ow.total_valid(ds["motion_ends"]))
    return mean[..., 0:3]


def landscape(ds, scales, batch_size, sim: gm.SimParams, theta_nominal=gm.THETA_NOMINAL):
    th = np.tile(np.asarray(theta_nominal, dtype=np.float64), (len(scales), 1))
    th[:, 0] = gm.BASE_MASS * np.asarray(scales, dtype=np.float64)
    costs = evaluate_reference(ds, th, batch_size, sim)
    total = oc.compute_cost(costs)
    return costs, total, int(np.argmin(total))
