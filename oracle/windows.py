"""Window construction and evaluation masks (test infrastructure).

Restates scripts/eval.py of the reference:
* ``load_dataset`` :101-171 -- per trajectory, init = frame[i], target =
  frame[i+H], actions = frames[i .. i+H-1], motion_ends[-1] = True, scalar
  Kp/Kd (first element) broadcast per window, trajectories concatenated.
  ``causal=True`` shifts the action window by one (frames[i+1 .. i+H]): a frame
  holds the state *after* its action (scripts/data/sine.py:51-72), so the
  reference pairing is one step early; the causal pairing replays exactly.
* ``eval_mask`` :279-280 -- within each env-batch chunk, windows at and after
  the first motion end are masked out; ``total_valid`` :304 counts all
  non-end windows.
"""
from __future__ import annotations

import numpy as np

STATE_KEYS = ("base_positions", "base_orientations", "base_linear_velocities",
              "base_angular_velocities", "joint_positions", "joint_velocities")


def load_dataset(trajectories, horizon, causal=False):
    """trajectories: list of dicts with the npz keys of scripts/data/common.py:format_data."""
    parts = []
    for d in trajectories:
        T = d["base_positions"].shape[0]
        shift = 1 if causal else 0
        n = T - horizon
        i = np.arange(n)
        t = i + horizon
        out = {
            "init_base_pos": d["base_positions"][i],
            "target_base_pos": d["base_positions"][t],
            "init_base_ori": d["base_orientations"][i],
            "target_base_ori": d["base_orientations"][t],
            "init_base_lin_vel": d["base_linear_velocities"][i],
            "init_base_ang_vel": d["base_angular_velocities"][i],
            "init_joint_pos": d["joint_positions"][i],
            "target_joint_pos": d["joint_positions"][t],
            "init_joint_vel": d["joint_velocities"][i],
            # extension: full target state for the weighted squared-error cost
            "target_base_lin_vel": d["base_linear_velocities"][t],
            "target_base_ang_vel": d["base_angular_velocities"][t],
            "target_joint_vel": d["joint_velocities"][t],
        }
        acts = d["actions"].astype(np.float32)
        idx = i[:, None] + np.arange(horizon)[None, :] + shift   # <= T-1 in both modes
        out["action_sequences"] = acts[idx]
        me = np.zeros(n, dtype=bool)
        if n:
            me[-1] = True
        out["motion_ends"] = me
        J = d["joint_positions"].shape[1]
        out["pd_gain_kp"] = np.full((n, J), float(np.asarray(d["pd_gain_kp"]).flat[0]), np.float32)
        out["pd_gain_kd"] = np.full((n, J), float(np.asarray(d["pd_gain_kd"]).flat[0]), np.float32)
        parts.append(out)
    cat = {k: np.concatenate([p[k] for p in parts], 0) for k in parts[0]}
    return cat["init_base_pos"].shape[0], cat


def init_states(ds):
    return np.concatenate([ds["init_base_pos"], ds["init_base_ori"], ds["init_base_lin_vel"],
                           ds["init_base_ang_vel"], ds["init_joint_pos"], ds["init_joint_vel"]], -1)


def target_states(ds):
    return np.concatenate([ds["target_base_pos"], ds["target_base_ori"], ds["target_base_lin_vel"],
                           ds["target_base_ang_vel"], ds["target_joint_pos"], ds["target_joint_vel"]], -1)


def eval_mask(motion_ends, batch_size):
    """Per-window 0/1 weight the reference applies, for a given env batch size."""
    me = np.asarray(motion_ends, dtype=bool)
    mask = np.zeros(me.shape[0], dtype=np.float64)
    for s in range(0, me.shape[0], batch_size):
        chunk = me[s:s + batch_size]
        mask[s:s + batch_size] = ~(np.cumsum(chunk.astype(np.float64)) > 0)
    return mask


def total_valid(motion_ends):
    return int((~np.asarray(motion_ends, dtype=bool)).sum())
