"""Ground-truth trajectories, reference evaluation and landscape in FP64 (test infrastructure).

* ``collect`` records frames the way scripts/data/sine.py:39-72 does: each
  frame holds the state *after* its action, plus the action itself; the dict
  keys follow scripts/data/common.py:format_data (:83-100).
* ``evaluate_reference`` restates scripts/eval.py:evaluate_batch (:217-310)
  for one theta: chunk by chunk, the chunk's first-row PD gains, reset every
  window to its logged state, replay H actions, reference L2 errors at the final
  step, per-chunk mask, mean over non-end windows -> (base_pos, base_quat,
  joint_pos).
* ``landscape`` restates scripts/mass_landscape.py:mass_sweep (:111-128) over
  base-mass scales, and the weighted total / argmin of :160-167.
"""
from __future__ import annotations

import dataclasses

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


THIGH = (1, 4, 7, 10)
CALF = (2, 5, 8, 11)
# (amplitude, frequency) per collector: scripts/data/sine.py:16-17, jump.py:16-17, stand.py (zero)
PROFILE = {"sine": (0.8, 1.0), "jump": (1.2, 1.5), "stand": (0.0, 0.0)}


def profile_actions(profile, steps, dt):
    """The collectors' action loop (scripts/data/sine.py:39-45, jump.py:39-45, stand.py:21-24),
    one step at a time: thigh actions +A sin(2 pi f t), calf actions -A sin(2 pi f t)."""
    amp, freq = PROFILE[profile]
    out = np.zeros((1, steps, 12))
    for step in range(steps):
        t = step * dt
        phase = amp * np.sin(2 * np.pi * freq * t)
        for j in THIGH:
            out[0, step, j] = phase
        for j in CALF:
            out[0, step, j] = -phase
    return out


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


def _chunk(ds, start, end):
    return {k: v[start:end] for k, v in ds.items()}


def evaluate_reference(ds, theta, batch_size, sim: gm.SimParams):
    """scripts/eval.py:evaluate_batch: chunk by chunk of ``batch_size`` windows, each chunk
    rolled with the PD gains of its first row (:243-250, apply_pd_gains_batch :192-201) when
    the dataset carries them, otherwise with ``sim``'s."""
    W = ds["motion_ends"].shape[0]
    theta = np.atleast_2d(np.asarray(theta, dtype=np.float64))
    parts = []
    for start in range(0, W, batch_size):
        end = min(start + batch_size, W)
        sim_c = sim
        if "pd_gain_kp" in ds:
            sim_c = dataclasses.replace(sim, kp=np.asarray(ds["pd_gain_kp"][start], dtype=np.float64),
                                        kd=np.asarray(ds["pd_gain_kd"][start], dtype=np.float64))
        parts.append(window_components(_chunk(ds, start, end), theta, sim_c))
    comp = np.concatenate(parts, axis=1)
    w = ow.eval_mask(ds["motion_ends"], batch_size)
    mean = oc.reduce_components(comp, w, ow.total_valid(ds["motion_ends"]))
    return mean[..., 0:3]


def landscape(ds, scales, batch_size, sim: gm.SimParams, theta_nominal=gm.THETA_NOMINAL):
    th = np.tile(np.asarray(theta_nominal, dtype=np.float64), (len(scales), 1))
    th[:, 0] = gm.BASE_MASS * np.asarray(scales, dtype=np.float64)
    costs = evaluate_reference(ds, th, batch_size, sim)
    total = oc.compute_cost(costs)
    return costs, total, int(np.argmin(total))
