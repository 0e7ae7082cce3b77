"""Logged-trajectory formats, windows, and the GPU data collector.

* ``format_data`` / npz keys follow the reference's collectors
  (scripts/data/common.py:83-100; frame layout scripts/data/sine.py:62-72):
  each frame holds the state *after* its action.
* ``load_dataset`` follows scripts/eval.py:101-171 (init = frame i, target =
  frame i+H, actions = frames i..i+H-1, last window of a trajectory flagged in
  ``motion_ends``, scalar Kp/Kd broadcast). ``causal=True`` takes actions
  i+1..i+H, the pairing under which a replay at the generating theta
  reproduces the target exactly.
* ``eval_weights`` is the per-chunk mask of scripts/eval.py:279-280 and the
  normaliser of :304.
* ``collect`` rolls trajectories on the GPU engine (the counterpart of the
  Isaac Gym collectors scripts/data/{sine,jump,stand}.py), with per-joint sine
  targets, the synchronized thigh/calf sine of sine.py:39-45 / jump.py:15-21
  or zero actions (stand.py); ``collect_profile`` runs one of the reference's
  three profiles end to end and returns its npz dict.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np
import torch

from .robot import DEFAULT_DOF_POS, STATE_DIM, SimConfig

STATE_KEYS = ("base_positions", "base_orientations", "base_linear_velocities",
              "base_angular_velocities", "joint_positions", "joint_velocities")
THIGH_IDX = (1, 4, 7, 10)
CALF_IDX = (2, 5, 8, 11)


def standing_state(n: int, z: float = 0.33) -> np.ndarray:
    x = np.zeros((n, STATE_DIM), dtype=np.float32)
    x[:, 2] = z
    x[:, 6] = 1.0
    x[:, 13:25] = DEFAULT_DOF_POS
    return x


def sine_actions(T, amp, freq, phase, control_dt, action_scale, settle=0) -> np.ndarray:
    """Per-joint sine joint-target offsets amp*sin(2 pi f t + phase), as raw actions [B,T,12]."""
    amp, freq, phase = (np.asarray(a, dtype=np.float64) for a in (amp, freq, phase))
    t = (np.arange(T) - settle) * control_dt
    a = (amp[:, None, :] / action_scale) * np.sin(2 * np.pi * freq[:, None, :] * t[None, :, None]
                                                 + phase[:, None, :])
    a[:, :settle] = 0.0
    return a.astype(np.float32)


def reference_sine_actions(T, amplitude, frequency, control_dt) -> np.ndarray:
    """The reference collectors' thigh/calf sine (sine.py: 0.8 rad-action at 1 Hz; jump.py: 1.2 at 1.5 Hz)."""
    t = np.arange(T) * control_dt
    phase = amplitude * np.sin(2 * np.pi * frequency * t)
    a = np.zeros((1, T, 12), dtype=np.float32)
    a[0][:, list(THIGH_IDX)] = phase[:, None]
    a[0][:, list(CALF_IDX)] = -phase[:, None]
    return a


# Open-loop profiles of the reference's collectors: thigh targets +A sin(2 pi f t), calf targets
# -A sin(2 pi f t) in action units, 5 s from a base height of 0.32 m (scripts/data/sine.py:15-21,
# 39-45; jump.py:15-21, 39-45), or zero actions (stand.py:14-15, 21).
PROFILES = {"sine": (0.8, 1.0), "jump": (1.2, 1.5), "stand": (0.0, 0.0)}
COLLECT_DURATION_S = 5.0
COLLECT_BASE_HEIGHT = 0.32


def profile_actions(profile: str, T: int, control_dt: float) -> np.ndarray:
    """Actions [1, T, 12] of a reference collector profile ("sine", "jump" or "stand")."""
    if profile not in PROFILES:
        raise ValueError(f"unknown collector profile {profile!r} (one of {sorted(PROFILES)})")
    amp, freq = PROFILES[profile]
    return reference_sine_actions(T, amp, freq, control_dt)


def collect_profile(engine, profile: str, duration_s: float = COLLECT_DURATION_S, theta=None,
                    base_height: float = COLLECT_BASE_HEIGHT) -> dict:
    """One trajectory of a reference collector profile rolled on the GPU engine, as the npz dict
    the reference's collectors write (states after each action, the action, PD gains)."""
    from .robot import THETA_NOMINAL
    cfg = engine.cfg
    T = int(round(duration_s / cfg.control_dt))
    if T <= 0:
        raise ValueError(f"duration {duration_s} s is shorter than one control step")
    acts = profile_actions(profile, T, cfg.control_dt)
    th = THETA_NOMINAL if theta is None else theta
    states = collect(engine, standing_state(1, z=base_height), acts, th)
    return format_data(states[0], acts[0], cfg)


def collect(engine, x0, actions, theta) -> np.ndarray:
    """Roll each initial state with its action sequence on the GPU; states after every step [B,T,37]."""
    x0 = torch.as_tensor(np.asarray(x0, dtype=np.float32))
    actions = torch.as_tensor(np.asarray(actions, dtype=np.float32))
    theta = torch.as_tensor(np.asarray(theta, dtype=np.float32)).reshape(1, -1)
    engine.load_windows(x0, actions, x0)
    _, _, tr = engine.evaluate(theta, trace=True)
    torch.cuda.synchronize()
    return tr[0].cpu().numpy()


def format_data(states: np.ndarray, actions: np.ndarray, cfg: SimConfig) -> dict:
    """One trajectory (states after each action [T,37], actions [T,12]) as the reference npz dict."""
    T = states.shape[0]
    s = np.asarray(states, dtype=np.float32)
    kp = np.broadcast_to(np.asarray(cfg.kp, dtype=np.float32), (12,)).copy()
    kd = np.broadcast_to(np.asarray(cfg.kd, dtype=np.float32), (12,)).copy()
    return {
        "joint_positions": s[:, 13:25], "joint_velocities": s[:, 25:37],
        "actions": np.asarray(actions, dtype=np.float32),
        "base_positions": s[:, 0:3], "base_orientations": s[:, 3:7],
        "base_linear_velocities": s[:, 7:10], "base_angular_velocities": s[:, 10:13],
        "timestamps": np.arange(T) * cfg.control_dt, "sim_duration": T * cfg.control_dt,
        "data_frequency": int(round(1.0 / cfg.control_dt)), "robot_type": "go2",
        "pd_gain_kp": kp, "pd_gain_kd": kd,
    }


def save_npz(path, data: dict) -> None:
    np.savez(path, **data)


def load_npz(path) -> dict:
    with np.load(Path(path), allow_pickle=False) as d:
        return {k: d[k] for k in d.files}


def load_dataset(trajectories, horizon: int, causal: bool = False):
    """Windows from trajectories (dicts or npz paths). Returns (num_samples, dict of arrays)."""
    parts = []
    for d in trajectories:
        if not isinstance(d, dict):
            d = load_npz(d)
        T = d["base_positions"].shape[0]
        n = T - horizon
        if n <= 0:
            raise ValueError(f"trajectory of {T} frames is too short for horizon {horizon}")
        i = np.arange(n)
        t = i + horizon
        out = {
            "init_base_pos": d["base_positions"][i], "target_base_pos": d["base_positions"][t],
            "init_base_ori": d["base_orientations"][i], "target_base_ori": d["base_orientations"][t],
            "init_base_lin_vel": d["base_linear_velocities"][i],
            "init_base_ang_vel": d["base_angular_velocities"][i],
            "init_joint_pos": d["joint_positions"][i], "target_joint_pos": d["joint_positions"][t],
            "init_joint_vel": d["joint_velocities"][i],
            "target_base_lin_vel": d["base_linear_velocities"][t],
            "target_base_ang_vel": d["base_angular_velocities"][t],
            "target_joint_vel": d["joint_velocities"][t],
        }
        idx = i[:, None] + np.arange(horizon)[None, :] + (1 if causal else 0)
        out["action_sequences"] = d["actions"].astype(np.float32)[idx]
        me = np.zeros(n, dtype=bool)
        me[-1] = True
        out["motion_ends"] = me
        J = d["joint_positions"].shape[1]
        out["pd_gain_kp"] = np.full((n, J), float(np.asarray(d["pd_gain_kp"]).flat[0]), np.float32)
        out["pd_gain_kd"] = np.full((n, J), float(np.asarray(d["pd_gain_kd"]).flat[0]), np.float32)
        parts.append(out)
    cat = {k: np.concatenate([p[k] for p in parts], 0) for k in parts[0]}
    return cat["init_base_pos"].shape[0], cat


def init_states(ds) -> np.ndarray:
    return np.concatenate([ds["init_base_pos"], ds["init_base_ori"], ds["init_base_lin_vel"],
                           ds["init_base_ang_vel"], ds["init_joint_pos"], ds["init_joint_vel"]],
                          -1).astype(np.float32)


def target_states(ds) -> np.ndarray:
    return np.concatenate([ds["target_base_pos"], ds["target_base_ori"], ds["target_base_lin_vel"],
                           ds["target_base_ang_vel"], ds["target_joint_pos"], ds["target_joint_vel"]],
                          -1).astype(np.float32)


def eval_weights(motion_ends, batch_size: int):
    """(per-window 0/1 weights, normaliser) of the reference's chunked evaluate_batch."""
    me = np.asarray(motion_ends, dtype=bool)
    w = np.zeros(me.shape[0], dtype=np.float32)
    for s in range(0, me.shape[0], batch_size):
        w[s:s + batch_size] = ~(np.cumsum(me[s:s + batch_size].astype(np.float64)) > 0)
    return w, int((~me).sum())


def synthetic_windows(engine, theta_true, n_windows, horizon, n_traj=4, settle=100, seed=0,
                      amp=(0.1, 0.4), freq=(1.0, 3.0)):
    """Seeded ground truth on the GPU: settle, then per-joint sine excitation; causal windows.

    Returns (init [W,37], actions [W,H,12], target [W,37]) as float32 numpy arrays.
    """
    cfg = engine.cfg
    rng = np.random.default_rng(seed)
    per = -(-n_windows // n_traj)
    T = per + horizon + 1
    a = rng.uniform(amp[0], amp[1], (n_traj, 12))
    f = rng.uniform(freq[0], freq[1], (n_traj, 12))
    ph = rng.uniform(0.0, 2 * np.pi, (n_traj, 12))
    acts = sine_actions(settle + T, a, f, ph, cfg.control_dt, cfg.action_scale, settle=settle)
    states = collect(engine, standing_state(n_traj), acts, theta_true)
    trajs = [format_data(states[b, settle:], acts[b, settle:], cfg) for b in range(n_traj)]
    _, ds = load_dataset(trajs, horizon, causal=True)
    sel = slice(0, n_windows)
    return (init_states(ds)[sel], ds["action_sequences"][sel].astype(np.float32), target_states(ds)[sel])
