"""Drop-in replacement of the reference's replay evaluator (scripts/eval.py).

Same names, arguments and results as the reference:

* ``DatasetBatch`` / ``MassEvalResult``            scripts/eval.py:21-42
* ``load_dataset(paths, horizon)``                 scripts/eval.py:101-171
* ``to_device(dataset, device)``                   scripts/eval.py:174-182
* ``instantiate_env(base_dir, num_envs, ...)``     scripts/eval.py:313-321
* ``capture_reference_masses(simulator)``          scripts/eval.py:185-189
* ``apply_pd_gains_batch(env, kp, kd)``            scripts/eval.py:192-201 (first row, as there)
* ``apply_base_mass(simulator, masses, m)``        scripts/eval.py:204-214
* ``evaluate_batch(env, horizon, buf, dataset)``   scripts/eval.py:217-310
* ``compute_cost(costs)``                          scripts/mass_opt.py:62-76
* ``mass_sweep(env, dataset, H, masses, scales)``  scripts/mass_landscape.py:111-128

``evaluate_batch`` reproduces the reference's chunked evaluation:

* windows at and after the first motion end of each ``num_envs`` chunk get
  weight 0, and sums are divided by the number of non-end windows
  (scripts/eval.py:279-280, 304-310);
* each chunk runs with the PD gains of its first window, the row that
  ``apply_pd_gains_batch`` takes from the chunk (scripts/eval.py:243-250), so a
  dataset concatenated from files logged with different gains is scored with
  each file's own gains.

The environment is the GPU engine. Chunks that share a gain set are rolled in one
launch (one engine per distinct gain set, all its windows at once), and the
weighted sums of the gain groups add up to the reference's totals. ``mass_sweep``
evaluates every mass scale in the same launches instead of one scale after another.
"""
from __future__ import annotations

from dataclasses import dataclass, fields
from pathlib import Path
from typing import Dict, Tuple

import numpy as np
import torch

from . import data as sd
from .engine import COST_REF, Engine
from .robot import BASE_MASS, THETA_NOMINAL, SimConfig, leg_links

COST_COEFF = {"base_pos": 10.0, "base_quat": 5.0, "joint_pos": 1.0}


@dataclass
class DatasetBatch:
    init_base_pos: torch.Tensor
    target_base_pos: torch.Tensor
    init_base_ori: torch.Tensor
    target_base_ori: torch.Tensor
    init_base_lin_vel: torch.Tensor
    init_base_ang_vel: torch.Tensor
    init_joint_pos: torch.Tensor
    target_joint_pos: torch.Tensor
    init_joint_vel: torch.Tensor
    action_sequences: torch.Tensor
    motion_ends: torch.Tensor
    pd_gain_kp: torch.Tensor
    pd_gain_kd: torch.Tensor
    # full target state (this engine's extension; zero when a dataset lacks it)
    target_base_lin_vel: torch.Tensor | None = None
    target_base_ang_vel: torch.Tensor | None = None
    target_joint_vel: torch.Tensor | None = None


@dataclass
class MassEvalResult:
    base_pos: float
    base_quat: float
    joint_pos: float


def load_dataset(paths, horizon: int) -> Tuple[int, Dict[str, np.ndarray]]:
    paths = [paths] if isinstance(paths, (str, Path)) else list(paths)
    n, ds = sd.load_dataset(paths, horizon)
    print(f"Loaded {len(paths)} trajectory(s) with {n} total samples")
    return n, ds


def to_device(dataset: Dict[str, np.ndarray], device) -> DatasetBatch:
    names = {f.name for f in fields(DatasetBatch)}
    t = {}
    for key, value in dataset.items():
        if key not in names:
            continue
        dtype = torch.bool if key == "motion_ends" else torch.float32
        t[key] = torch.from_numpy(np.asarray(value)).to(device=device, dtype=dtype)
    return DatasetBatch(**t)


class EngineSimulatorHandle:
    """The ``simulator`` attribute of the evaluation env: holds the per-env theta."""

    def __init__(self, env):
        self._env = env
        masses = [BASE_MASS]
        for leg in range(4):
            masses += [link[0] for link in leg_links(leg)]
        self.body_masses = np.asarray(masses, dtype=np.float32)


def chunk_gains(kp, kd, batch_size: int):
    """Per-window PD gains as the reference's evaluate_batch applies them: every window of a
    ``batch_size`` chunk runs with the chunk's first row (scripts/eval.py:243-250 with
    apply_pd_gains_batch :192-201). kp, kd [W, 12] -> two [W, 12] float32 arrays."""
    kp = np.asarray(kp, dtype=np.float32).reshape(len(kp), -1)
    kd = np.asarray(kd, dtype=np.float32).reshape(len(kd), -1)
    W = kp.shape[0]
    first = (np.arange(W) // int(batch_size)) * int(batch_size)
    return kp[first], kd[first]


class EvalEnv:
    """Stands in for the LeggedRobotBase that ``instantiate_env`` returns in the reference.

    One GPU engine per distinct PD-gain set (the gains are part of the engine's robot model);
    ``load`` splits a dataset's windows into gain groups by the reference's chunk rule."""

    def __init__(self, num_envs: int, cfg: SimConfig | None = None, device=None):
        self.num_envs = int(num_envs)
        self.dim_actions = 12
        self.cfg = cfg or SimConfig.reference_compatible()
        self.device = torch.device(device) if device is not None else torch.device("cuda")
        self._engines: dict = {}
        self.simulator = EngineSimulatorHandle(self)
        self.theta = torch.tensor(THETA_NOMINAL, dtype=torch.float32, device=self.device)[None].clone()
        self._loaded = None
        self._groups = []
        self.p_gains = torch.tensor(np.broadcast_to(np.asarray(self.cfg.kp, np.float32), (12,)).copy(),
                                    device=self.device)
        self.d_gains = torch.tensor(np.broadcast_to(np.asarray(self.cfg.kd, np.float32), (12,)).copy(),
                                    device=self.device)

    def engine_for(self, kp, kd) -> Engine:
        """The engine whose robot model carries these per-joint gains (created once per gain set)."""
        key = (tuple(float(v) for v in np.broadcast_to(np.asarray(kp, np.float32), (12,))),
               tuple(float(v) for v in np.broadcast_to(np.asarray(kd, np.float32), (12,))))
        eng = self._engines.get(key)
        if eng is None:
            cfg = SimConfig(**{**self.cfg.__dict__, "kp": key[0], "kd": key[1]})
            eng = Engine(cfg, device=self.device)
            eng.set_cost(COST_REF)
            self._engines[key] = eng
        return eng

    @property
    def engine(self) -> Engine:
        """The engine of the environment's current gains (p_gains / d_gains)."""
        return self.engine_for(self.p_gains.detach().cpu().numpy(), self.d_gains.detach().cpu().numpy())

    def load(self, dataset: DatasetBatch):
        key = (id(dataset), self.num_envs)
        if self._loaded == key:
            return
        me = dataset.motion_ends.detach().cpu().numpy()
        weight, n_valid = sd.eval_weights(me, self.num_envs)
        W = me.shape[0]
        kp, kd = chunk_gains(dataset.pd_gain_kp.detach().cpu().numpy(),
                             dataset.pd_gain_kd.detach().cpu().numpy(), self.num_envs)
        z3 = torch.zeros((W, 3), device=self.device)
        z12 = torch.zeros((W, 12), device=self.device)
        init = torch.cat([dataset.init_base_pos, dataset.init_base_ori, dataset.init_base_lin_vel,
                          dataset.init_base_ang_vel, dataset.init_joint_pos, dataset.init_joint_vel], -1)
        tgt = torch.cat([dataset.target_base_pos, dataset.target_base_ori,
                         dataset.target_base_lin_vel if dataset.target_base_lin_vel is not None else z3,
                         dataset.target_base_ang_vel if dataset.target_base_ang_vel is not None else z3,
                         dataset.target_joint_pos,
                         dataset.target_joint_vel if dataset.target_joint_vel is not None else z12], -1)
        gains = np.concatenate([kp, kd], 1)
        _, group_of = np.unique(gains, axis=0, return_inverse=True)
        group_of = group_of.reshape(-1)
        self._groups = []
        for gid in range(int(group_of.max()) + 1):
            rows = np.flatnonzero(group_of == gid)
            if not np.any(weight[rows] > 0):
                continue                     # every window of this gain set is masked out
            eng = self.engine_for(kp[rows[0]], kd[rows[0]])
            idx = torch.from_numpy(rows).to(self.device)
            eng.load_windows(init.index_select(0, idx), dataset.action_sequences.index_select(0, idx),
                             tgt.index_select(0, idx), torch.from_numpy(weight[rows]), norm=n_valid)
            self._groups.append(eng)
        # the reference leaves the last chunk's gains applied
        last = ((W - 1) // self.num_envs) * self.num_envs
        self.p_gains[:] = torch.from_numpy(kp[last])
        self.d_gains[:] = torch.from_numpy(kd[last])
        self._loaded = key

    def evaluate_thetas(self, dataset: DatasetBatch, theta: torch.Tensor) -> np.ndarray:
        """Reference (base_pos, base_quat, joint_pos) means for every row of theta [N,13]: the
        weighted sums of every gain group over the dataset's non-end window count."""
        self.load(dataset)
        total = np.zeros((int(theta.shape[0]), 3))
        for eng in self._groups:
            comp, _ = eng.evaluate(theta)
            total += comp[:, 0:3].double().cpu().numpy()
        return total


def instantiate_env(base_dir=None, num_envs: int = 4096, config_name: str = "env/go2_test", seed: int = 0,
                    cfg: SimConfig | None = None) -> EvalEnv:
    return EvalEnv(num_envs, cfg)


def capture_reference_masses(simulator) -> np.ndarray:
    return simulator.body_masses.copy()


def apply_pd_gains_batch(env: EvalEnv, kp_batch: torch.Tensor, kd_batch: torch.Tensor) -> None:
    """The env's current gains become the batch's first row (``env.engine`` then runs with them).
    evaluate_batch applies each chunk's own first row itself."""
    env.p_gains[:] = kp_batch[0]
    env.d_gains[:] = kd_batch[0]


def apply_base_mass(simulator, reference_masses: np.ndarray, base_mass: float) -> None:
    simulator._env.theta[:, 0] = float(base_mass)


@torch.no_grad()
def evaluate_batch(env: EvalEnv, horizon: int, action_buffer: torch.Tensor, dataset: DatasetBatch) -> MassEvalResult:
    if dataset.action_sequences.shape[1] != horizon:
        raise ValueError(f"dataset horizon {dataset.action_sequences.shape[1]} != {horizon}")
    r = env.evaluate_thetas(dataset, env.theta)[0]
    return MassEvalResult(base_pos=float(r[0]), base_quat=float(r[1]), joint_pos=float(r[2]))


def compute_cost(costs) -> float:
    return (costs[0] * COST_COEFF["base_pos"] + costs[1] * COST_COEFF["base_quat"]
            + costs[2] * COST_COEFF["joint_pos"])


@torch.no_grad()
def mass_sweep(env: EvalEnv, dataset: DatasetBatch, horizon: int, reference_masses: np.ndarray,
               mass_scales) -> np.ndarray:
    """All scales in one launch; returns [S, 3] float32 like the reference."""
    scales = np.asarray(list(mass_scales), dtype=np.float32)
    base_nominal = float(reference_masses[0])
    theta = env.theta.repeat(len(scales), 1)
    theta[:, 0] = torch.from_numpy((base_nominal * scales.astype(np.float64)).astype(np.float32)).to(theta.device)
    return env.evaluate_thetas(dataset, theta).astype(np.float32)
