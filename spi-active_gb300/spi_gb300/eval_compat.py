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

``evaluate_batch`` reproduces the reference's chunked masking: windows at and
after the first motion end of each ``num_envs`` chunk get weight 0, sums are
divided by the number of non-end windows. The environment is the GPU engine: all
windows of all chunks are rolled in one launch. ``mass_sweep`` evaluates every
mass scale in the same launch instead of one scale after another.
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


class EvalEnv:
    """Stands in for the LeggedRobotBase that ``instantiate_env`` returns in the reference."""

    def __init__(self, num_envs: int, cfg: SimConfig | None = None, device=None):
        self.num_envs = int(num_envs)
        self.dim_actions = 12
        self.cfg = cfg or SimConfig.reference_compatible()
        self.device = torch.device(device) if device is not None else torch.device("cuda")
        self.engine = Engine(self.cfg, device=self.device)
        self.engine.set_cost(COST_REF)
        self.simulator = EngineSimulatorHandle(self)
        self.theta = torch.tensor(THETA_NOMINAL, dtype=torch.float32, device=self.device)[None].clone()
        self._loaded = None
        self.p_gains = torch.tensor(np.broadcast_to(np.asarray(self.cfg.kp, np.float32), (12,)).copy(),
                                    device=self.device)
        self.d_gains = torch.tensor(np.broadcast_to(np.asarray(self.cfg.kd, np.float32), (12,)).copy(),
                                    device=self.device)

    def _sync_gains(self):
        kp = self.p_gains.detach().cpu().numpy().astype(np.float64)
        kd = self.d_gains.detach().cpu().numpy().astype(np.float64)
        if not (np.array_equal(np.broadcast_to(np.asarray(self.cfg.kp, np.float64), (12,)), kp)
                and np.array_equal(np.broadcast_to(np.asarray(self.cfg.kd, np.float64), (12,)), kd)):
            self.cfg = SimConfig(**{**self.cfg.__dict__, "kp": tuple(kp), "kd": tuple(kd)})
            self.engine = Engine(self.cfg, device=self.device)
            self.engine.set_cost(COST_REF)
            self._loaded = None

    def load(self, dataset: DatasetBatch):
        self._sync_gains()
        key = (id(dataset), self.num_envs)
        if self._loaded == key:
            return
        me = dataset.motion_ends.detach().cpu().numpy()
        weight, n_valid = sd.eval_weights(me, self.num_envs)
        W = me.shape[0]
        z3 = torch.zeros((W, 3), device=self.device)
        z12 = torch.zeros((W, 12), device=self.device)
        init = torch.cat([dataset.init_base_pos, dataset.init_base_ori, dataset.init_base_lin_vel,
                          dataset.init_base_ang_vel, dataset.init_joint_pos, dataset.init_joint_vel], -1)
        tgt = torch.cat([dataset.target_base_pos, dataset.target_base_ori,
                         dataset.target_base_lin_vel if dataset.target_base_lin_vel is not None else z3,
                         dataset.target_base_ang_vel if dataset.target_base_ang_vel is not None else z3,
                         dataset.target_joint_pos,
                         dataset.target_joint_vel if dataset.target_joint_vel is not None else z12], -1)
        self.engine.load_windows(init, dataset.action_sequences, tgt, torch.from_numpy(weight), norm=n_valid)
        self._loaded = key

    def evaluate_thetas(self, dataset: DatasetBatch, theta: torch.Tensor) -> np.ndarray:
        """Reference (base_pos, base_quat, joint_pos) means for every row of theta [N,13]."""
        self.load(dataset)
        comp, _ = self.engine.evaluate(theta)
        return comp[:, 0:3].double().cpu().numpy()


def instantiate_env(base_dir=None, num_envs: int = 4096, config_name: str = "env/go2_test", seed: int = 0,
                    cfg: SimConfig | None = None) -> EvalEnv:
    return EvalEnv(num_envs, cfg)


def capture_reference_masses(simulator) -> np.ndarray:
    return simulator.body_masses.copy()


def apply_pd_gains_batch(env: EvalEnv, kp_batch: torch.Tensor, kd_batch: torch.Tensor) -> None:
    env.p_gains[:] = kp_batch[0]
    env.d_gains[:] = kd_batch[0]


def apply_base_mass(simulator, reference_masses: np.ndarray, base_mass: float) -> None:
    simulator._env.theta[:, 0] = float(base_mass)


@torch.no_grad()
def evaluate_batch(env: EvalEnv, horizon: int, action_buffer: torch.Tensor, dataset: DatasetBatch) -> MassEvalResult:
    if dataset.action_sequences.shape[1] != horizon:
        raise ValueError(f"dataset horizon {dataset.action_sequences.shape[1]} != {horizon}")
    apply_pd_gains_batch(env, dataset.pd_gain_kp, dataset.pd_gain_kd)
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
    apply_pd_gains_batch(env, dataset.pd_gain_kp, dataset.pd_gain_kd)
    return env.evaluate_thetas(dataset, theta).astype(np.float32)
