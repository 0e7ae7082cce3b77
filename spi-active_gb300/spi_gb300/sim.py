"""A BaseSimulator-style view of the engine for code written against the reference's simulator.

Mirrors the parts of spigym/simulator/base_simulator/base_simulator.py (and the Isaac Gym
adapter's tensor layout, spigym/simulator/isaacgym/isaacgym.py:536-626) that the
evaluation path uses:

* ``robot_root_states`` [N, 13] (pos, quat xyzw, lin vel, ang vel), ``dof_pos`` / ``dof_vel``
  [N, 12] -- live views of the engine-side state;
* ``dof_state`` [N*12, 2] -- (pos, vel) rows, materialised on read;
* ``set_actor_root_state_tensor(env_ids, root_states)`` and
  ``set_dof_state_tensor(env_ids, dof_states)`` -- indexed writes;
* ``refresh_sim_tensors()`` -- nothing to do, the views are live;
* ``step(actions, control_steps=1)`` -- the env.step physics (clip, PD, motor model,
  ``decimation`` substeps) on every env, on the GPU;
* per-env parameters through ``set_theta`` or the reference's ``params_dict`` keys
  (``apply_params_dict``, spigym/simulator/isaacgym/isaacgym_active_sysid.py:39-95).
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .engine import Engine
from .robot import BASE_COM, BASE_INERTIA, STATE_DIM, THETA_DIM, THETA_NOMINAL, SimConfig
from .data import standing_state


class EngineSimulator:
    def __init__(self, num_envs: int, cfg: SimConfig | None = None, device=None):
        self.engine = Engine(cfg, device=device)
        self.num_envs = int(num_envs)
        self.device = self.engine.device
        self.state = torch.from_numpy(standing_state(self.num_envs)).to(self.device)
        self.theta = torch.tensor(THETA_NOMINAL, dtype=torch.float32, device=self.device).repeat(self.num_envs, 1)

    # --- tensor views (isaacgym.py:567-577) -------------------------------------------------
    @property
    def robot_root_states(self):
        return self.state[:, 0:13]

    @property
    def all_root_states(self):
        return self.state[:, 0:13]

    @property
    def dof_pos(self):
        return self.state[:, 13:25]

    @property
    def dof_vel(self):
        return self.state[:, 25:37]

    @property
    def dof_state(self):
        return torch.stack([self.dof_pos, self.dof_vel], -1).reshape(self.num_envs * 12, 2)

    # --- setters (base_simulator.py:130-147) ------------------------------------------------
    def set_actor_root_state_tensor(self, set_env_ids, root_states):
        ids = torch.as_tensor(set_env_ids, device=self.device, dtype=torch.long)
        self.state[ids, 0:13] = root_states.to(self.device, torch.float32)[ids]

    def set_dof_state_tensor(self, set_env_ids, dof_states):
        ids = torch.as_tensor(set_env_ids, device=self.device, dtype=torch.long)
        ds = dof_states.to(self.device, torch.float32).reshape(self.num_envs, 12, 2)
        self.state[ids, 13:25] = ds[ids, :, 0]
        self.state[ids, 25:37] = ds[ids, :, 1]

    def refresh_sim_tensors(self):
        return None

    # --- parameters -------------------------------------------------------------------------
    def set_theta(self, theta):
        self.theta = torch.as_tensor(theta, dtype=torch.float32, device=self.device).reshape(-1, THETA_DIM)
        if self.theta.shape[0] == 1:
            self.theta = self.theta.repeat(self.num_envs, 1)

    def apply_params_dict(self, params_dict):
        """Per-env values of the reference's keys: mass, comx/y/z (absolute base CoM), and
        inertiax/inertiay/inertiaz (absolute base diagonal inertia; the engine has one diagonal
        scale, so the three must share one ratio to the URDF values)."""
        th = self.theta.clone()
        n = self.num_envs
        if "mass" in params_dict:
            th[:, 0] = torch.as_tensor(np.asarray(params_dict["mass"]["value"], np.float32)[:n], device=self.device)
        for i, key in enumerate(("comx", "comy", "comz")):
            if key in params_dict:
                v = np.asarray(params_dict[key]["value"], np.float64)[:n] - BASE_COM[i]
                th[:, 1 + i] = torch.as_tensor(v.astype(np.float32), device=self.device)
        keys = [k for k in ("inertiax", "inertiay", "inertiaz") if k in params_dict]
        if keys:
            ratios = np.stack([np.asarray(params_dict[k]["value"], np.float64)[:n] / BASE_INERTIA["xyz".index(k[-1])]
                               for k in keys])
            if not np.allclose(ratios, ratios[0], rtol=1e-6):
                raise NotImplementedError("independent inertia-diagonal entries: the engine identifies one "
                                          "diagonal scale (theta slot 4)")
            th[:, 4] = torch.as_tensor(ratios[0].astype(np.float32), device=self.device)
        self.theta = th

    # --- stepping ---------------------------------------------------------------------------
    def step(self, actions, control_steps: int = 1):
        a = torch.as_tensor(actions, dtype=torch.float32, device=self.device)
        a = a.reshape(self.num_envs, control_steps, 12).contiguous()
        _lib.check(self.engine.lib.spi_step_states(self.engine._h, self.state.data_ptr(), a.data_ptr(),
                                                   self.theta.contiguous().data_ptr(), self.num_envs,
                                                   int(control_steps)))
        self._last_actions = a      # alive until the kernel ran
