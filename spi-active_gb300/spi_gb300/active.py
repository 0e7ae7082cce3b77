"""Active exploration on the engine: the reference's finite-difference Fisher objective and an
iterative excitation search driven by the device CEM.

* ``fd_fisher`` scores candidate excitations the way the reference's open-loop active-sysid
  env does (spigym/envs/sysid/active_sysid_openloop.py): each candidate runs as a group of one
  main and P auxiliary rollouts, aux k with +delta on parameter k (:29-80); after every control
  step the reward trace(J^T J) of J = (s_main - s_aux) / delta over the root state and joint
  positions is added (:402-426); every ``ksync`` steps the aux rollouts are reset to the main's
  state (:246-252, :316-330). As in the reference, ``reset_all`` first runs one zero-action step
  (spigym/envs/base_task/base_task.py:90-100), after which the aux rollouts take the main's
  state, and the reported objective is the reward sum of the loop steps divided by the loop's
  step counter (spigym/agents/sysid/active_sysid.py:527-600). One fused kernel runs every group
  of every candidate (``spi_fd_fisher``).
* ``excitation_search`` replaces the reference's Optuna ask / tell over command parameters
  (active_sysid.py:165-257, CmaEsSampler) with the device CEM (``spi_search``) over a 12-value
  excitation family (``GroupMultisine``); each iteration samples a population on the device,
  turns it into action sequences on the device, scores them with ``fd_fisher`` (or the exact
  Fisher log det of the forward-mode sensitivities) and refits, and the best objective of every
  iteration is reported.

The reference drives its excitations through a trained locomotion policy, which is not
available here; candidates are open-loop joint-target offsets, as in the multi-sine
excitations of the sensitivity-based scorer (spi_gb300.sensitivity).
"""
from __future__ import annotations

import ctypes
import math

import numpy as np
import torch

from . import _lib
from .cem import SpiCemConfig
from .data import standing_state
from .robot import STATE_DIM, THETA_DIM, THETA_NOMINAL


def fd_fisher(engine, x0, actions, theta, param_ids, delta=0.1, ksync=5, reset_step=True, trace=False):
    """The reference's FD-Fisher objective of each candidate excitation.

    x0 [C, 37] start states, actions [C, n, 12] raw actions, theta [13] or [C, 13] (each group's
    main), param_ids the theta slots of the aux rollouts (P <= 13). Returns the objective [C]
    (reward sum over the n loop steps / (n + 1)) as a device tensor, and with ``trace`` also the
    per-step rewards [C, n].

    ksync: the aux rollouts take the main's state every ksync steps, as the reference's docstrings
    and config describe (`_reset_envs_states_to_main_envs`); ksync < 0 never resyncs. The
    reference writes that resync into the simulator's state-tensor views only, without the
    set_actor_root_state_tensor / set_dof_state_tensor call that pushes them to the simulator,
    and the next refresh overwrites the views; under Isaac Gym its aux envs may therefore never
    be resynced, which is what ksync < 0 reproduces."""
    dev = engine.device
    actions = torch.as_tensor(actions, dtype=torch.float32, device=dev)
    C, n = int(actions.shape[0]), int(actions.shape[1])
    x0 = torch.as_tensor(x0, dtype=torch.float32, device=dev).reshape(C, STATE_DIM).contiguous()
    theta = torch.as_tensor(theta, dtype=torch.float32, device=dev).reshape(-1, THETA_DIM)
    theta = theta.expand(C, THETA_DIM).contiguous()
    skip = 1 if reset_step else 0
    if skip:
        actions = torch.cat([torch.zeros((C, 1, 12), device=dev), actions], 1)
    actions = actions.contiguous()
    T = n + skip
    ids = (ctypes.c_int32 * len(param_ids))(*[int(i) for i in param_ids])
    rsum = torch.empty((C,), device=dev)
    rtr = torch.empty((C, T), device=dev) if trace else None
    with torch.cuda.device(dev):
        _lib.check(engine.lib.spi_fd_fisher(engine._h, x0.data_ptr(), actions.data_ptr(), theta.data_ptr(), C, T,
                                            ids, len(param_ids), float(delta), int(ksync), skip, rsum.data_ptr(),
                                            rtr.data_ptr() if trace else None))
    engine._fd_keep = (x0, actions, theta, ids)   # the last call's inputs stay alive until its kernel ran
    obj = rsum / float(n + 1)
    return (obj, rtr[:, skip:]) if trace else obj


# ----------------------------------------------------------------------------------------
# excitation family searched by the device CEM
# ----------------------------------------------------------------------------------------
class GroupMultisine:
    """Joint-target excitations from 12 numbers: for each of six joint groups (front / rear legs
    x hip / thigh / calf) an amplitude a in [0.05, 0.4] rad and a base frequency f in [0.5, 4] Hz.
    Every joint of a group moves as a * sum_c w_c sin(2 pi f r_c t + phi_jc) with harmonic ratios
    r = (1, 2, 3), weights w = (0.6, 0.3, 0.1) and seeded phases phi, so each joint carries three
    components (the C3 multi-sine shape) and the search stays within the 13 slots the device CEM
    refits. Slot 2 g is group g's amplitude, slot 2 g + 1 its frequency."""

    GROUPS = ((0, 3), (1, 4), (2, 5), (6, 9), (7, 10), (8, 11))
    NAMES = ("front_hip", "front_thigh", "front_calf", "rear_hip", "rear_thigh", "rear_calf")
    AMP = (0.05, 0.4)
    FREQ = (0.5, 4.0)
    RATIOS = (1.0, 2.0, 3.0)
    WEIGHTS = (0.6, 0.3, 0.1)
    dim = 12

    def __init__(self, seed=0):
        self.phase = np.random.default_rng(seed).uniform(0.0, 2.0 * np.pi, (12, 3))
        self.group_of = np.zeros(12, dtype=np.int64)
        for g, joints in enumerate(self.GROUPS):
            self.group_of[list(joints)] = g

    def bounds(self):
        lo = np.array([self.AMP[0], self.FREQ[0]] * 6)
        hi = np.array([self.AMP[1], self.FREQ[1]] * 6)
        return lo, hi

    def actions(self, params, T, control_dt, action_scale):
        """params [N, >= 12] (device or host) -> raw actions [N, T, 12] on params' device."""
        p = torch.as_tensor(params, dtype=torch.float32)
        dev = p.device
        amp = p[:, 0:12:2][:, self.group_of]                        # [N, 12]
        freq = p[:, 1:12:2][:, self.group_of]
        t = torch.arange(T, device=dev, dtype=torch.float32) * control_dt
        ph = torch.as_tensor(self.phase, dtype=torch.float32, device=dev)
        out = torch.zeros((p.shape[0], T, 12), device=dev)
        for c, (r, w) in enumerate(zip(self.RATIOS, self.WEIGHTS)):
            arg = 2.0 * math.pi * r * freq[:, None, :] * t[None, :, None] + ph[None, None, :, c]
            out += w * torch.sin(arg)
        return out * (amp[:, None, :] / action_scale)


class DeviceSearch:
    """The device CEM over a caller-scored population (spi_search_* of the C ABI)."""

    def __init__(self, n_samples, lo, hi, elite_frac=0.1, alpha=0.7, min_std_frac=0.02, seed=0, stream=None):
        self.lib = _lib.engine_lib()
        lo, hi = np.asarray(lo, np.float64), np.asarray(hi, np.float64)
        P = lo.shape[0]
        c = SpiCemConfig()
        c.n_samples, c.dim = int(n_samples), P
        for d in range(P):
            c.param_ids[d] = d
            c.lo[d], c.hi[d] = float(lo[d]), float(hi[d])
        c.elite_frac, c.alpha, c.min_std_frac = elite_frac, alpha, min_std_frac
        c.seed, c.job_id = int(seed), 0
        self.n, self.P = int(n_samples), P
        self.stream = stream or torch.cuda.current_stream()
        h = ctypes.c_void_p()
        _lib.check(self.lib.spi_search_create(ctypes.byref(c), ctypes.c_void_p(self.stream.cuda_stream),
                                              ctypes.byref(h)))
        self._h = h

    def sample(self) -> torch.Tensor:
        """The next population [n, 13] (a view of the search's own device buffer)."""
        ptr = ctypes.c_void_p()
        _lib.check(self.lib.spi_search_sample(self._h, ctypes.byref(ptr)))
        return _device_view(ptr.value, (self.n, THETA_DIM))

    def refit(self, cost: torch.Tensor):
        cost = cost.to(torch.float32).contiguous()
        _lib.check(self.lib.spi_search_refit(self._h, cost.data_ptr()))
        self._cost = cost

    def read(self):
        mu = np.zeros(self.P)
        cov = np.zeros((self.P, self.P))
        best = np.zeros(THETA_DIM, dtype=np.float32)
        bc = ctypes.c_float()
        it = ctypes.c_int32()
        _lib.check(self.lib.spi_search_read(self._h, mu.ctypes.data, cov.ctypes.data, best.ctypes.data,
                                            ctypes.addressof(bc), ctypes.addressof(it)))
        return {"mu": mu, "cov": cov, "best": best, "best_cost": float(bc.value), "iteration": int(it.value)}

    def close(self):
        if getattr(self, "_h", None):
            self.lib.spi_search_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _device_view(ptr, shape):
    """A float32 tensor over device memory the engine owns (valid while its owner lives)."""
    numel = int(np.prod(shape))

    class _Cuda:
        __cuda_array_interface__ = {"shape": tuple(shape), "typestr": "<f4", "data": (int(ptr), False),
                                    "version": 2, "strides": None}
    t = torch.as_tensor(_Cuda(), device="cuda")
    assert t.numel() == numel
    return t


def excitation_search(engine, theta=THETA_NOMINAL, n_candidates=256, iterations=8, steps=200, param_ids=(0,),
                      delta=0.1, ksync=5, objective="fd_fisher", family=None, seed=0, base_height=0.32):
    """Search the excitation family for the candidate that maximises the identification objective.

    objective "fd_fisher": the reference's FD-Fisher reward (``fd_fisher``) of ``param_ids``;
    "logdet": log det of the exact Fisher information of the final states of 8 windows of
    steps / 8 control steps (forward-mode sensitivities). Every iteration samples a population on
    the device, scores it and refits; returns the best parameters and objective and, per
    iteration, the population's best and mean objective."""
    fam = family or GroupMultisine(seed)
    lo, hi = fam.bounds()
    search = DeviceSearch(n_candidates, lo, hi, seed=seed + 1, stream=engine.stream)
    cfg = engine.cfg
    x0 = torch.from_numpy(np.repeat(standing_state(1, z=base_height), n_candidates, 0)).to(engine.device)
    best_val, best_params = -math.inf, None
    per_iter = []
    stats = []
    with torch.cuda.stream(engine.stream):
        for _ in range(iterations):
            pop = search.sample()
            acts = fam.actions(pop[:, :fam.dim], steps, cfg.control_dt, cfg.action_scale)
            if objective == "fd_fisher":
                score = fd_fisher(engine, x0, acts, theta, param_ids, delta=delta, ksync=ksync)
            elif objective == "logdet":
                score = _logdet_objective(engine, x0, acts, theta, param_ids)
            else:
                raise ValueError(f"unknown objective {objective!r}")
            score = torch.nan_to_num(score, nan=-math.inf)
            k = torch.argmax(score)
            fin = torch.isfinite(score)
            mean = torch.where(fin, score, torch.zeros_like(score)).sum() / fin.sum().clamp(min=1)
            stats.append((score.max(), mean, pop[k, :fam.dim].clone()))
            search.refit(-score)
        for mx, mean, p in stats:
            v = float(mx)
            per_iter.append({"best": v, "mean": float(mean)})
            if v > best_val:
                best_val, best_params = v, p.cpu().numpy()
    out = {"best_objective": best_val, "best_params": best_params, "per_iteration": per_iter,
           "objective": objective, "param_ids": list(param_ids), "family": fam}
    search.close()
    return out


def _logdet_objective(engine, x0, actions, theta, param_ids, windows=8):
    """log det(F + eps I) of the forward-mode Fisher information of `windows` consecutive windows
    of each candidate's excitation (the scorer of spi_gb300.sensitivity, on these candidates)."""
    from .sensitivity import block_weights, fisher, sensitivities
    C, T = actions.shape[:2]
    H = T // windows
    engine.load_windows(x0, actions, x0)
    _, _, tr = engine.evaluate(torch.as_tensor(np.asarray(theta, np.float32)).reshape(1, -1), trace=True)
    tr = tr[0]                                                    # [C, T, 37]
    starts = [w * H for w in range(windows)]
    init = torch.stack([x0 if s == 0 else tr[:, s - 1] for s in starts], 1).reshape(-1, STATE_DIM)
    act = torch.stack([actions[:, s:s + H] for s in starts], 1).reshape(-1, H, 12)
    engine.load_windows(init, act, init)
    J, _ = sensitivities(engine, torch.as_tensor(np.asarray(theta, np.float32)).reshape(1, -1), list(param_ids))
    J = J.reshape(C, windows, STATE_DIM, len(param_ids))
    _, logdet, _ = fisher(J, block_weights((10.0, 5.0, 0.1, 0.1, 1.0, 0.01)), 1e-9)
    return logdet.to(torch.float32)
