"""FP operation counts of the rollout, from instrumented host builds of the dynamics source.

Two counts per physics substep (one rollout, each +, -, *, /, sqrt, tanh, sin, cos once; the
base solve once):

* ``algorithmic``: the oracle's equations -- the legs by Featherstone's articulated-body
  algorithm (``csrc/aba_reference.h``). This is the roofline's per-unit figure, fixed by the
  formulation, not by how the kernel evaluates it.
* ``executed``: the kernel's own formulation (``csrc/dynamics.cuh``: each leg condensed through
  its joint-space inertia), which reaches the same result in fewer operations.
* ``dual``: the kernel's formulation on the forward-mode dual scalar (value + one tangent, as
  ``csrc/dual.cuh`` evaluates each operation): the work of one sensitivity direction.
"""
from __future__ import annotations

import ctypes
from functools import lru_cache

import numpy as np

from . import _lib
from .data import standing_state
from .robot import SimConfig, THETA_NOMINAL, to_struct


@lru_cache(maxsize=16)
def _count(cfg_key, aba):
    cfg = SimConfig(**dict(cfg_key))
    r = to_struct(cfg)
    x = np.ascontiguousarray(standing_state(1)[0], dtype=np.float64)
    th = np.ascontiguousarray(THETA_NOMINAL, dtype=np.float64)
    a = np.zeros(12, dtype=np.float64)
    n1, n2 = ctypes.c_longlong(), ctypes.c_longlong()
    lib = _lib.hostemu_lib()
    fn = lib.spi_hostemu_count_ops_aba if aba else lib.spi_hostemu_count_ops
    rc = fn(ctypes.byref(r), x.ctypes.data, th.ctypes.data, a.ctypes.data, ctypes.byref(n1), ctypes.byref(n2))
    if rc:
        raise _lib.SpiError(rc, "flop count failed")
    return n1.value, n2.value


def _key(cfg):
    return tuple(sorted(cfg.__dict__.items()))


def flops_per_substep(cfg: SimConfig) -> int:
    """Algorithmic FP operations of one physics substep (the articulated-body formulation)."""
    return _count(_key(cfg), True)[0]


def executed_flops_per_substep(cfg: SimConfig) -> int:
    """FP operations the kernel's formulation performs in one physics substep."""
    return _count(_key(cfg), False)[0]


def flops_per_rollout_step(cfg: SimConfig) -> int:
    """One rollout-step = one control step = ``decimation`` physics substeps of one (theta, window)."""
    return cfg.decimation * flops_per_substep(cfg)


def executed_flops_per_rollout_step(cfg: SimConfig) -> int:
    return cfg.decimation * executed_flops_per_substep(cfg)


@lru_cache(maxsize=16)
def _count_dual(cfg_key):
    cfg = SimConfig(**dict(cfg_key))
    r = to_struct(cfg)
    x = np.ascontiguousarray(standing_state(1)[0], dtype=np.float64)
    th = np.ascontiguousarray(THETA_NOMINAL, dtype=np.float64)
    a = np.zeros(12, dtype=np.float64)
    n = ctypes.c_longlong()
    rc = _lib.hostemu_lib().spi_hostemu_count_ops_dual(ctypes.byref(r), x.ctypes.data, th.ctypes.data,
                                                       a.ctypes.data, ctypes.byref(n))
    if rc:
        raise _lib.SpiError(rc, "dual flop count failed")
    return n.value


def dual_flops_per_rollout_step(cfg: SimConfig) -> int:
    """FP operations of one control step of one sensitivity direction (dual scalar, phase B once)."""
    return cfg.decimation * _count_dual(_key(cfg))
