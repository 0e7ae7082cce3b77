"""Algorithmic FP operation count of the rollout, from an instrumented host build of the kernel source."""
from __future__ import annotations

import ctypes
from functools import lru_cache

import numpy as np

from . import _lib
from .data import standing_state
from .robot import SimConfig, THETA_NOMINAL, to_struct


@lru_cache(maxsize=8)
def _count(cfg_key):
    cfg = SimConfig(**dict(cfg_key))
    r = to_struct(cfg)
    x = np.ascontiguousarray(standing_state(1)[0], dtype=np.float64)
    th = np.ascontiguousarray(THETA_NOMINAL, dtype=np.float64)
    a = np.zeros(12, dtype=np.float64)
    n1, n2 = ctypes.c_longlong(), ctypes.c_longlong()
    rc = _lib.hostemu_lib().spi_hostemu_count_ops(ctypes.byref(r), x.ctypes.data, th.ctypes.data,
                                                  a.ctypes.data, ctypes.byref(n1), ctypes.byref(n2))
    if rc:
        raise _lib.SpiError(rc, "flop count failed")
    return n1.value, n2.value


def flops_per_substep(cfg: SimConfig) -> int:
    return _count(tuple(sorted(cfg.__dict__.items())))[0]


def flops_per_rollout_step(cfg: SimConfig) -> int:
    """One rollout-step = one control step = ``decimation`` physics substeps of one (theta, window)."""
    return cfg.decimation * flops_per_substep(cfg)
