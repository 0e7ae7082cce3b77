"""Device cross-entropy method over theta (spi_cem_* of the C ABI).

The counterpart of the reference's Optuna loops (scripts/mass_opt.py:203-219,
TPE over one base-mass scale; scripts/mass_landscape.py:153, a 20-point grid):
here a population of N theta vectors over up to 13 parameters is sampled,
evaluated against every window and refit on the device each iteration.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .robot import THETA_DIM


class SpiCemConfig(ctypes.Structure):
    _fields_ = [
        ("n_samples", ctypes.c_int32), ("dim", ctypes.c_int32),
        ("param_ids", ctypes.c_int32 * THETA_DIM), ("nominal", ctypes.c_float * THETA_DIM),
        ("lo", ctypes.c_double * THETA_DIM), ("hi", ctypes.c_double * THETA_DIM),
        ("elite_frac", ctypes.c_double), ("alpha", ctypes.c_double), ("min_std_frac", ctypes.c_double),
        ("seed", ctypes.c_uint64), ("job_id", ctypes.c_int32),
    ]


_API = {
    "spi_cem_init": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(SpiCemConfig)]),
    "spi_cem_sample": (ctypes.c_int, [ctypes.c_void_p]),
    "spi_cem_refit": (ctypes.c_int, [ctypes.c_void_p]),
    "spi_cem_step": (ctypes.c_int, [ctypes.c_void_p]),
    "spi_cem_run": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    "spi_cem_read": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.c_void_p, ctypes.c_void_p]),
}


def _bind(lib):
    for name, (res, args) in _API.items():
        fn = getattr(lib, name)
        fn.restype, fn.argtypes = res, args
    return lib


class CEM:
    """CEM identification of ``param_ids`` (theta slots) on an engine with loaded windows."""

    launches_per_step = 5   # sample, rollout-table fill, rollout, cost finalize, refit

    def __init__(self, engine, n_samples, param_ids, lo, hi, nominal, elite_frac=0.1, alpha=1.0,
                 min_std_frac=1e-3, seed=0, job_id=0):
        self.engine = engine
        self.lib = _bind(_lib.engine_lib())
        self.param_ids = list(param_ids)
        P = len(self.param_ids)
        lo, hi = np.asarray(lo, np.float64), np.asarray(hi, np.float64)
        if lo.shape[0] == THETA_DIM and P < THETA_DIM:
            lo, hi = lo[self.param_ids], hi[self.param_ids]
        c = SpiCemConfig()
        c.n_samples, c.dim = int(n_samples), P
        for d, s in enumerate(self.param_ids):
            c.param_ids[d] = s
            c.lo[d], c.hi[d] = float(lo[d]), float(hi[d])
        c.nominal[:] = tuple(float(v) for v in np.asarray(nominal, np.float64))
        c.elite_frac, c.alpha, c.min_std_frac = elite_frac, alpha, min_std_frac
        c.seed, c.job_id = int(seed), int(job_id)
        self.cfg = c
        self.lo, self.hi = lo, hi
        _lib.check(self.lib.spi_cem_init(engine._h, ctypes.byref(c)))
        engine.N = int(n_samples)

    def step(self, rollout_events=None):
        """One iteration: sample, roll every (theta, window), refit. Events bracket the rollout."""
        h = self.engine._h
        _lib.check(self.lib.spi_cem_sample(h))
        if rollout_events:
            rollout_events[0].record(self.engine.stream)
        _lib.check(self.engine.lib.spi_run(h))
        if rollout_events:
            rollout_events[1].record(self.engine.stream)
        _lib.check(self.lib.spi_cem_refit(h))

    def sample(self):
        _lib.check(self.lib.spi_cem_sample(self.engine._h))

    def refit(self):
        _lib.check(self.lib.spi_cem_refit(self.engine._h))

    def run(self, iterations, graph=True):
        _lib.check(self.lib.spi_cem_run(self.engine._h, int(iterations), int(bool(graph))))

    def read(self):
        P = len(self.param_ids)
        mu = np.zeros(P)
        cov = np.zeros((P, P))
        best = np.zeros(THETA_DIM, dtype=np.float32)
        bc = ctypes.c_float()
        it = ctypes.c_int32()
        _lib.check(self.lib.spi_cem_read(self.engine._h, mu.ctypes.data, cov.ctypes.data, best.ctypes.data,
                                         ctypes.addressof(bc), ctypes.addressof(it)))
        return {"mu": mu, "cov": cov, "best_theta": best, "best_cost": float(bc.value), "iteration": int(it.value)}

    def theta(self):
        """The current population [N, 13] (the engine's theta batch)."""
        e = self.engine
        out = torch.empty((e.N, THETA_DIM), device=e.device)
        _lib.check(e.lib.spi_read_theta(e._h, out.data_ptr()))
        return out

    def best_cost(self):
        return self.read()["best_cost"]

    def theta_error(self, theta_true):
        """Largest |mean - truth| over the identified parameters, in units of each prior range."""
        return float(np.max(self.theta_errors(theta_true)["err_frac"]))

    def theta_errors(self, theta_true):
        """Per identified parameter: truth, distribution mean, |mean - truth| and the
        distribution's std, the last two in units of the parameter's prior range (hi - lo)."""
        r = self.read()
        est = np.array(r["mu"])
        true = np.asarray(theta_true, np.float64)[self.param_ids]
        rng = self.hi - self.lo
        return {"true": true, "est": est, "err_frac": np.abs(est - true) / rng,
                "std_frac": np.sqrt(np.maximum(np.diag(r["cov"]), 0.0)) / rng}

    def sample_host(self, k):
        """k host-side uniform prior populations (for end-to-end host-buffer timing)."""
        rng = np.random.default_rng(int(self.cfg.seed) + 99)
        P = len(self.param_ids)
        th = np.tile(np.array(self.cfg.nominal[:], np.float32), (k, self.cfg.n_samples, 1))
        u = rng.random((k, self.cfg.n_samples, P))
        th[..., self.param_ids] = (self.lo + (self.hi - self.lo) * u).astype(np.float32)
        return th
