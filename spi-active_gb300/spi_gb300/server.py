"""Continuous-batching identification server (spi_server_* of the C ABI).

Jobs are CEM identifications over their own windows. They are admitted into
slots against an HBM budget and advanced one CEM iteration per tick, all active
jobs in one rollout launch (the same compiled kernel as the single-job engine, so a
job's results equal the engine's bit for bit). Finished jobs free their slot and memory.
"""
from __future__ import annotations

import ctypes
import time

import numpy as np
import torch

from . import _lib
from .cem import SpiCemConfig
from .robot import THETA_DIM, SimConfig, SpiRobot, to_struct


class SpiJob(ctypes.Structure):
    _fields_ = [("init", ctypes.c_void_p), ("actions", ctypes.c_void_p), ("target", ctypes.c_void_p),
                ("weight", ctypes.c_void_p), ("W", ctypes.c_int32), ("H", ctypes.c_int32),
                ("norm", ctypes.c_float), ("iterations", ctypes.c_int32), ("cem", SpiCemConfig)]


class SpiJobResult(ctypes.Structure):
    _fields_ = [("job_id", ctypes.c_int32), ("iterations", ctypes.c_int32), ("best_cost", ctypes.c_float),
                ("best_theta", ctypes.c_float * THETA_DIM), ("mu", ctypes.c_double * THETA_DIM),
                ("dim", ctypes.c_int32), ("status", ctypes.c_int32)]


_API = {
    "spi_server_create": (ctypes.c_int, [ctypes.POINTER(SpiRobot), ctypes.c_int, ctypes.c_int, ctypes.c_size_t,
                                         ctypes.POINTER(ctypes.c_void_p)]),
    "spi_server_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "spi_server_set_stream": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "spi_server_set_cost": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_float)]),
    "spi_server_job_bytes": (ctypes.c_size_t, [ctypes.POINTER(SpiJob)]),
    "spi_server_submit": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(SpiJob), ctypes.POINTER(ctypes.c_int32)]),
    "spi_server_tick": (ctypes.c_int, [ctypes.c_void_p]),
    "spi_server_poll": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(SpiJobResult), ctypes.c_int,
                                       ctypes.POINTER(ctypes.c_int32)]),
    "spi_server_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32),
                                        ctypes.POINTER(ctypes.c_size_t)]),
    "spi_server_config": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    "spi_server_wait": (ctypes.c_int, [ctypes.c_void_p]),
    "spi_server_set_kernel_config": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "spi_server_set_kernel_layout": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "spi_server_set_rounds": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "spi_server_set_work_cap": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_longlong]),
}


def _bind(lib):
    for name, (res, args) in _API.items():
        fn = getattr(lib, name)
        fn.restype, fn.argtypes = res, args
    return lib


def cem_config(n_samples, param_ids, lo, hi, nominal, elite_frac=0.1, alpha=1.0, min_std_frac=1e-3, seed=0,
               job_id=0):
    c = SpiCemConfig()
    c.n_samples, c.dim = int(n_samples), len(param_ids)
    for d, s in enumerate(param_ids):
        c.param_ids[d] = int(s)
        c.lo[d], c.hi[d] = float(lo[d]), float(hi[d])
    c.nominal[:] = tuple(float(v) for v in np.asarray(nominal, np.float64))
    c.elite_frac, c.alpha, c.min_std_frac = elite_frac, alpha, min_std_frac
    c.seed, c.job_id = int(seed), int(job_id)
    return c


class Server:
    def __init__(self, cfg: SimConfig | None = None, max_slots=64, max_samples=4096, hbm_budget_bytes=150 << 30,
                 cost_mode=1, sq_weights=(10.0, 5.0, 0.1, 0.1, 1.0, 0.01), device=None):
        if not torch.cuda.is_available():
            raise RuntimeError("spi_gb300.Server needs a CUDA device")
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.lib = _bind(_lib.engine_lib())
        self._robot = to_struct(cfg or SimConfig())
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(self.lib.spi_server_create(ctypes.byref(self._robot), int(max_slots), int(max_samples),
                                                  int(hbm_budget_bytes), ctypes.byref(h)))
        self._h = h
        self.stream = torch.cuda.current_stream(self.device)
        _lib.check(self.lib.spi_server_set_stream(self._h, ctypes.c_void_p(self.stream.cuda_stream)))
        w = (ctypes.c_float * 6)(*sq_weights)
        _lib.check(self.lib.spi_server_set_cost(self._h, int(cost_mode), w))
        self.max_slots = max_slots
        self.submitted = {}          # job_id -> submit time
        self._keep = {}

    def close(self):
        if getattr(self, "_h", None):
            torch.cuda.synchronize(self.device)
            self.lib.spi_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def config(self, ctas_per_sm=0, items_per_claim=1):
        _lib.check(self.lib.spi_server_config(self._h, int(ctas_per_sm), int(items_per_claim)))

    @staticmethod
    def make_job(init, actions, target, cem, iterations, weight=None, norm=0.0):
        j = SpiJob()
        j.init, j.actions, j.target = init.data_ptr(), actions.data_ptr(), target.data_ptr()
        j.weight = weight.data_ptr() if weight is not None else None
        j.W, j.H = int(actions.shape[0]), int(actions.shape[1])
        j.norm, j.iterations, j.cem = float(norm), int(iterations), cem
        return j

    def job_bytes(self, job):
        return int(self.lib.spi_server_job_bytes(ctypes.byref(job)))

    def submit(self, job) -> int | None:
        """Slot of the admitted job, or None when no slot / budget is free right now."""
        slot = ctypes.c_int32()
        rc = self.lib.spi_server_submit(self._h, ctypes.byref(job), ctypes.byref(slot))
        if rc == -6:
            return None
        _lib.check(rc)
        self.submitted[job.cem.job_id] = time.perf_counter()
        return int(slot.value)

    def tick(self):
        _lib.check(self.lib.spi_server_tick(self._h))

    def poll(self, max_results=None):
        m = max_results or self.max_slots
        buf = (SpiJobResult * m)()
        n = ctypes.c_int32()
        _lib.check(self.lib.spi_server_poll(self._h, buf, m, ctypes.byref(n)))
        now = time.perf_counter()
        out = []
        for i in range(n.value):
            r = buf[i]
            out.append({"job_id": r.job_id, "iterations": r.iterations, "best_cost": r.best_cost,
                        "best_theta": np.array(r.best_theta[:], np.float32), "mu": np.array(r.mu[:r.dim]),
                        "status": r.status, "latency_s": now - self.submitted.pop(r.job_id, now)})
        return out

    def set_kernel_config(self, min_blocks):
        _lib.check(self.lib.spi_server_set_kernel_config(self._h, int(min_blocks)))

    def set_kernel_layout(self, layout):
        """0 = quad layout (4 lanes per rollout), 1 = lane layout (one lane per rollout)."""
        _lib.check(self.lib.spi_server_set_kernel_layout(self._h, int(layout)))

    def set_rounds(self, rounds):
        """CEM-iteration rounds per tick: small jobs take up to this many iterations per tick."""
        _lib.check(self.lib.spi_server_set_rounds(self._h, int(rounds)))

    # rollout-kernel variants the server runs, by the autotuner's names
    VARIANTS = {"quad3": (0, 3), "quad4": (0, 4), "lane2": (1, 2), "lane3": (1, 3), "lane4": (1, 4)}

    def set_variant(self, name):
        layout, min_blocks = self.VARIANTS[name]
        self.set_kernel_layout(layout)
        self.set_kernel_config(min_blocks)

    def set_work_cap(self, max_items):
        _lib.check(self.lib.spi_server_set_work_cap(self._h, int(max_items)))

    def wait(self):
        _lib.check(self.lib.spi_server_wait(self._h))

    def run_until_done(self, expected):
        """Tick until `expected` results were collected; returns them by job id."""
        out = {}
        while len(out) < expected:
            active, _ = self.stats()
            if active:
                self.tick()
            else:
                self.tick()          # retires the jobs that finished on the last tick
                self.wait()
            for r in self.poll():
                out[r["job_id"]] = r
        return out

    def stats(self):
        a, f = ctypes.c_int32(), ctypes.c_size_t()
        _lib.check(self.lib.spi_server_stats(self._h, ctypes.byref(a), ctypes.byref(f)))
        return int(a.value), int(f.value)
