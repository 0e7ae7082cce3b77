"""Engine: torch-facing wrapper of the C ABI (include/spi_engine.h).

One engine holds a robot model, a window set and a theta batch on one CUDA
device and stream. ``evaluate(theta)`` is the batched counterpart of the
reference's per-theta ``apply_base_mass`` + ``evaluate_batch``
(scripts/eval.py:204-310): every (theta, window) pair is reset to its logged
state, rolled H control steps and scored in one kernel launch.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib
from .robot import N_COMP, STATE_DIM, THETA_DIM, SimConfig, to_struct

COST_REF = 0   # reference L2 norms, weights 10 / 5 / 1 (scripts/mass_opt.py:28-32)
COST_SQ = 1    # weighted squared error over the six state blocks
DEFAULT_SQ_WEIGHTS = (10.0, 5.0, 0.1, 0.1, 1.0, 0.01)


def _f32(t, shape, name, device):
    if not isinstance(t, torch.Tensor):
        t = torch.as_tensor(t)
    t = t.to(device=device, dtype=torch.float32).contiguous()
    if tuple(t.shape) != tuple(shape):
        raise ValueError(f"{name}: expected shape {tuple(shape)}, got {tuple(t.shape)}")
    return t


class Engine:
    """Batched evaluation of theta samples against logged windows (the C ABI's spi_engine).

    variant: the rollout-kernel variant (see spi_gb300.autotune.VARIANTS). The default, lane3
    (one lane per rollout, a 168-register cap, 3 CTAs per SM), is the fastest on the C1
    workload; spi_gb300.autotune.tune_engine times every variant on the caller's own batch."""

    def __init__(self, cfg: SimConfig | None = None, device=None, stream: torch.cuda.Stream | None = None,
                 variant: str | None = "lane3"):
        if not torch.cuda.is_available():
            raise RuntimeError("spi_gb300.Engine needs a CUDA device (no CPU fallback exists)")
        self.cfg = cfg or SimConfig()
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.lib = _lib.engine_lib()
        self._robot = to_struct(self.cfg)
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(self.lib.spi_create(ctypes.byref(self._robot), ctypes.byref(h)))
        self._h = h
        self.stream = stream or torch.cuda.current_stream(self.device)
        _lib.check(self.lib.spi_set_stream(self._h, ctypes.c_void_p(self.stream.cuda_stream)))
        self.W = self.H = self.N = 0
        self._keep = []
        if variant is not None:
            from .autotune import set_variant
            with torch.cuda.device(self.device):
                set_variant(self, variant)

    def close(self):
        if getattr(self, "_h", None):
            self.lib.spi_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def load_windows(self, init, actions, target, weight=None, norm=None):
        """init / target [W,37] world-frame states, actions [W,H,12] raw actions."""
        W, H = int(actions.shape[0]), int(actions.shape[1])
        init = _f32(init, (W, STATE_DIM), "init", self.device)
        target = _f32(target, (W, STATE_DIM), "target", self.device)
        actions = _f32(actions, (W, H, 12), "actions", self.device)
        wptr = None
        if weight is not None:
            weight = _f32(weight, (W,), "weight", self.device)
            wptr = weight.data_ptr()
        with torch.cuda.stream(self.stream):
            _lib.check(self.lib.spi_load_windows(self._h, init.data_ptr(), actions.data_ptr(), target.data_ptr(),
                                                 wptr, W, H, float(norm) if norm else 0.0))
        self._keep = [init, target, actions, weight]   # alive until the copy kernels ran
        self.W, self.H = W, H
        self.target = target

    def set_theta(self, theta):
        theta = _f32(theta, (int(theta.shape[0]), THETA_DIM), "theta", self.device)
        _lib.check(self.lib.spi_set_theta(self._h, theta.data_ptr(), theta.shape[0]))
        self._theta = theta
        self.N = theta.shape[0]

    def set_cost(self, mode=COST_SQ, sq_weights=DEFAULT_SQ_WEIGHTS):
        w = (ctypes.c_float * 6)(*sq_weights)
        _lib.check(self.lib.spi_set_cost(self._h, int(mode), w))

    def run(self, trace=False):
        if trace:
            tr = torch.empty((self.N, self.W, self.H, STATE_DIM), device=self.device, dtype=torch.float32)
            _lib.check(self.lib.spi_run_trace(self._h, tr.data_ptr()))
            return tr
        _lib.check(self.lib.spi_run(self._h))
        return None

    def read(self, out_comp=None, out_cost=None):
        comp = out_comp if out_comp is not None else torch.empty((self.N, N_COMP), device=self.device)
        cost = out_cost if out_cost is not None else torch.empty((self.N,), device=self.device)
        _lib.check(self.lib.spi_read_costs(self._h, comp.data_ptr(), cost.data_ptr()))
        return comp, cost

    def sync(self) -> int:
        n = ctypes.c_int64()
        _lib.check(self.lib.spi_sync(self._h, ctypes.byref(n)))
        return int(n.value)

    def evaluate(self, theta, trace=False):
        """Mean error components [N,9], scalar cost [N] (and the trace [N,W,H,37])."""
        self.set_theta(theta)
        tr = self.run(trace=trace)
        comp, cost = self.read()
        return (comp, cost, tr) if trace else (comp, cost)


def probe_fp32_peak() -> float:
    v = ctypes.c_double()
    _lib.check(_lib.engine_lib().spi_probe_fp32_peak(ctypes.byref(v)))
    return float(v.value)
