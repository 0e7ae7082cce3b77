"""State sensitivities, Fisher information and excitation scoring (spi_sensitivity / spi_fisher).

Gradients of the windowed cost in theta come from the hand-written adjoint of the rollout
(``adjoint``, ``WindowCost``); per-window Jacobians from forward-mode derivatives.

The reference scores candidate excitations with a finite-difference Fisher proxy:
main and auxiliary envs with theta + 0.1 (spigym/envs/sysid/active_sysid_openloop.py:29-80,
402-426) and trace(J^T J) as the objective. Here J_w = d s_H / d theta comes from forward-mode
derivatives of the rollout on the GPU, and a candidate is scored by log det of
F = sum_w J_w^T Q J_w (D-optimal; trace is reported as well).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .data import standing_state
from .robot import STATE_DIM, THETA_DIM


def sensitivities(engine, theta, param_ids):
    """J [N, W, 37, K] and final states xH [N, W, 37] for the engine's loaded windows."""
    theta = torch.as_tensor(theta, dtype=torch.float32, device=engine.device).contiguous()
    ids = (ctypes.c_int32 * len(param_ids))(*[int(i) for i in param_ids])
    N, K = theta.shape[0], len(param_ids)
    J = torch.empty((N, engine.W, STATE_DIM, K), device=engine.device)
    xH = torch.empty((N, engine.W, STATE_DIM), device=engine.device)
    _lib.check(engine.lib.spi_sensitivity(engine._h, theta.data_ptr(), N, ids, K, J.data_ptr(), xH.data_ptr()))
    return J, xH


def fisher(J, state_weight=None, eps=1e-9, stream=None, tensor_cores=False):
    """F [N, K, K], log det(F + eps I) and trace(F) (FP64) from J [N, W, 37, K].

    tensor_cores: accumulate J^T Q J on the tensor cores (BF16 operands, FP32 accumulation)
    instead of FP32 on the CUDA cores."""
    J = J.contiguous()
    N, W, S, K = J.shape
    F = torch.empty((N, K, K), device=J.device)
    logdet = torch.empty((N,), device=J.device, dtype=torch.float64)
    trace = torch.empty((N,), device=J.device, dtype=torch.float64)
    q = None
    if state_weight is not None:
        q = torch.as_tensor(state_weight, dtype=torch.float32, device=J.device).contiguous()
    s = stream or torch.cuda.current_stream(J.device)
    _lib.check(_lib.engine_lib().spi_fisher_ex(J.data_ptr(), N, W, K, q.data_ptr() if q is not None else None,
                                               float(eps), int(bool(tensor_cores)), F.data_ptr(), logdet.data_ptr(),
                                               trace.data_ptr(), ctypes.c_void_p(s.cuda_stream)))
    return F, logdet, trace


def block_weights(sq_weights):
    """Per-state-component weights [37] from the six block weights (pos, quat, linvel, angvel, q, qd)."""
    sizes = (3, 4, 3, 3, 12, 12)
    return np.concatenate([np.full(n, w, np.float32) for n, w in zip(sizes, sq_weights)])


def adjoint(engine, theta):
    """(cost [N], d cost / d theta [N, 13]) of the engine's cost by the hand-written adjoint
    (spi_adjoint): one reverse sweep per rollout, checkpoints every 5 control steps."""
    theta = torch.as_tensor(theta, dtype=torch.float32, device=engine.device).reshape(-1, THETA_DIM).contiguous()
    N = theta.shape[0]
    cost = torch.empty((N,), device=engine.device)
    grad = torch.empty((N, THETA_DIM), device=engine.device)
    with torch.cuda.device(engine.device):
        _lib.check(engine.lib.spi_adjoint(engine._h, theta.data_ptr(), N, cost.data_ptr(), grad.data_ptr()))
    engine._adj_keep = theta
    return cost, grad


def tangent_gradient(engine, theta, sq_weights=(10.0, 5.0, 0.1, 0.1, 1.0, 0.01)):
    """The same gradient of the squared-error cost from the 13 forward-mode tangent sweeps
    (d cost / d theta = 2 sum_w diff_w^T Q J_w / W), for comparison with ``adjoint``."""
    J, xH = sensitivities(engine, theta, list(range(THETA_DIM)))
    q = torch.as_tensor(block_weights(sq_weights), device=J.device)
    diff = xH - engine.target[None]
    cost = (q * diff * diff).sum(-1).mean(1)
    return cost, 2.0 * torch.einsum("nwi,i,nwik->nk", diff, q, J) / engine.W


class WindowCost(torch.autograd.Function):
    """The engine's squared-error cost per theta sample, differentiable in theta.

    forward(theta [N,13], engine, sq_weights) -> cost [N] = sum_w weight_w sum_i q_i
    (s_H,i - target_i)^2 / norm over the engine's windows (mean over windows for unit weights),
    from one spi_run; backward runs the hand-written adjoint of the rollout (``adjoint``) for
    d cost / d theta. The per-window Jacobians d s_H / d theta stay with the forward-mode
    ``sensitivities`` (13 directions against 37 outputs).
    """

    @staticmethod
    def forward(ctx, theta, engine, sq_weights):
        from .engine import COST_SQ
        engine.set_cost(COST_SQ, sq_weights)
        th = theta.detach().to(torch.float32).contiguous()
        _, cost = engine.evaluate(th)
        ctx.engine = engine
        ctx.save_for_backward(th)
        return cost.clone()

    @staticmethod
    def backward(ctx, g):
        (th,) = ctx.saved_tensors
        _, grad = adjoint(ctx.engine, th)
        return g[:, None] * grad, None, None


def multisine_actions(n_cand, T, control_dt, action_scale, n_comp=3, amp=(0.05, 0.4), freq=(0.5, 4.0), seed=0,
                      settle=0):
    """Candidate excitations: per joint a sum of n_comp sines (amplitudes in rad of joint target)."""
    rng = np.random.default_rng(seed)
    A = rng.uniform(amp[0], amp[1], (n_cand, 12, n_comp))
    f = rng.uniform(freq[0], freq[1], (n_cand, 12, n_comp))
    ph = rng.uniform(0.0, 2.0 * np.pi, (n_cand, 12, n_comp))
    t = np.arange(T) * control_dt
    s = np.sin(2.0 * np.pi * f[:, None] * t[None, :, None, None] + ph[:, None])      # [n, T, 12, c]
    a = (A[:, None] * s).sum(-1) / action_scale
    if settle:
        a = np.concatenate([np.zeros((n_cand, settle, 12)), a], 1)
    return a.astype(np.float32), dict(amp=A, freq=f, phase=ph)


def score_excitations(engine, theta, actions, windows_per_cand=8, horizon=20, settle=100, param_ids=None,
                      sq_weights=(10.0, 5.0, 0.1, 0.1, 1.0, 0.01), eps=1e-9, tensor_cores=True, timing=None):
    """Fisher scores of candidate excitations at theta.

    actions [n_cand, settle + windows_per_cand * horizon, 12] (host array or device tensor; a
    device tensor stays on the device). Each candidate is rolled from a standing start; windows
    of `horizon` steps start every `horizon` steps after `settle`. Returns dict(logdet [n],
    trace [n], best, F [n,K,K], J). timing: a dict that receives the device time in ms of the
    settle trace, the sensitivities and the Fisher reduction (CUDA events on the engine stream).
    """
    param_ids = list(range(THETA_DIM)) if param_ids is None else list(param_ids)
    dev = engine.device
    acts = torch.as_tensor(actions, dtype=torch.float32, device=dev)
    n, T = int(acts.shape[0]), int(acts.shape[1])
    th = torch.as_tensor(np.asarray(theta, np.float32).reshape(1, THETA_DIM), device=dev)
    x0 = torch.from_numpy(standing_state(n)).to(dev)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)] if timing is not None else None
    if ev:
        ev[0].record(engine.stream)
    engine.load_windows(x0, acts, x0)
    _, _, tr = engine.evaluate(th, trace=True)                                # [1, n, T, 37]
    tr = tr[0]
    starts = settle - 1 + horizon * np.arange(windows_per_cand)               # state index before each window
    init = tr[:, torch.as_tensor(starts, device=dev)].reshape(-1, STATE_DIM)  # [n * wpc, 37]
    steps = torch.as_tensor(starts[:, None] + 1 + np.arange(horizon)[None, :], device=dev)
    act = acts[:, steps].reshape(-1, horizon, 12)                              # [n * wpc, H, 12]
    if ev:
        ev[1].record(engine.stream)
    engine.load_windows(init, act, init)
    J, _ = sensitivities(engine, th, param_ids)                               # [1, n*wpc, 37, K]
    J = J.reshape(n, windows_per_cand, STATE_DIM, len(param_ids))
    if ev:
        ev[2].record(engine.stream)
    F, logdet, trace = fisher(J, block_weights(sq_weights), eps, tensor_cores=tensor_cores)
    if ev:
        ev[3].record(engine.stream)
    ld = logdet.cpu().numpy()
    if ev:
        timing.update(settle_trace_ms=ev[0].elapsed_time(ev[1]), sensitivities_ms=ev[1].elapsed_time(ev[2]),
                      fisher_ms=ev[2].elapsed_time(ev[3]))
    return {"logdet": ld, "trace": trace.cpu().numpy(), "best": int(np.argmax(ld)), "F": F, "J": J}
