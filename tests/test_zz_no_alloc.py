"""spi_eval_windows_noalloc: the evaluation entry point that allocates no device memory.

It exists for callers that must not let a library call cudaMalloc: a serving process that
reserves its whole HBM budget at start-up, a host framework that owns every device
allocation, or a loop where cudaMalloc's implicit device synchronisation would stall other
streams. These tests call it through the C ABI with caller-owned buffers and check it
against the engine path (spi_load_windows + spi_set_theta + spi_run + spi_read_costs) on
two calls in a row, with the same 1e-4 tolerance the other parity tests use; once with every
optional argument left out (no weights, default squared-error weights, norm <= 0, no comp);
and against the FP64 oracle's rollout and cost. This file is collected last so that a
failing run that stops at the first failure has run everything else.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

TOL = 1e-4


def _rel_err(gpu, ref):
    gpu = np.asarray(gpu, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    scale = np.maximum(np.abs(ref), 1e-3 * np.abs(ref).max())
    return float(np.max(np.abs(gpu - ref) / scale))


def _windows(seed, W, H):
    """Seeded windows: standing states with small random motion and random actions."""
    rng = np.random.default_rng(seed)
    from spi_gb300.data import standing_state
    init = np.repeat(standing_state(1, z=0.31), W, 0)
    init[:, 7:13] += 0.2 * rng.standard_normal((W, 6)).astype(np.float32)
    init[:, 25:37] += rng.standard_normal((W, 12)).astype(np.float32)
    actions = (0.8 * rng.standard_normal((W, H, 12))).astype(np.float32)
    target = init + 0.01 * rng.standard_normal(init.shape).astype(np.float32)
    weight = (rng.random(W) > 0.2).astype(np.float32)
    return init, actions, target, weight


def _theta(seed, N):
    from spi_gb300.robot import THETA_PRIOR_HI, THETA_PRIOR_LO
    rng = np.random.default_rng(seed)
    return (THETA_PRIOR_LO + (THETA_PRIOR_HI - THETA_PRIOR_LO) * rng.random((N, 13))).astype(np.float32)


def _noalloc(lib, robot, dev_in, theta, W, H, norm, mode):
    init, actions, target, weight = dev_in
    N = theta.shape[0]
    comp = torch.full((N, 9), float("nan"), device="cuda")
    cost = torch.full((N,), float("nan"), device="cuda")
    w = (ctypes.c_float * 6)(10.0, 5.0, 0.1, 0.1, 1.0, 0.01)
    rc = lib.spi_eval_windows_noalloc(ctypes.byref(robot), init.data_ptr(), actions.data_ptr(),
                                      target.data_ptr(), weight.data_ptr(), W, H, float(norm),
                                      theta.data_ptr(), N, mode, w, comp.data_ptr(), cost.data_ptr(),
                                      ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0, lib.spi_last_error()
    return comp, cost


def test_noalloc_matches_engine_two_calls_in_a_row():
    import __graft_entry__
    __graft_entry__.build()
    from spi_gb300 import _lib, robot as rb
    from spi_gb300.engine import COST_REF, COST_SQ, Engine
    lib = _lib.engine_lib()
    cfg = rb.SimConfig()
    robot = rb.to_struct(cfg)
    W, H = 29, 6                        # W not a multiple of the 8-window group
    host = _windows(3, W, H)
    dev_in = [torch.from_numpy(a).cuda() for a in host]
    norm = float(host[3].sum())
    eng = Engine(cfg)
    eng.load_windows(dev_in[0], dev_in[1], dev_in[2], dev_in[3], norm=norm)
    for call, (seed, N, mode) in enumerate(((5, 37, 1), (6, 64, 0))):
        theta = torch.from_numpy(_theta(seed, N)).cuda()
        eng.set_cost(COST_SQ if mode == 1 else COST_REF)
        ref_comp, ref_cost = eng.evaluate(theta)
        comp, cost = _noalloc(lib, robot, dev_in, theta, W, H, norm, mode)
        torch.cuda.synchronize()
        assert torch.isfinite(comp).all() and torch.isfinite(cost).all(), f"call {call}"
        assert _rel_err(comp.cpu(), ref_comp.cpu()) <= TOL, f"call {call}"
        assert _rel_err(cost.cpu(), ref_cost.cpu()) <= TOL, f"call {call}"


def test_noalloc_rejects_sizes_beyond_its_scratch():
    from spi_gb300 import _lib, robot as rb
    lib = _lib.engine_lib()
    robot = rb.to_struct(rb.SimConfig())
    W, H = 16, 2
    dev_in = [torch.from_numpy(a).cuda() for a in _windows(4, W, H)]
    N = 65536 // 2 + 1                   # ceil(16 / 8) = 2 groups per theta: one slot too many
    theta = torch.zeros((N, 13), device="cuda")
    comp = torch.empty((N, 9), device="cuda")
    rc = lib.spi_eval_windows_noalloc(ctypes.byref(robot), dev_in[0].data_ptr(), dev_in[1].data_ptr(),
                                      dev_in[2].data_ptr(), None, W, H, 0.0, theta.data_ptr(), N, 1, None,
                                      comp.data_ptr(), None, None)
    assert rc == -1
    assert b"exceeds the fixed scratch" in lib.spi_last_error()


def test_noalloc_optional_arguments_left_out():
    """weight NULL (all 1), sq_weights NULL (built-in defaults), norm 0 (divide by W), comp NULL."""
    from spi_gb300 import _lib, robot as rb
    from spi_gb300.engine import COST_SQ, Engine
    lib = _lib.engine_lib()
    cfg = rb.SimConfig()
    robot = rb.to_struct(cfg)
    W, H, N = 21, 4, 19
    host = _windows(8, W, H)
    dev_in = [torch.from_numpy(a).cuda() for a in host[:3]]
    eng = Engine(cfg)
    eng.load_windows(dev_in[0], dev_in[1], dev_in[2], None, norm=None)
    eng.set_cost(COST_SQ)
    theta = torch.from_numpy(_theta(9, N)).cuda()
    _, ref_cost = eng.evaluate(theta)
    cost = torch.full((N,), float("nan"), device="cuda")
    rc = lib.spi_eval_windows_noalloc(ctypes.byref(robot), dev_in[0].data_ptr(), dev_in[1].data_ptr(),
                                      dev_in[2].data_ptr(), None, W, H, 0.0, theta.data_ptr(), N, 1, None,
                                      None, cost.data_ptr(), None)
    assert rc == 0, lib.spi_last_error()
    torch.cuda.synchronize()
    assert torch.isfinite(cost).all()
    assert _rel_err(cost.cpu(), ref_cost.cpu()) <= TOL


def test_noalloc_matches_fp64_oracle():
    """Rollout and weighted cost against the FP64 oracle on the same windows and theta."""
    from oracle import cost as oc
    from oracle import dynamics as dyn
    from oracle import go2_model as gm
    from spi_gb300 import _lib, robot as rb
    lib = _lib.engine_lib()
    robot = rb.to_struct(rb.SimConfig())
    W, H, N = 13, 5, 6
    init, actions, target, weight = _windows(11, W, H)
    norm = float(weight.sum())
    dev_in = [torch.from_numpy(a).cuda() for a in (init, actions, target, weight)]
    theta = torch.from_numpy(_theta(12, N)).cuda()
    for mode in (1, 0):
        comp, cost = _noalloc(lib, robot, dev_in, theta, W, H, norm, mode)
        torch.cuda.synchronize()
        th = theta.cpu().numpy().astype(np.float64)
        fin = dyn.rollout(np.tile(init.astype(np.float64), (N, 1)), np.tile(actions.astype(np.float64), (N, 1, 1)),
                          np.repeat(th, W, 0), gm.SimParams())
        wc = oc.window_components(fin, np.tile(target.astype(np.float64), (N, 1))).reshape(N, W, oc.N_COMP)
        ref_comp = oc.reduce_components(wc, weight, norm)
        ref_cost = oc.scalar_cost(ref_comp, mode="sq" if mode == 1 else "ref")
        assert _rel_err(comp.cpu(), ref_comp) <= TOL, mode
        assert _rel_err(cost.cpu(), ref_cost) <= TOL, mode
