"""CUDA rollout kernel (through the C ABI) against the FP64 oracle.

Tolerances: states <= 1e-4 relative (|gpu - ref| / max(|ref|, 1)) at every control
step over H = 20; window error components and costs <= 1e-4 relative to the oracle
cost scale (see ``cost_error``).
"""
import numpy as np
import pytest
import torch

from oracle import cost as oc
from oracle import dynamics as dyn
from oracle import go2_model as gm
from oracle import sysid as osy
from helpers import oracle_windows, random_theta, state_error

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def engine_mod(built):
    from spi_gb300.engine import Engine
    return Engine


def _engine(Engine, init, actions, target, weight=None, norm=None, cfg=None):
    e = Engine(cfg)
    e.load_windows(torch.from_numpy(init), torch.from_numpy(actions), torch.from_numpy(target),
                   None if weight is None else torch.from_numpy(np.asarray(weight, np.float32)), norm)
    return e


def cost_error(gpu, ref):
    """Relative error of a vector of costs / components against its own scale."""
    gpu = np.asarray(gpu, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    scale = np.maximum(np.abs(ref), 1e-3 * np.abs(ref).max())
    return float(np.max(np.abs(gpu - ref) / scale))


def test_trace_matches_oracle_every_step_h20(engine_mod):
    """64 theta x 8 windows x H = 20: every state at every control step <= 1e-4."""
    rng = np.random.default_rng(100)
    ds, init, actions, target = oracle_windows(1, n_traj=2, T=24, H=20)
    sel = rng.choice(init.shape[0], 8, replace=False)
    init, actions, target = init[sel], actions[sel], target[sel]
    th = random_theta(rng, 64).astype(np.float32)
    e = _engine(engine_mod, init, actions, target)
    comp, cost, tr = e.evaluate(torch.from_numpy(th), trace=True)
    torch.cuda.synchronize()
    assert e.sync() == 0
    N, W, H = 64, 8, 20
    x0 = np.tile(init.astype(np.float64), (N, 1))
    ref = dyn.rollout(x0, np.tile(actions.astype(np.float64), (N, 1, 1)),
                      np.repeat(th.astype(np.float64), W, 0), gm.SimParams(), trace=True)
    gpu = tr.cpu().numpy().reshape(N * W, H, 37)
    err = state_error(gpu, ref)
    assert err <= 1e-4, err
    # costs: components from the oracle's final states
    refc = oc.window_components(ref[:, -1], np.tile(target.astype(np.float64), (N, 1))).reshape(N, W, 9).mean(1)
    assert cost_error(comp.cpu().numpy(), refc) <= 1e-4
    assert cost_error(cost.cpu().numpy(), oc.scalar_cost(refc)) <= 1e-4


def test_reference_cost_mode_and_mask(engine_mod):
    """Reference L2 cost with the per-chunk mask and the non-end normaliser."""
    from oracle import windows as ow
    ds, init, actions, target = oracle_windows(2, n_traj=3, T=14, H=5, causal=False)
    W = init.shape[0]
    mask = ow.eval_mask(ds["motion_ends"], 16)
    n_valid = ow.total_valid(ds["motion_ends"])
    rng = np.random.default_rng(3)
    th = random_theta(rng, 16).astype(np.float32)
    e = _engine(engine_mod, init, actions, target, weight=mask, norm=n_valid)
    from spi_gb300.engine import COST_REF
    e.set_cost(COST_REF)
    comp, cost = e.evaluate(torch.from_numpy(th))
    ref = osy.window_components(ds, th.astype(np.float64), gm.SimParams())
    refm = oc.reduce_components(ref, mask, n_valid)
    assert cost_error(comp.cpu().numpy(), refm) <= 1e-4
    assert cost_error(cost.cpu().numpy(), oc.compute_cost(refm[:, :3])) <= 1e-4


@pytest.mark.parametrize("W,H,N", [(1, 1, 1), (13, 3, 5), (8, 7, 3), (33, 2, 9)])
def test_ragged_sizes(engine_mod, W, H, N):
    """Window counts that are not multiples of the 8-window warp group, H = 1, N = 1."""
    rng = np.random.default_rng(W * 100 + H)
    ds, init, actions, target = oracle_windows(W, n_traj=1, T=W + H, H=H)
    init, actions, target = init[:W], actions[:W], target[:W]
    th = random_theta(rng, N).astype(np.float32)
    e = _engine(engine_mod, init, actions, target)
    comp, cost, tr = e.evaluate(torch.from_numpy(th), trace=True)
    ref = dyn.rollout(np.tile(init.astype(np.float64), (N, 1)), np.tile(actions.astype(np.float64), (N, 1, 1)),
                      np.repeat(th.astype(np.float64), W, 0), gm.SimParams(), trace=True)
    assert state_error(tr.cpu().numpy().reshape(N * W, H, 37), ref) <= 1e-4
    refc = oc.window_components(ref[:, -1], np.tile(target.astype(np.float64), (N, 1))).reshape(N, W, 9).mean(1)
    assert cost_error(comp.cpu().numpy(), refc) <= 1e-4


def test_deterministic_and_permutation_consistent(engine_mod):
    """Bitwise-identical reruns; permuting theta rows permutes costs bitwise."""
    rng = np.random.default_rng(7)
    ds, init, actions, target = oracle_windows(3, n_traj=2, T=40, H=10)
    th = torch.from_numpy(random_theta(rng, 96).astype(np.float32))
    e = _engine(engine_mod, init, actions, target)
    c1 = e.evaluate(th)[1].clone()
    c2 = e.evaluate(th)[1].clone()
    perm = torch.from_numpy(rng.permutation(96))
    c3 = e.evaluate(th[perm])[1].clone()
    assert torch.equal(c1, c2)
    assert torch.equal(c1[perm.to(c1.device)], c3)


def test_nonfinite_theta_is_counted_not_fatal(engine_mod):
    ds, init, actions, target = oracle_windows(4, n_traj=1, T=12, H=4)
    th = np.tile(gm.THETA_NOMINAL.astype(np.float32), (4, 1))
    th[2, 0] = np.nan
    e = _engine(engine_mod, init, actions, target)
    comp, cost = e.evaluate(torch.from_numpy(th))
    bad = e.sync()
    c = cost.cpu().numpy()
    assert bad == init.shape[0]
    assert np.isnan(c[2]) and np.isfinite(c[[0, 1, 3]]).all()


def test_true_theta_has_near_zero_cost(engine_mod):
    """Causal windows replayed at the generating theta reproduce the targets (FP32 rounding only)."""
    rng = np.random.default_rng(9)
    true = random_theta(rng, 1)[0]
    ds, init, actions, target = oracle_windows(5, n_traj=2, T=30, H=20, theta=true)
    others = random_theta(rng, 15)
    th = np.vstack([true, others]).astype(np.float32)
    e = _engine(engine_mod, init, actions, target)
    comp, cost = e.evaluate(torch.from_numpy(th))
    c = cost.cpu().numpy()
    assert c[0] < 1e-6 * np.median(c[1:])
    assert int(np.argmin(c)) == 0
