"""The rollout kernel's other layouts against the FP64 oracle and against the quad layout:
SPI_LAYOUT_LANE (one lane per rollout through four legs) and SPI_LAYOUT_BLOCK (the quad
layout with each rollout's base solved once per substep by one warp of the CTA).

Tolerances as the quad layout's parity tests: window error components and costs <= 1e-4
relative to the oracle cost scale; the layouts agree within 1e-5 of the cost scale (each is
compiled separately, so multiply-add fusion, and the lane layout's leg summation order,
differ).
"""
import numpy as np
import pytest
import torch

from oracle import cost as oc
from oracle import dynamics as dyn
from oracle import go2_model as gm
from oracle import sysid as osy
from helpers import oracle_windows, random_theta

pytestmark = pytest.mark.gpu
LANE_VARIANTS = ("lane2", "lane3", "lane4")
BLOCK_VARIANTS = ("block3", "block4", "block5")


def _engine(init, actions, target, variant, weight=None, norm=None):
    from spi_gb300.autotune import set_variant
    from spi_gb300.engine import Engine
    e = Engine()
    e.load_windows(torch.from_numpy(init), torch.from_numpy(actions), torch.from_numpy(target),
                   None if weight is None else torch.from_numpy(np.asarray(weight, np.float32)), norm)
    set_variant(e, variant)
    return e


def cost_error(gpu, ref):
    gpu = np.asarray(gpu, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    scale = np.maximum(np.abs(ref), 1e-3 * np.abs(ref).max())
    return float(np.max(np.abs(gpu - ref) / scale))


def _oracle_comp(init, actions, target, th):
    N, W = th.shape[0], init.shape[0]
    ref = dyn.rollout(np.tile(init.astype(np.float64), (N, 1)), np.tile(actions.astype(np.float64), (N, 1, 1)),
                      np.repeat(th.astype(np.float64), W, 0), gm.SimParams())
    return oc.window_components(ref, np.tile(target.astype(np.float64), (N, 1))).reshape(N, W, 9).mean(1)


@pytest.mark.parametrize("variant", LANE_VARIANTS + BLOCK_VARIANTS)
def test_layout_matches_oracle_h20(built, variant):
    """48 theta x 40 windows (one full and one partial block of 32) x H = 20."""
    rng = np.random.default_rng(200)
    _, init, actions, target = oracle_windows(11, n_traj=3, T=40, H=20)
    sel = rng.choice(init.shape[0], 40, replace=False)
    init, actions, target = init[sel], actions[sel], target[sel]
    th = random_theta(rng, 48).astype(np.float32)
    e = _engine(init, actions, target, variant)
    comp, cost = e.evaluate(torch.from_numpy(th))
    assert e.sync() == 0
    refc = _oracle_comp(init, actions, target, th)
    assert cost_error(comp.cpu().numpy(), refc) <= 1e-4
    assert cost_error(cost.cpu().numpy(), oc.scalar_cost(refc)) <= 1e-4


@pytest.mark.parametrize("variant", ("lane4", "block4"))
@pytest.mark.parametrize("W,H,N", [(1, 1, 1), (13, 3, 5), (33, 2, 9), (64, 5, 3)])
def test_layout_ragged_sizes(built, W, H, N, variant):
    rng = np.random.default_rng(W * 10 + H)
    _, init, actions, target = oracle_windows(W + 1, n_traj=1, T=W + H, H=H)
    init, actions, target = init[:W], actions[:W], target[:W]
    th = random_theta(rng, N).astype(np.float32)
    e = _engine(init, actions, target, variant)
    comp, _ = e.evaluate(torch.from_numpy(th))
    assert cost_error(comp.cpu().numpy(), _oracle_comp(init, actions, target, th)) <= 1e-4


@pytest.mark.parametrize("kw", [dict(tanh_a=(15.0, 18.0, 25.0), hip_action_scale=0.5),
                                dict(motor_gain=(0.9, 1.1, 1.05), torque_speed=False),
                                dict(torque_speed=False)])
def test_lane_motor_models_match_oracle(built, kw):
    """The lane kernels run an instantiation specialised to the default motor model (torque-speed
    limit, unit gains, no tanh saturation) and the run-time-flag kernel for any other; each
    motor model here takes the latter, against the FP64 oracle with the same settings, over
    H = 10."""
    from spi_gb300.autotune import set_variant
    from spi_gb300.engine import Engine
    from spi_gb300.robot import SimConfig
    sim = gm.SimParams(**{k: (np.asarray(v, dtype=np.float64) if isinstance(v, tuple) else v) for k, v in kw.items()})
    rng = np.random.default_rng(202)
    _, init, actions, target = oracle_windows(13, n_traj=2, T=40, H=10, sim=sim)
    init, actions, target = init[:48], actions[:48], target[:48]
    th = random_theta(rng, 16).astype(np.float32)
    e = Engine(SimConfig(**kw))
    e.load_windows(torch.from_numpy(init), torch.from_numpy(actions), torch.from_numpy(target))
    set_variant(e, "lane4")
    comp, cost = e.evaluate(torch.from_numpy(th))
    assert e.sync() == 0
    N, W = th.shape[0], init.shape[0]
    ref = dyn.rollout(np.tile(init.astype(np.float64), (N, 1)), np.tile(actions.astype(np.float64), (N, 1, 1)),
                      np.repeat(th.astype(np.float64), W, 0), sim)
    refc = oc.window_components(ref, np.tile(target.astype(np.float64), (N, 1))).reshape(N, W, 9).mean(1)
    assert cost_error(comp.cpu().numpy(), refc) <= 1e-4
    assert cost_error(cost.cpu().numpy(), oc.scalar_cost(refc)) <= 1e-4


def test_layouts_agree(built):
    rng = np.random.default_rng(201)
    _, init, actions, target = oracle_windows(12, n_traj=4, T=60, H=10)
    init, actions, target = init[:100], actions[:100], target[:100]
    th = torch.from_numpy(random_theta(rng, 256).astype(np.float32))
    costs = {}
    others = ("quad4", "quad5") + LANE_VARIANTS + BLOCK_VARIANTS
    for v in ("quad3",) + others:
        e = _engine(init, actions, target, v)
        costs[v] = e.evaluate(th)[1].cpu().numpy()
    for v in others:
        assert cost_error(costs[v], costs["quad3"]) <= 1e-5, v


@pytest.mark.parametrize("variant", ("lane4", "block4"))
def test_layout_reference_cost_mode_and_mask(built, variant):
    from oracle import windows as ow
    from spi_gb300.engine import COST_REF
    ds, init, actions, target = oracle_windows(2, n_traj=3, T=14, H=5, causal=False)
    mask = ow.eval_mask(ds["motion_ends"], 16)
    n_valid = ow.total_valid(ds["motion_ends"])
    th = random_theta(np.random.default_rng(3), 16).astype(np.float32)
    e = _engine(init, actions, target, variant, weight=mask, norm=n_valid)
    e.set_cost(COST_REF)
    comp, cost = e.evaluate(torch.from_numpy(th))
    refm = oc.reduce_components(osy.window_components(ds, th.astype(np.float64), gm.SimParams()), mask, n_valid)
    assert cost_error(comp.cpu().numpy(), refm) <= 1e-4
    assert cost_error(cost.cpu().numpy(), oc.compute_cost(refm[:, :3])) <= 1e-4


@pytest.mark.parametrize("variant", ("lane4", "block4"))
def test_layout_deterministic_and_counts_nonfinite(built, variant):
    rng = np.random.default_rng(8)
    _, init, actions, target = oracle_windows(3, n_traj=2, T=40, H=10)
    th = random_theta(rng, 40).astype(np.float32)
    th[5, 0] = np.nan
    e = _engine(init, actions, target, variant)
    c1 = e.evaluate(torch.from_numpy(th))[1].clone()
    bad = e.sync()
    c2 = e.evaluate(torch.from_numpy(th))[1].clone()
    assert torch.equal(torch.nan_to_num(c1, nan=-1.0), torch.nan_to_num(c2, nan=-1.0))
    assert bad == init.shape[0]
    c = c1.cpu().numpy()
    assert np.isnan(c[5]) and np.isfinite(np.delete(c, 5)).all()


def test_layouts_under_cem_graph(built):
    """The CEM graph captures the lane kernel (model passed by value) and the block kernel."""
    from spi_gb300.autotune import set_variant
    from spi_gb300.cem import CEM
    from spi_gb300.engine import Engine
    _, init, actions, target = oracle_windows(4, n_traj=2, T=30, H=8)
    res = {}
    for v in ("quad3", "lane4", "block4"):
        e = Engine()
        e.load_windows(torch.from_numpy(init), torch.from_numpy(actions), torch.from_numpy(target))
        set_variant(e, v)
        cem = CEM(e, n_samples=256, param_ids=[0, 4], lo=gm.THETA_PRIOR_LO[[0, 4]], hi=gm.THETA_PRIOR_HI[[0, 4]],
                  nominal=gm.THETA_NOMINAL, seed=5)
        cem.run(3, graph=True)
        res[v] = cem.read()
    # the first iteration's population is identical; later ones may part at the ulp level
    for v in ("lane4", "block4"):
        assert np.isfinite(res[v]["best_cost"])
        assert abs(np.log(res[v]["best_cost"] / res["quad3"]["best_cost"])) < np.log(10.0)
