"""The evaluation path at the full C1 size (4096 theta x 256 windows x H = 20, 13 parameters),
checked through properties that do not depend on size:

* every cost finite, the generating theta the minimum (FP32 rounding only);
* bitwise-identical reruns; permuting theta rows permutes costs bitwise; a sub-batch of rows
  gives bitwise the same costs as inside the full batch;
* window linearity: the weighted-squares cost over 256 windows is the mean of the costs over
  the two halves (1e-5 relative; summation order differs);
* the lane and quad layouts agree (1e-5 relative);
* four prior-sampled theta rows against the FP64 oracle over all 256 windows (1e-4 relative,
  the parity bar).
"""
import numpy as np
import pytest
import torch

from oracle import cost as oc
from oracle import dynamics as dyn
from oracle import go2_model as gm

pytestmark = pytest.mark.gpu
N, W, H = 4096, 256, 20


@pytest.fixture(scope="module")
def c1(built):
    from spi_gb300.data import synthetic_windows
    from spi_gb300.engine import Engine
    rng = np.random.default_rng(1234)
    lo, hi = gm.THETA_PRIOR_LO, gm.THETA_PRIOR_HI
    true = lo + (hi - lo) * rng.random(13)
    e = Engine()
    init, act, tgt = synthetic_windows(e, true, W, H, seed=77)
    e.load_windows(torch.from_numpy(init), torch.from_numpy(act), torch.from_numpy(tgt))
    th = (lo + (hi - lo) * rng.random((N, 13))).astype(np.float32)
    th[0] = true.astype(np.float32)
    th = torch.from_numpy(th)
    comp, cost = e.evaluate(th)
    return e, (init, act, tgt), th, comp.clone(), cost.clone()


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-3 * np.abs(b).max())))


def test_costs_finite_and_generating_theta_is_the_minimum(c1):
    e, _, th, comp, cost = c1
    c = cost.cpu().numpy()
    assert e.sync() == 0 and np.isfinite(c).all()
    assert int(np.argmin(c)) == 0
    assert c[0] < 1e-6 * np.median(c[1:])


def test_reruns_permutations_and_sub_batches_are_bitwise_consistent(c1):
    e, _, th, comp, cost = c1
    assert torch.equal(e.evaluate(th)[1], cost)
    perm = torch.from_numpy(np.random.default_rng(5).permutation(N))
    assert torch.equal(e.evaluate(th[perm])[1], cost[perm.to(cost.device)])
    assert torch.equal(e.evaluate(th[1000:1777])[1], cost[1000:1777])


def test_window_linearity(c1):
    from spi_gb300.engine import Engine
    e, (init, act, tgt), th, comp, cost = c1
    halves = []
    for sl in (slice(0, W // 2), slice(W // 2, W)):
        h = Engine()
        h.load_windows(torch.from_numpy(init[sl]), torch.from_numpy(act[sl]), torch.from_numpy(tgt[sl]))
        halves.append(h.evaluate(th)[1].cpu().numpy())
    assert _rel(0.5 * (halves[0] + halves[1]), cost.cpu().numpy()) <= 1e-5


def test_lane_and_quad_layouts_agree_at_full_size(c1):
    from spi_gb300.autotune import set_variant
    e, _, th, comp, cost = c1
    set_variant(e, "quad4")
    try:
        other = e.evaluate(th)[1].cpu().numpy()
    finally:
        set_variant(e, "lane4")
    assert _rel(other, cost.cpu().numpy()) <= 1e-5


def test_four_rows_against_the_fp64_oracle(c1):
    e, (init, act, tgt), th, comp, cost = c1
    rows = [1, 1000, 2049, 4095]
    t = th.numpy()[rows].astype(np.float64)
    xs = dyn.rollout(np.tile(init.astype(np.float64), (4, 1)), np.tile(act.astype(np.float64), (4, 1, 1)),
                     np.repeat(t, W, 0), gm.SimParams())
    ref = oc.window_components(xs, np.tile(tgt.astype(np.float64), (4, 1))).reshape(4, W, 9).mean(1)
    assert _rel(comp.cpu().numpy()[rows], ref) <= 1e-4
    assert _rel(cost.cpu().numpy()[rows], oc.scalar_cost(ref)) <= 1e-4
