"""Device CEM (spi_cem_*) against the FP64 oracle CEM (oracle/cem.py)."""
import numpy as np
import pytest
import torch

from oracle import cem as ocem
from oracle import go2_model as gm
from helpers import oracle_windows, random_theta

pytestmark = pytest.mark.gpu


def _setup(P=13, N=256, seed=11, alpha=1.0, H=5, theta_true=None):
    from spi_gb300.cem import CEM
    from spi_gb300.engine import Engine
    ds, init, actions, target = oracle_windows(21, n_traj=2, T=16, H=H, theta=theta_true)
    e = Engine()
    e.load_windows(torch.from_numpy(init), torch.from_numpy(actions), torch.from_numpy(target))
    ids = list(range(P))
    cem = CEM(e, n_samples=N, param_ids=ids, lo=gm.THETA_PRIOR_LO[ids], hi=gm.THETA_PRIOR_HI[ids],
              nominal=gm.THETA_NOMINAL, elite_frac=0.1, alpha=alpha, min_std_frac=1e-3, seed=seed, job_id=3)
    return e, cem, ids


@pytest.mark.parametrize("P,N", [(1, 256), (5, 256), (13, 256), (13, 3000), (13, 4096)])
def test_sampling_and_refit_match_oracle(built, P, N):
    """N = 3000 pads the sort to 4096 keys; 3000 and 4096 put four keys on each sort thread."""
    seed = 11
    e, cem, ids = _setup(P=P, N=N, seed=seed, alpha=0.9)
    lo, hi = gm.THETA_PRIOR_LO[ids], gm.THETA_PRIOR_HI[ids]
    # iteration 0: uniform prior box
    cem.sample()
    th0 = cem.theta().cpu().numpy()
    ref0 = ocem.init_samples(lo, hi, seed, 3, N)
    np.testing.assert_allclose(th0[:, ids], ref0.astype(np.float32), rtol=1e-6, atol=1e-7)
    others = [i for i in range(13) if i not in ids]
    assert np.array_equal(th0[:, others], np.tile(gm.THETA_NOMINAL.astype(np.float32), (N, 1))[:, others])
    # rollout + refit
    e.run()
    _, cost = e.read()
    cem.refit()
    r = cem.read()
    mu0, cov0 = ocem.prior_moments(lo, hi)
    mu, cov = ocem.refit(th0[:, ids].astype(np.float64), cost.cpu().numpy(), ocem.n_elite(N), mu0, cov0, 0.9,
                         1e-3 * (hi - lo))
    np.testing.assert_allclose(r["mu"], mu, rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(r["cov"], cov, rtol=1e-9, atol=1e-15)
    assert r["iteration"] == 1
    # iteration 1: Gaussian samples from the refit distribution
    cem.sample()
    th1 = cem.theta().cpu().numpy()
    ref1 = ocem.sample(mu, cov, lo, hi, seed, 3, 1, N)
    np.testing.assert_allclose(th1[:, ids], ref1.astype(np.float32), rtol=2e-6, atol=1e-7)


@pytest.mark.parametrize("n", [64, 1000, 4096, 16384])
def test_refit_elite_selection_with_ties_and_nonfinite_costs(built, n):
    """The refit's elite set under costs with many ties, NaN, +inf and -inf: the n_elite smallest
    by (cost, index) with NaN after +inf, as the oracle orders them, at populations up to the
    16384 maximum (the largest shared-memory footprint of the refit kernel)."""
    from spi_gb300.active import DeviceSearch
    P = 5
    lo, hi = np.zeros(P), np.ones(P)
    s = DeviceSearch(n, lo, hi, elite_frac=0.1, alpha=0.8, min_std_frac=1e-3, seed=5)
    pop = s.sample()
    theta = pop.cpu().numpy()[:, :P].astype(np.float64)
    rng = np.random.default_rng(n)
    cost = rng.integers(0, 7, n).astype(np.float32)          # seven distinct values: ties everywhere
    cost[rng.choice(n, n // 10, replace=False)] = np.nan
    cost[rng.choice(n, n // 20, replace=False)] = np.inf
    cost[rng.choice(n, 3, replace=False)] = -np.inf
    s.refit(torch.from_numpy(cost).cuda())
    r = s.read()
    mu0, cov0 = ocem.prior_moments(lo, hi)
    mu, cov = ocem.refit(theta, cost, ocem.n_elite(n), mu0, cov0, 0.8, 1e-3 * (hi - lo))
    np.testing.assert_allclose(r["mu"], mu, rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(r["cov"], cov, rtol=1e-9, atol=1e-15)
    best = ocem.elite_order(cost)[0]
    assert r["best_cost"] == -np.inf
    np.testing.assert_array_equal(r["best"][:P], pop.cpu().numpy()[best, :P])
    s.close()


def test_graph_replay_equals_eager_steps(built):
    e1, c1, _ = _setup(P=4, N=512, seed=5)
    for _ in range(6):
        c1.step()
    r1 = c1.read()
    e2, c2, _ = _setup(P=4, N=512, seed=5)
    c2.run(6, graph=True)
    r2 = c2.read()
    assert r2["iteration"] == 6
    assert np.array_equal(r1["mu"], r2["mu"]) and np.array_equal(r1["cov"], r2["cov"])
    assert r1["best_cost"] == r2["best_cost"]


def test_mass_identification_converges(built):
    """Mass-only identification (C0-style: 64 samples, H=5, 5 iterations) finds the true mass."""
    true = gm.THETA_NOMINAL.copy()
    true[0] = 7.4
    from spi_gb300.cem import CEM
    from spi_gb300.engine import Engine
    ds, init, actions, target = oracle_windows(31, n_traj=2, T=12, H=5, theta=true)
    e = Engine()
    e.load_windows(torch.from_numpy(init), torch.from_numpy(actions), torch.from_numpy(target))
    cem = CEM(e, n_samples=64, param_ids=[0], lo=[4.0], hi=[10.0], nominal=gm.THETA_NOMINAL,
              elite_frac=0.1, seed=1)
    for _ in range(5):
        cem.step()
    r = cem.read()
    assert abs(r["best_theta"][0] - 7.4) < 0.05
    assert abs(r["mu"][0] - 7.4) < 0.1
