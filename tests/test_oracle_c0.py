"""C0, the plain method in FP64 on the CPU: base-mass identification on the oracle alone.

Ground truth at m = 6.921 kg with per-joint sine targets (amplitude U(0.1, 0.4) rad, frequency
U(1, 3) Hz, seeded phases); 64 mass samples U(4, 10) kg, 8 windows, H = 5, 5 CEM iterations,
10 % elite, weighted-squares window cost. The oracle's CEM (same Philox streams as the device
CEM) and the oracle's dynamics must recover the mass.
"""
import numpy as np

from oracle import cem as ocem
from oracle import cost as oc
from oracle import go2_model as gm
from oracle import sysid as osy
from helpers import oracle_windows


def test_c0_mass_identification_on_the_oracle():
    true_mass = 6.921
    theta_true = gm.THETA_NOMINAL.copy()
    theta_true[0] = true_mass
    ds, init, actions, target = oracle_windows(5, n_traj=1, T=12, H=5, theta=theta_true)
    sel = np.arange(8)
    ds = {k: (v[sel] if isinstance(v, np.ndarray) and v.shape[:1] == (init.shape[0],) else v) for k, v in ds.items()}
    lo, hi = np.array([4.0]), np.array([10.0])
    n, seed, job = 64, 3, 0
    ne = ocem.n_elite(n, 0.1)
    mu, cov = ocem.prior_moments(lo, hi)
    best_cost, best_mass = np.inf, None
    for it in range(5):
        x = ocem.init_samples(lo, hi, seed, job, n) if it == 0 else ocem.sample(mu, cov, lo, hi, seed, job, it, n)
        theta = np.tile(gm.THETA_NOMINAL, (n, 1))
        theta[:, 0] = x[:, 0]
        comp = osy.window_components(ds, theta, gm.SimParams()).mean(1)     # [n, 9]
        cost = oc.scalar_cost(comp)
        k = int(np.argmin(cost))
        if cost[k] < best_cost:
            best_cost, best_mass = float(cost[k]), float(x[k, 0])
        mu, cov = ocem.refit(x, cost, ne, mu, cov, 1.0, 1e-3 * (hi - lo))
    assert abs(best_mass - true_mass) < 0.05, best_mass
    assert abs(float(mu[0]) - true_mass) < 0.1, mu
