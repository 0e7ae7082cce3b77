"""Internal invariants of the FP64 oracle dynamics (dynamics parity with PhysX is unpinned)."""
import numpy as np
import pytest

from oracle import cem
from oracle import checks
from oracle import dynamics as dyn
from oracle import go2_model as gm
from oracle import sysid as osy


def _random_state(rng, B, z=0.3):
    x = np.zeros((B, 37))
    x[:, 2] = z + 0.05 * rng.random(B)
    q = rng.normal(size=(B, 4))
    x[:, 3:7] = q / np.linalg.norm(q, axis=1, keepdims=True)
    x[:, 7:13] = rng.normal(size=(B, 6))
    x[:, 13:25] = gm.DEFAULT_DOF_POS + 0.3 * rng.normal(size=(B, 12))
    x[:, 25:37] = rng.normal(size=(B, 12))
    return x


def _random_theta(rng, B):
    return gm.THETA_PRIOR_LO + (gm.THETA_PRIOR_HI - gm.THETA_PRIOR_LO) * rng.random((B, 13))


def test_aba_inverse_dynamics_round_trip():
    """RNEA(q, qd, ABA(q, qd, tau)) reproduces tau and a zero base wrench, contacts included."""
    rng = np.random.default_rng(0)
    B = 16
    sim = gm.SimParams()
    x = _random_state(rng, B, z=0.2)            # low: some feet and corners penetrate
    th = _random_theta(rng, B)
    act = rng.normal(size=(B, 12))
    _, aux = dyn.substep(x, act, th, sim, return_aux=True)
    assert any(np.abs(m).max() > 0 for m in aux["I_imp"])        # some contacts are active
    fb, tau = checks.rnea(x, aux["a0"], aux["qdd"], th, sim, fext=aux["fext"], I_extra=aux["I_imp"])
    _, arm = dyn.motor_torques(x[:, 13:25], x[:, 25:37], act, th, sim)
    assert np.abs(fb).max() < 1e-9
    assert np.abs(tau + arm * aux["qdd"] - aux["tau"]).max() < 1e-9


def test_mass_matrix_symmetric_positive_definite():
    rng = np.random.default_rng(1)
    x = _random_state(rng, 8)
    M = checks.mass_matrix(x, _random_theta(rng, 8), gm.SimParams())
    assert np.abs(M - np.swapaxes(M, 1, 2)).max() < 1e-12
    assert np.linalg.eigvalsh(M).min() > 0


def _drift(dt, T=0.2):
    rng = np.random.default_rng(2)
    sim = gm.SimParams(gravity=0.0, sim_dt=dt, kp=np.zeros(12), kd=np.zeros(12))
    x = _random_state(rng, 4, z=5.0)
    th = np.tile(gm.THETA_NOMINAL, (4, 1))
    h0 = checks.momentum_world(x, th, sim)
    for _ in range(int(round(T / dt))):
        x = dyn.substep(x, np.zeros((4, 12)), th, sim)
    h1 = checks.momentum_world(x, th, sim)
    return np.abs(h1 - h0).max() / np.abs(h0).max()


def test_free_flight_momentum_drift_is_first_order():
    d1, d2 = _drift(0.002), _drift(0.001)
    assert d1 < 5e-2
    assert 1.5 < d1 / d2 < 2.6


def _energy_drift(dt, T=0.2):
    rng = np.random.default_rng(3)
    sim = gm.SimParams(sim_dt=dt, kp=np.zeros(12), kd=np.zeros(12))
    x = _random_state(rng, 4, z=50.0)                  # far above the ground: no contact
    th = np.tile(gm.THETA_NOMINAL, (4, 1))             # no friction, no armature, no motor torque
    e0 = checks.energy_world(x, th, sim)
    for _ in range(int(round(T / dt))):
        x = dyn.substep(x, np.zeros((4, 12)), th, sim)
    return np.abs(checks.energy_world(x, th, sim) - e0).max() / np.abs(e0).max()


def test_free_flight_energy_drift_is_first_order():
    """Contact and PD off, gravity on: kinetic + potential energy drifts at first order in dt
    (semi-implicit Euler), 2e-5 of the total over 0.2 s at dt = 1 ms."""
    d1, d2 = _energy_drift(0.001), _energy_drift(0.0005)
    assert d1 < 1e-4
    assert 1.8 < d1 / d2 < 2.2


def test_free_fall_from_rest():
    sim = gm.SimParams(kp=np.zeros(12), kd=np.zeros(12))
    x = osy.standing_state(1, z=5.0)
    th = gm.THETA_NOMINAL[None]
    xn = dyn.substep(x, np.zeros((1, 12)), th, sim)
    h = checks.momentum_world(xn, th, sim)
    _, m, _, _ = gm.body_tables()
    m_tot = gm.BASE_MASS + 2 * gm.HEAD_MASS + m[1:].sum()
    np.testing.assert_allclose(h[0, 3:], [0, 0, -m_tot * sim.gravity * sim.sim_dt], rtol=1e-9, atol=1e-12)


def test_quaternion_stays_normalised_and_rollout_finite():
    rng = np.random.default_rng(3)
    sim = gm.SimParams()
    th = _random_theta(rng, 8)
    x0 = osy.standing_state(8)
    acts = osy.sine_actions(60, rng.uniform(0.1, 0.4, (8, 12)), rng.uniform(1, 3, (8, 12)),
                            rng.uniform(0, 6.28, (8, 12)), sim.control_dt, sim.action_scale)
    tr = dyn.rollout(x0, acts, th, sim, trace=True)
    assert np.isfinite(tr).all()
    np.testing.assert_allclose(np.linalg.norm(tr[..., 3:7], axis=-1), 1.0, atol=1e-12)


def test_standing_robot_settles_on_its_feet():
    sim = gm.SimParams()
    tr = dyn.rollout(osy.standing_state(1), np.zeros((1, 100, 12)), gm.THETA_NOMINAL, sim, trace=True)
    z = tr[0, -1, 2]
    assert 0.15 < z < 0.34
    assert np.abs(tr[0, -1, 7:13]).max() < 0.2


@pytest.mark.parametrize("ctr,key,out", [
    ([0, 0, 0, 0], [0, 0], [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]),
    ([0xffffffff] * 4, [0xffffffff] * 2, [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]),
    ([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0],
     [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]),
])
def test_philox_known_answers(ctr, key, out):
    """Random123 known-answer vectors for Philox4x32-10."""
    r = cem.philox4x32_10(np.array(ctr, dtype=np.uint64), np.array(key, dtype=np.uint64))
    assert [int(v) for v in r] == out


def test_cem_converges_on_quadratic():
    lo, hi = np.array([-1.0, -2.0]), np.array([3.0, 2.0])
    target = np.array([1.2, -0.7])
    th = cem.init_samples(lo, hi, 7, 0, 256)
    mu, cov = cem.prior_moments(lo, hi)
    for it in range(1, 25):
        c = np.sum((th - target) ** 2, 1)
        mu, cov = cem.refit(th, c, cem.n_elite(256), mu, cov, 1.0, 1e-4 * (hi - lo))
        th = cem.sample(mu, cov, lo, hi, 7, 0, it, 256)
    assert np.abs(mu - target).max() < 1e-2


def test_elite_order_ties_inf_and_nan():
    """Same order as the device keys: cost ascending, ties by index, +inf, then NaN."""
    c = np.array([3.0, np.nan, 1.0, 1.0, 0.0, np.inf, 2.0], dtype=np.float32)
    assert list(cem.elite_order(c)) == [4, 2, 3, 6, 0, 5, 1]
