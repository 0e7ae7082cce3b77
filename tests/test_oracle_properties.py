"""Property tests of the FP64 oracle (hypothesis): bounds of the motor model, the cost's
zero and sign, and the CEM elite order, over generated inputs."""
import numpy as np
import pytest

hypothesis = pytest.importorskip("hypothesis")
from hypothesis import given, settings                  # noqa: E402
from hypothesis import strategies as st                 # noqa: E402
from hypothesis.extra import numpy as hnp               # noqa: E402

from oracle import cem as ocem                          # noqa: E402
from oracle import cost as oc                           # noqa: E402
from oracle import dynamics as dyn                      # noqa: E402
from oracle import go2_model as gm                      # noqa: E402

finite = st.floats(-50.0, 50.0, allow_nan=False, allow_infinity=False)


@settings(max_examples=200, deadline=None)
@given(q=hnp.arrays(np.float64, 12, elements=st.floats(-3.0, 3.0)),
       qd=hnp.arrays(np.float64, 12, elements=st.floats(-40.0, 40.0)),
       action=hnp.arrays(np.float64, 12, elements=finite),
       u=hnp.arrays(np.float64, 13, elements=st.floats(0.0, 1.0)),
       reference=st.booleans())
def test_motor_torque_stays_within_its_limits(q, qd, action, u, reference):
    sim = gm.SimParams(torque_speed=not reference)
    th = gm.THETA_PRIOR_LO + (gm.THETA_PRIOR_HI - gm.THETA_PRIOR_LO) * u
    tau, arm = dyn.motor_torques(q, qd, action, th, sim)
    grp, jtype = dyn.joint_groups()
    ts, fc = th[8 + 4 * grp], th[6 + 4 * grp]
    bound = ts * sim.torque_limit * np.abs(sim.motor_gain[jtype]) + fc
    assert np.all(np.abs(tau) <= bound + 1e-9)
    assert np.all(arm >= 0.0)


@settings(max_examples=200, deadline=None)
@given(a=hnp.arrays(np.float64, (3, 37), elements=finite), b=hnp.arrays(np.float64, (3, 37), elements=finite))
def test_window_cost_is_non_negative_and_zero_on_target(a, b):
    c = oc.window_components(a, b)
    assert np.all(c >= 0.0)
    assert np.all(oc.scalar_cost(c) >= 0.0)
    assert np.all(oc.window_components(a, a) == 0.0)


@settings(max_examples=200, deadline=None)
@given(cost=hnp.arrays(np.float64, st.integers(2, 64),
                       elements=st.one_of(st.floats(-1e6, 1e6), st.sampled_from([np.nan, np.inf, -np.inf]))))
def test_elite_order_sorts_finite_costs_first_and_nan_last(cost):
    order = ocem.elite_order(cost)
    assert sorted(order.tolist()) == list(range(cost.shape[0]))
    c = cost[order]
    nan = np.isnan(c)
    assert not np.any(nan[:-1] & ~nan[1:])                       # NaN only at the end
    f = c[~nan]
    assert np.all(f[:-1] <= f[1:])
