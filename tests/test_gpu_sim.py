"""EngineSimulator (BaseSimulator-style state stepping) against the engine's trace and the oracle."""
import numpy as np
import pytest
import torch

from oracle import dynamics as dyn
from oracle import go2_model as gm
from helpers import oracle_windows, random_theta, state_error

pytestmark = pytest.mark.gpu


def test_step_states_matches_trace_and_oracle(built):
    from spi_gb300.engine import Engine
    from spi_gb300.sim import EngineSimulator
    rng = np.random.default_rng(12)
    _, init, actions, target = oracle_windows(9, n_traj=1, T=20, H=6)
    init, actions = init[:13], actions[:13]
    th = random_theta(rng, 13).astype(np.float32)
    sim = EngineSimulator(13)
    ids = torch.arange(13)
    root = torch.from_numpy(init[:, :13])
    dof = torch.from_numpy(np.stack([init[:, 13:25], init[:, 25:37]], -1).reshape(13 * 12, 2))
    sim.set_actor_root_state_tensor(ids, root)
    sim.set_dof_state_tensor(ids, dof)
    sim.set_theta(th)
    for h in range(6):
        sim.step(torch.from_numpy(actions[:, h]))
    torch.cuda.synchronize()
    ref = dyn.rollout(init.astype(np.float64), actions.astype(np.float64), th.astype(np.float64), gm.SimParams())
    assert state_error(sim.state.cpu().numpy(), ref) <= 1e-4
    # the same physics as the window engine: per-row rollouts with a trace
    e = Engine()
    e.load_windows(torch.from_numpy(init), torch.from_numpy(actions), torch.from_numpy(init))
    sim2 = EngineSimulator(13)
    sim2.state = torch.from_numpy(init).cuda()
    sim2.set_theta(th[:1])
    sim2.step(torch.from_numpy(actions), control_steps=6)
    _, _, tr = e.evaluate(torch.from_numpy(th[:1]), trace=True)
    torch.cuda.synchronize()
    # the same substep code in two kernels: rounding may differ at the ulp level where the
    # compiler fuses multiply-adds differently, so the check is a tolerance, not equality
    assert state_error(sim2.state.cpu().numpy(), tr[0, :, -1].cpu().numpy()) <= 1e-5


def test_params_dict_mapping(built):
    from spi_gb300.robot import BASE_COM, BASE_INERTIA
    from spi_gb300.sim import EngineSimulator
    sim = EngineSimulator(3)
    pd = {"mass": {"body_name": "base", "value": [6.0, 7.0, 8.0]},
          "comx": {"body_name": "base", "value": [BASE_COM[0] + 0.01] * 3},
          "inertiax": {"body_name": "base", "value": [BASE_INERTIA[0] * 1.2] * 3},
          "inertiay": {"body_name": "base", "value": [BASE_INERTIA[1] * 1.2] * 3},
          "inertiaz": {"body_name": "base", "value": [BASE_INERTIA[2] * 1.2] * 3}}
    sim.apply_params_dict(pd)
    t = sim.theta.cpu().numpy()
    np.testing.assert_allclose(t[:, 0], [6, 7, 8])
    np.testing.assert_allclose(t[:, 1], 0.01, rtol=1e-5)
    np.testing.assert_allclose(t[:, 4], 1.2, rtol=1e-6)
    pd["inertiay"]["value"] = [BASE_INERTIA[1] * 1.1] * 3
    with pytest.raises(NotImplementedError):
        sim.apply_params_dict(pd)
