"""The reference's open-loop collectors (sine, jump, stand) run on the GPU engine, against the
FP64 oracle's collector (scripts/data/sine.py:39-72, jump.py:39-72, stand.py:17-47).

Tolerances, in |gpu - ref| / max(|ref|, 1) at every control step of the first 20: positions,
orientations and joint angles <= 1e-4 (the bar of the rollout parity tests); velocities <= 5e-4.
The profiles start at the reference collectors' base height of 0.32 m and the feet land within
the first control steps; through that impact the joint velocities are the most sensitive
values (the kernel source built for the host in FP32 with exact sine and cosine already differs
from FP64 by 7e-5 there, and the device's fast sine, cosine and reciprocal add to it). Standing
stays within 1e-3 over one second (200 control steps). Actions equal the oracle's to float32
rounding.
"""
import numpy as np
import pytest

from oracle import go2_model as gm
from oracle import sysid as osy
from helpers import state_error

pytestmark = pytest.mark.gpu

STATE_KEYS = ("base_positions", "base_orientations", "base_linear_velocities", "base_angular_velocities",
              "joint_positions", "joint_velocities")


def _states(d):
    return np.concatenate([np.asarray(d[k], dtype=np.float64) for k in STATE_KEYS], -1)


POS = np.r_[0:7, 13:25]       # base position, quaternion, joint angles
VEL = np.r_[7:13, 25:37]      # base linear / angular velocity, joint velocities


def _check_states(got, ref, tol_pos=1e-4, tol_vel=5e-4):
    e = np.abs(got - ref) / np.maximum(np.abs(ref), 1.0)
    ep, ev = float(e[:, POS].max()), float(e[:, VEL].max())
    where = np.unravel_index(np.argmax(e), e.shape)
    assert ep <= tol_pos and ev <= tol_vel, f"positions {ep:.2e}, velocities {ev:.2e}, worst (step, index) {where}"


def _oracle(profile, steps, sim, theta=gm.THETA_NOMINAL):
    acts = osy.profile_actions(profile, steps, sim.control_dt)
    x0 = osy.standing_state(1, z=0.32)
    return acts, osy.collect(x0, acts, theta, sim)[0]


@pytest.mark.parametrize("profile", ["sine", "jump", "stand"])
def test_collector_profile_matches_oracle(built, profile):
    from spi_gb300.data import collect_profile
    from spi_gb300.engine import Engine
    eng = Engine()
    steps = 20
    d = collect_profile(eng, profile, duration_s=steps * eng.cfg.control_dt)
    acts, ref = _oracle(profile, steps, gm.SimParams())
    assert d["actions"].shape == (steps, 12)
    np.testing.assert_allclose(d["actions"], acts[0], rtol=1e-6, atol=1e-7)
    _check_states(_states(d), _states(ref))
    np.testing.assert_allclose(d["timestamps"], np.arange(steps) * eng.cfg.control_dt, atol=1e-12)
    assert d["data_frequency"] == int(round(1.0 / eng.cfg.control_dt))
    np.testing.assert_array_equal(d["pd_gain_kp"], np.full(12, 20.0, np.float32))
    if profile != "stand":
        assert np.ptp(d["joint_positions"][:, 1]) > 1e-3     # the thighs do move


def test_stand_profile_one_second(built):
    from spi_gb300.data import collect_profile
    from spi_gb300.engine import Engine
    eng = Engine()
    d = collect_profile(eng, "stand", duration_s=1.0)
    steps = d["actions"].shape[0]
    assert steps == int(round(1.0 / eng.cfg.control_dt))
    _, ref = _oracle("stand", steps, gm.SimParams())
    assert state_error(_states(d), _states(ref)) <= 1e-3


def test_collected_file_feeds_the_window_loader(built, tmp_path):
    """collect -> npz -> load_dataset -> evaluation at the generating theta reproduces the
    targets (causal windows): the data path a sysid run takes."""
    import torch
    from spi_gb300.data import collect_profile, init_states, load_dataset, save_npz, target_states
    from spi_gb300.engine import Engine
    from spi_gb300.robot import THETA_NOMINAL
    eng = Engine()
    d = collect_profile(eng, "sine", duration_s=0.2)
    save_npz(tmp_path / "sine.npz", d)
    n, ds = load_dataset([tmp_path / "sine.npz"], 5, causal=True)
    assert n == d["actions"].shape[0] - 5
    eng.load_windows(torch.from_numpy(init_states(ds)), torch.from_numpy(ds["action_sequences"]),
                     torch.from_numpy(target_states(ds)))
    comp, _ = eng.evaluate(torch.tensor(THETA_NOMINAL, dtype=torch.float32)[None])
    torch.cuda.synchronize()
    # the trace kernel and the evaluation kernel are separate builds of the same rollout
    assert float(comp[0, 0]) < 1e-4 and float(comp[0, 2]) < 1e-4
