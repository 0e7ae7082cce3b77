"""eval_compat (the drop-in for scripts/eval.py) against the reference's own evaluate_batch.

The golden values were produced by the reference's evaluate_batch / mass_sweep /
compute_cost running on the FP64 oracle physics (tests/golden/make_golden.py).
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _trajs(g):
    out = []
    for k in range(int(g["n_traj"])):
        pre = f"traj{k}_"
        out.append({key[len(pre):]: g[key] for key in g.files if key.startswith(pre)})
    return out


def _env_and_ds(golden, batch, name="evaluate"):
    from spi_gb300 import eval_compat as ec
    from spi_gb300.data import load_dataset
    from spi_gb300.robot import SimConfig
    g = golden(name)
    cfg = SimConfig.reference_compatible(sim_dt=float(g["sim_dt"]), decimation=int(g["decimation"]))
    _, ds_np = load_dataset(_trajs(g), int(g["horizon"]))
    env = ec.instantiate_env(None, batch, cfg=cfg)
    return g, ec, env, ec.to_device(ds_np, env.device)


@pytest.mark.parametrize("batch", [16, 40])
def test_evaluate_batch_matches_reference(built, golden, batch):
    g, ec, env, ds = _env_and_ds(golden, batch)
    ref_masses = ec.capture_reference_masses(env.simulator)
    buf = torch.zeros(batch, 12, device=env.device)
    for scale in (0.8, 1.0, 1.3):
        ec.apply_base_mass(env.simulator, ref_masses, float(ref_masses[0]) * scale)
        r = ec.evaluate_batch(env, int(g["horizon"]), buf, ds)
        got = np.array([r.base_pos, r.base_quat, r.joint_pos])
        want = g[f"res_b{batch}_s{scale}"]
        np.testing.assert_allclose(got, want, rtol=1e-4, atol=1e-7)


def test_mass_landscape_argmin_matches_reference(built, golden):
    g, ec, env, ds = _env_and_ds(golden, 40)
    ref_masses = ec.capture_reference_masses(env.simulator)
    land = ec.mass_sweep(env, ds, int(g["horizon"]), ref_masses, g["landscape_scales"])
    total = np.array([ec.compute_cost(r) for r in land])
    np.testing.assert_allclose(land, g["landscape"], rtol=1e-4, atol=1e-7)
    assert int(np.argmin(total)) == int(g["landscape_argmin"])


@pytest.mark.parametrize("batch", [16, 40, 50])
def test_evaluate_batch_mixed_gains_matches_reference(built, golden, batch):
    """Three files logged with Kp / Kd of 20 / 0.5, 25 / 0.6 and 17 / 0.4: every env-batch
    chunk runs with its first row's gains, as scripts/eval.py:243-250 applies them."""
    g, ec, env, ds = _env_and_ds(golden, batch, "evaluate_mixed")
    ref_masses = ec.capture_reference_masses(env.simulator)
    buf = torch.zeros(batch, 12, device=env.device)
    for scale in (0.8, 1.0, 1.3):
        ec.apply_base_mass(env.simulator, ref_masses, float(ref_masses[0]) * scale)
        r = ec.evaluate_batch(env, int(g["horizon"]), buf, ds)
        got = np.array([r.base_pos, r.base_quat, r.joint_pos])
        want = g[f"res_b{batch}_s{scale}"]
        np.testing.assert_allclose(got, want, rtol=1e-4, atol=1e-7)
    # the last chunk's gains stay applied, as in the reference
    assert float(env.p_gains[0]) == float(ds.pd_gain_kp[((ds.pd_gain_kp.shape[0] - 1) // batch) * batch, 0])


def test_mass_landscape_mixed_gains_matches_reference(built, golden):
    g, ec, env, ds = _env_and_ds(golden, 40, "evaluate_mixed")
    ref_masses = ec.capture_reference_masses(env.simulator)
    land = ec.mass_sweep(env, ds, int(g["horizon"]), ref_masses, g["landscape_scales"])
    total = np.array([ec.compute_cost(r) for r in land])
    np.testing.assert_allclose(land, g["landscape"], rtol=1e-4, atol=1e-7)
    assert int(np.argmin(total)) == int(g["landscape_argmin"])
