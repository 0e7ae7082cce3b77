"""The FP64 oracle against golden vectors produced by the reference's own functions."""
import numpy as np
import pytest

from oracle import commands as oc_cmd
from oracle import cost as oc
from oracle import dynamics as dyn
from oracle import fisher as ofi
from oracle import go2_model as gm
from oracle import sysid as osy
from oracle import windows as ow


def _theta_kp(kp_scale):
    th = np.tile(gm.THETA_NOMINAL, (kp_scale.shape[0], 1))
    th[:, 5] = kp_scale[:, 0]
    th[:, 9] = kp_scale[:, 0]
    return th


def test_action_clip(golden):
    g = golden("motor")
    np.testing.assert_allclose(np.clip(g["action"], -20, 20), g["clipped"], rtol=1e-6)


@pytest.mark.parametrize("variant", ["base", "omni", "tanh", "vec3"])
def test_motor_model_matches_reference(golden, variant):
    """legged_robot_base._compute_torques, go2_omni hip x0.5, act2tau_vec3(_tanh): <= 1e-5 rel."""
    g = golden("motor")
    sim = gm.SimParams(torque_speed=False, kd_scale=float(g["kd_scale"]))
    if variant in ("omni", "tanh"):
        sim.hip_action_scale = 0.5
    if variant == "tanh":
        sim.tanh_a = g["tanh_a"]
    if variant == "vec3":
        sim.motor_gain = g["gains"]
    tau, arm = dyn.motor_torques(g["q"].astype(np.float32), g["qd"].astype(np.float32),
                                 g["action"].astype(np.float32), _theta_kp(g["kp_scale"]), sim)
    ref = g[f"tau_{variant}"]
    err = np.abs(tau - ref) / np.maximum(np.abs(ref), 1.0)
    assert err.max() <= 1e-5, err.max()
    assert np.all(arm == 0)


def test_scalar_gain_motor(golden):
    g = golden("motor")
    np.testing.assert_allclose(g["tau_base"] * 1.3, g["tau_scalar"], rtol=1e-6, atol=1e-6)


def _trajs(g, prefix_count):
    out = []
    for k in range(prefix_count):
        pre = f"traj{k}_"
        out.append({key[len(pre):]: g[key] for key in g.files if key.startswith(pre)})
    return out


def test_load_dataset_matches_reference(golden):
    g = golden("dataset")
    trajs = _trajs(g, int(g["n_traj"]))
    n, ds = ow.load_dataset(trajs, int(g["horizon"]))
    assert n == int(g["n"])
    for key in g.files:
        if key.startswith("ds_"):
            np.testing.assert_array_equal(ds[key[3:]], g[key], err_msg=key)


def test_evaluate_batch_matches_reference(golden):
    """evaluate_batch glue (chunking, padding, masks, normaliser) on the same physics."""
    g = golden("evaluate")
    sim = gm.SimParams(torque_speed=False, sim_dt=float(g["sim_dt"]), decimation=int(g["decimation"]))
    _, ds = ow.load_dataset(_trajs(g, int(g["n_traj"])), int(g["horizon"]))
    for key in g.files:
        if not key.startswith("res_"):
            continue
        batch, scale = key[4:].split("_")
        th = gm.THETA_NOMINAL.copy()
        th[0] = np.float32(gm.BASE_MASS) * np.float32(float(scale[1:]))
        res = osy.evaluate_reference(ds, th, int(batch[1:]), sim)[0]
        # the reference pipeline stores states in float32: 1e-8 absolute floor
        np.testing.assert_allclose(res, g[key], rtol=1e-5, atol=1e-8, err_msg=key)


def test_evaluate_batch_mixed_gains_matches_reference(golden):
    """Trajectories logged with different Kp / Kd: each env-batch chunk runs with its first
    row's gains (scripts/eval.py:243-250), at batch sizes that put several files in one chunk."""
    g = golden("evaluate_mixed")
    sim = gm.SimParams(torque_speed=False, sim_dt=float(g["sim_dt"]), decimation=int(g["decimation"]))
    _, ds = ow.load_dataset(_trajs(g, int(g["n_traj"])), int(g["horizon"]))
    assert len(np.unique(ds["pd_gain_kp"][:, 0])) == 3
    for key in g.files:
        if not key.startswith("res_"):
            continue
        batch, scale = key[4:].split("_")
        th = gm.THETA_NOMINAL.copy()
        th[0] = np.float32(gm.BASE_MASS) * np.float32(float(scale[1:]))
        res = osy.evaluate_reference(ds, th, int(batch[1:]), sim)[0]
        np.testing.assert_allclose(res, g[key], rtol=1e-5, atol=1e-8, err_msg=key)
    # the same data scored with one gain set for every window gives different numbers
    one = {k: (np.repeat(v[:1], len(v), 0) if k.startswith("pd_gain") else v) for k, v in ds.items()}
    res_one = osy.evaluate_reference(one, gm.THETA_NOMINAL, 40, sim)[0]
    assert np.max(np.abs(res_one - g["res_b40_s1.0"]) / np.abs(g["res_b40_s1.0"])) > 1e-3
    scales = g["landscape_scales"].astype(np.float32).astype(np.float64)
    costs, total, amin = osy.landscape(ds, scales, 40, sim)
    np.testing.assert_allclose(costs, g["landscape"], rtol=1e-5, atol=1e-8)
    assert amin == int(g["landscape_argmin"])


def test_mass_landscape_argmin_matches_reference(golden):
    g = golden("evaluate")
    sim = gm.SimParams(torque_speed=False, sim_dt=float(g["sim_dt"]), decimation=int(g["decimation"]))
    _, ds = ow.load_dataset(_trajs(g, int(g["n_traj"])), int(g["horizon"]))
    scales = g["landscape_scales"].astype(np.float32).astype(np.float64)
    costs, total, amin = osy.landscape(ds, scales, 40, sim)
    np.testing.assert_allclose(costs, g["landscape"], rtol=1e-5, atol=1e-8)
    np.testing.assert_allclose(total, g["landscape_total"], rtol=1e-5, atol=1e-8)
    assert amin == int(g["landscape_argmin"])


def test_compute_cost_weights():
    assert oc.compute_cost([1.0, 1.0, 1.0]) == 16.0
    assert oc.compute_cost([0.1, 0.2, 0.3]) == pytest.approx(1.0 + 1.0 + 0.3)


def test_fd_fisher_matches_reference(golden):
    g = golden("fisher")
    r = ofi.fd_fisher_reward(g["root"], g["dof"], g["origins"], int(g["n_main"]), int(g["P"]),
                             float(g["delta"]))
    np.testing.assert_allclose(r, g["reward"], rtol=1e-5)


def test_command_parametrisations_match_reference(golden):
    g = golden("commands")
    idxs = list(g["idxs"])
    nu, steps = int(g["n_updates"]), int(g["steps_per_update"])
    c = oc_cmd.constant(g["constant_values"], nu, len(idxs), steps)
    np.testing.assert_allclose(oc_cmd.expand(c, g["default_command"], idxs), g["constant_commands"],
                               rtol=1e-6, atol=1e-6)
    p = oc_cmd.polynomial(g["polynomial_values"], g["ranges"], idxs, nu, steps, int(g["poly_degree"]))
    np.testing.assert_allclose(oc_cmd.expand(p, g["default_command"], idxs),
                               g["polynomial_commands"], rtol=1e-5, atol=1e-6)
    b = oc_cmd.bezier(g["bezier_values"], g["ranges"], idxs, nu, steps, int(g["bezier_points"]))
    np.testing.assert_allclose(oc_cmd.expand(b, g["default_command"], idxs), g["bezier_commands"],
                               rtol=1e-5, atol=1e-6)
    from math import comb
    # the reference helper is only called with k <= n (Bernstein basis of degree n)
    for n in range(8):
        for k in range(n + 1):
            assert g["binom"][n, k] == comb(n, k)
