"""Generate the golden vectors in this folder by executing the reference's own code.

Run where a reference checkout exists, naming it in ``SPI_REFERENCE``::

    SPI_REFERENCE=<path of the reference checkout> PYTHONPATH=. python tests/golden/make_golden.py

The reference cannot be imported whole (Isaac Gym, Hydra and Optuna are not
installable), so each function below is pulled out of its source file with
``ast`` and executed against small stand-in objects: a fake env/simulator whose
physics substep is the FP64 oracle's, a fake Optuna trial that returns seeded
values. Nothing from the reference is copied into this repository; only the
inputs and outputs are saved (``*.npz``).

Pinned functions (reference file:line):
* LeggedRobotBase._pre_physics_step / _compute_torques / step / _physics_step /
  _apply_force_in_physics_step  spigym/envs/legged_base_task/legged_robot_base.py:169-209, 529-560
* go2_omni_interface._compute_torques  spigym/envs/locomotion/go2_omni.py:423-466
* ActiveSysId_OpenLoop.act2tau_scalar / act2tau_vec3 / act2tau_vec3_tanh /
  _reward_fisher_information_matrix  spigym/envs/sysid/active_sysid_openloop.py:356-426
* load_dataset / to_device / capture_reference_masses / apply_pd_gains_batch /
  apply_base_mass / evaluate_batch  scripts/eval.py:101-310 (also on trajectories logged with
  different PD gains, at env batch sizes that split files across chunks)
* compute_cost  scripts/mass_opt.py:62-76;  mass_sweep  scripts/mass_landscape.py:111-128
* format_data  scripts/data/common.py:83-100
* ActiveSysId.sample_commands / _sample_constant / _sample_polynomial /
  _sample_bezier / _binomial_coefficient  spigym/agents/sysid/active_sysid.py:259-400
"""
from __future__ import annotations

import ast
import os
import sys
import tempfile
import textwrap
from dataclasses import dataclass
from pathlib import Path
from types import SimpleNamespace

import numpy as np
import torch

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

from oracle import dynamics as dyn  # noqa: E402
from oracle import go2_model as gm  # noqa: E402
from oracle import sysid as osy  # noqa: E402

REF = Path(os.environ["SPI_REFERENCE"]) if os.environ.get("SPI_REFERENCE") else None


def extract(relpath, name, cls=None):
    """Source of a top-level function/class or of a method, with its decorators."""
    src = (REF / relpath).read_text()
    tree = ast.parse(src)
    scope = tree.body
    if cls is not None:
        scope = next(n for n in tree.body if isinstance(n, ast.ClassDef) and n.name == cls).body
    node = next(n for n in scope if isinstance(n, (ast.FunctionDef, ast.ClassDef)) and n.name == name)
    lines = src.splitlines()
    start = min([node.lineno] + [d.lineno for d in node.decorator_list]) - 1
    return textwrap.dedent("\n".join(lines[start:node.end_lineno]))


def load(relpath, names, cls=None, extra=None):
    ns = {"torch": torch, "np": np, "Tensor": torch.Tensor, "dataclass": dataclass,
          "Path": Path, "Dict": dict, "Tuple": tuple, "List": list}
    ns.update(extra or {})
    for n in names:
        exec(compile(extract(relpath, n, cls), f"{relpath}:{n}", "exec"), ns)
    return ns


def cfg(**kw):
    return SimpleNamespace(**kw)


# ----------------------------------------------------------------------------
# 1. action clip, PD law, motor models
# ----------------------------------------------------------------------------
def motor_golden(rng):
    N = 64
    lrb = load("spigym/envs/legged_base_task/legged_robot_base.py",
               ["_pre_physics_step", "_compute_torques"], cls="LeggedRobotBase")
    omni = load("spigym/envs/locomotion/go2_omni.py", ["_compute_torques"], cls="go2_omni_interface")
    aso = load("spigym/envs/sysid/active_sysid_openloop.py",
               ["act2tau_scalar", "act2tau_vec3", "act2tau_vec3_tanh"], cls="ActiveSysId_OpenLoop")
    q = gm.DEFAULT_DOF_POS + 0.5 * rng.standard_normal((N, 12))
    qd = 3.0 * rng.standard_normal((N, 12))
    act = 6.0 * rng.standard_normal((N, 12))
    act[:4] *= 8.0                                    # hit the +-20 clip
    kp_scale = rng.uniform(0.8, 1.2, (N, 1))
    kd_scale = 1.1
    tanh_a = np.array([15.0, 18.0, 25.0])
    gains = np.array([0.9, 1.1, 1.05])
    env = SimpleNamespace(
        config=cfg(robot=cfg(control=cfg(action_clip_value=20.0, action_scale=0.25, control_type="P",
                                         clip_torques=True)),
                   domain_rand=cfg(randomize_ctrl_delay=False, randomize_torque_rfi=False,
                                   randomize_motor_model=False)),
        device="cpu", log_dict={}, num_envs=N,
        p_gains=torch.full((12,), 20.0), d_gains=torch.full((12,), 0.5),
        _kp_scale=torch.tensor(np.repeat(kp_scale, 12, 1), dtype=torch.float32),
        _kd_scale=torch.full((N, 12), kd_scale),
        default_dof_pos=torch.tensor(gm.DEFAULT_DOF_POS, dtype=torch.float32)[None],
        torque_limits=torch.tensor(gm.TORQUE_LIMIT, dtype=torch.float32),
        simulator=SimpleNamespace(dof_pos=torch.tensor(q, dtype=torch.float32),
                                  dof_vel=torch.tensor(qd, dtype=torch.float32)),
        params_dict={"motor_model_hip_a": {"value": [tanh_a[0]] * N},
                     "motor_model_thigh_a": {"value": [tanh_a[1]] * N},
                     "motor_model_calf_a": {"value": [tanh_a[2]] * N}},
    )
    lrb["_pre_physics_step"](env, torch.tensor(act, dtype=torch.float32))
    clipped = env.actions.clone()
    tau_base = lrb["_compute_torques"](env, env.actions_after_delay.clone())
    tau_omni = omni["_compute_torques"](env, env.actions_after_delay.clone())
    tau_tanh = aso["act2tau_vec3_tanh"](env, tau_omni.clone())
    tau_vec3 = aso["act2tau_vec3"](env, tau_base.clone(), hip_gain=[gains[0]] * N,
                                   thigh_gain=[gains[1]] * N, calf_gain=[gains[2]] * N)
    tau_scalar = aso["act2tau_scalar"](env, tau_base.clone(), scalar_gain=[1.3] * N)
    np.savez(HERE / "motor.npz", q=q, qd=qd, action=act, kp_scale=kp_scale, kd_scale=kd_scale,
             tanh_a=tanh_a, gains=gains, clipped=clipped.numpy(), tau_base=tau_base.numpy(),
             tau_omni=tau_omni.numpy(), tau_tanh=tau_tanh.numpy(), tau_vec3=tau_vec3.numpy(),
             tau_scalar=tau_scalar.numpy())


# ----------------------------------------------------------------------------
# 2. format_data + load_dataset (window construction)
# ----------------------------------------------------------------------------
def dataset_golden(rng):
    common = load("scripts/data/common.py", ["format_data"])
    ev = load("scripts/eval.py", ["load_dataset"])
    env = SimpleNamespace(p_gains=torch.full((2, 12), 20.0), d_gains=torch.full((2, 12), 0.5))
    lengths = (30, 17, 23)
    trajs = []
    with tempfile.TemporaryDirectory() as td:
        paths = []
        for k, T in enumerate(lengths):
            frames = []
            for t in range(T):
                frames.append({
                    "timestamp": t * 0.02,
                    "joint_positions": rng.standard_normal(12).astype(np.float32),
                    "joint_velocities": rng.standard_normal(12).astype(np.float32),
                    "joint_torques": rng.standard_normal(12).astype(np.float32),
                    "actions": rng.standard_normal(12).astype(np.float32),
                    "base_positions": rng.standard_normal(3).astype(np.float32),
                    "base_orientations": rng.standard_normal(4).astype(np.float32),
                    "base_linear_velocities": rng.standard_normal(3).astype(np.float32),
                    "base_angular_velocities": rng.standard_normal(3).astype(np.float32),
                })
            data = common["format_data"](frames, env, 0.02)
            p = Path(td) / f"traj{k}.npz"
            np.savez(p, **data)
            paths.append(p)
            trajs.append({kk: np.asarray(vv) for kk, vv in data.items()})
        n, ds = ev["load_dataset"](paths, 5)
    out = {f"traj{k}_{kk}": v for k, t in enumerate(trajs) for kk, v in t.items()
           if kk != "robot_type"}
    out.update({f"ds_{k}": v for k, v in ds.items()})
    np.savez(HERE / "dataset.npz", n=n, horizon=5, n_traj=len(lengths), **out)


# ----------------------------------------------------------------------------
# 3. evaluate_batch / apply_base_mass / mass_sweep / compute_cost on oracle physics
# ----------------------------------------------------------------------------
class _Prop:
    def __init__(self, mass):
        self.mass = mass


class FakeGym:
    def __init__(self, masses, n_envs):
        self.props = [[_Prop(float(m)) for m in masses] for _ in range(n_envs)]

    def get_actor_rigid_body_properties(self, env_ptr, actor):
        return [_Prop(p.mass) for p in self.props[env_ptr]]

    def set_actor_rigid_body_properties(self, env_ptr, actor, props, recomputeInertia=False):
        self.props[env_ptr] = [_Prop(p.mass) for p in props]

    def refresh_mass_matrix_tensors(self, sim):
        pass


class FakeSimulator:
    """Stand-in for the Isaac Gym adapter: tensor views + one oracle substep per simulate."""

    def __init__(self, n_envs, sim_params):
        self.num_envs = n_envs
        self.sim_params = sim_params
        self.sim = None
        self.envs = list(range(n_envs))
        self.robot_handles = [0] * n_envs
        masses = [gm.BASE_MASS] + [0.0] * 12
        _, bm, _, _ = gm.body_tables()
        masses[1:] = list(bm[1:])
        self.gym = FakeGym(masses, n_envs)
        self.x = osy.standing_state(n_envs)
        self.robot_root_states = torch.zeros(n_envs, 13)
        self.all_root_states = self.robot_root_states
        self.dof_state = torch.zeros(n_envs * 12, 2)
        self.dof_pos = self.dof_state.view(n_envs, 12, 2)[..., 0]
        self.dof_vel = self.dof_state.view(n_envs, 12, 2)[..., 1]
        self._torques = None
        self.refresh_sim_tensors()

    def theta(self):
        th = np.tile(gm.THETA_NOMINAL, (self.num_envs, 1))
        th[:, 0] = [self.gym.props[e][0].mass for e in range(self.num_envs)]
        return th

    def refresh_sim_tensors(self):
        self.robot_root_states[:] = torch.tensor(self.x[:, :13], dtype=torch.float32)
        self.dof_pos[:] = torch.tensor(self.x[:, 13:25], dtype=torch.float32)
        self.dof_vel[:] = torch.tensor(self.x[:, 25:37], dtype=torch.float32)

    def set_actor_root_state_tensor(self, env_ids, root_states):
        ids = env_ids.numpy()
        self.x[ids, :13] = root_states[ids].double().numpy()

    def set_dof_state_tensor(self, env_ids, dof_states):
        ids = env_ids.numpy()
        ds = dof_states.view(self.num_envs, 12, 2).double().numpy()
        self.x[ids, 13:25] = ds[ids, :, 0]
        self.x[ids, 25:37] = ds[ids, :, 1]

    def apply_torques_at_dof(self, torques):
        self._torques = torques.double().numpy().copy()

    def simulate_at_each_physics_step(self):
        self.x = dyn.substep(self.x, np.zeros((self.num_envs, 12)), self.theta(), self.sim_params,
                             tau_override=self._torques)
        self.refresh_sim_tensors()


def make_fake_env(n_envs, sim_params):
    lrb = load("spigym/envs/legged_base_task/legged_robot_base.py",
               ["step", "_pre_physics_step", "_physics_step", "_apply_force_in_physics_step",
                "_compute_torques"], cls="LeggedRobotBase")

    class FakeEnv:
        step = lrb["step"]
        _pre_physics_step = lrb["_pre_physics_step"]
        _physics_step = lrb["_physics_step"]
        _apply_force_in_physics_step = lrb["_apply_force_in_physics_step"]
        _compute_torques = lrb["_compute_torques"]

        def __init__(self):
            self.num_envs = n_envs
            self.dim_actions = 12
            self.device = "cpu"
            self.simulator = FakeSimulator(n_envs, sim_params)
            self.config = cfg(
                robot=cfg(control=cfg(action_clip_value=20.0, action_scale=0.25, control_type="P",
                                      clip_torques=True)),
                domain_rand=cfg(randomize_ctrl_delay=False, randomize_torque_rfi=False),
                simulator=cfg(config=cfg(sim=cfg(control_decimation=sim_params.decimation))))
            self.log_dict = {}
            self.p_gains = torch.zeros(12)
            self.d_gains = torch.zeros(12)
            self._kp_scale = torch.ones(n_envs, 12)
            self._kd_scale = torch.ones(n_envs, 12)
            self.default_dof_pos = torch.tensor(gm.DEFAULT_DOF_POS, dtype=torch.float32)[None]
            self.torque_limits = torch.tensor(gm.TORQUE_LIMIT, dtype=torch.float32)
            self.torques = torch.zeros(n_envs, 12)
            for k in ("actions", "last_actions", "actions_after_delay", "last_dof_vel",
                      "feet_air_time"):
                setattr(self, k, torch.zeros(n_envs, 12))
            self.episode_length_buf = torch.zeros(n_envs, dtype=torch.long)
            self.reset_buf = torch.zeros(n_envs, dtype=torch.long)
            self.obs_buf_dict, self.rew_buf, self.extras = {}, torch.zeros(n_envs), {}

        def render(self, sync_frame_time=True):
            pass

        def _post_physics_step(self):
            self.simulator.refresh_sim_tensors()

        def reset_all(self):
            self.step({"actions": torch.zeros(self.num_envs, 12)})

    return FakeEnv()


def ground_truth(rng, sim_params, n_traj=2, T=40):
    settle = 60
    amp = rng.uniform(0.1, 0.4, (n_traj, 12))
    freq = rng.uniform(1.0, 3.0, (n_traj, 12))
    ph = rng.uniform(0, 2 * np.pi, (n_traj, 12))
    acts = osy.sine_actions(settle + T, amp, freq, ph, sim_params.control_dt,
                            sim_params.action_scale, settle=settle)
    x0 = osy.standing_state(n_traj)
    frames = osy.collect(x0, acts, gm.THETA_NOMINAL, sim_params)
    return [{k: (v[settle:] if isinstance(v, np.ndarray) and v.ndim and v.shape[0] == settle + T
                 else v) for k, v in f.items()} for f in frames]


def _eval_functions():
    ev_names = ["DatasetBatch", "MassEvalResult", "load_dataset", "to_device",
                "capture_reference_masses", "apply_pd_gains_batch", "apply_base_mass",
                "evaluate_batch"]
    import tqdm
    ev = load("scripts/eval.py", ev_names, extra={"tqdm": tqdm.tqdm, "LeggedRobotBase": object})
    mass_eval = SimpleNamespace(**{k: ev[k] for k in ev_names})
    ml = load("scripts/mass_landscape.py", ["mass_sweep"],
              extra={"mass_eval": mass_eval, "Iterable": object})
    mo = load("scripts/mass_opt.py", ["compute_cost"],
              extra={"COST_COEFF": {"base_pos": 10.0, "base_quat": 5.0, "joint_pos": 1.0}})
    return ev, ml, mo


def evaluate_golden(rng):
    sp = gm.SimParams(torque_speed=False)
    trajs = ground_truth(rng, sp)
    ev, ml, mo = _eval_functions()
    with tempfile.TemporaryDirectory() as td:
        paths = []
        for k, t in enumerate(trajs):
            p = Path(td) / f"gt{k}.npz"
            np.savez(p, **t)
            paths.append(p)
        H = 5
        n, ds_np = ev["load_dataset"](paths, H)
    results = {}
    for batch in (16, 40):
        env = make_fake_env(batch, sp)
        ds = ev["to_device"](ds_np, torch.device("cpu"))
        ref_masses = ev["capture_reference_masses"](env.simulator)
        action_buffer = torch.zeros(batch, 12)
        scales = np.array([0.8, 1.0, 1.3])
        for s in scales:
            ev["apply_base_mass"](env.simulator, ref_masses, float(ref_masses[0]) * float(s))
            r = ev["evaluate_batch"](env, H, action_buffer, ds)
            results[f"b{batch}_s{s}"] = np.array([r.base_pos, r.base_quat, r.joint_pos])
    # mass landscape (20-point grid of the reference) + compute_cost + argmin
    env = make_fake_env(40, sp)
    ds = ev["to_device"](ds_np, torch.device("cpu"))
    ref_masses = ev["capture_reference_masses"](env.simulator)
    scales = np.linspace(0.5, 2.0, 20)
    land = ml["mass_sweep"](env, ds, H, ref_masses, scales)
    total = np.array([mo["compute_cost"](row) for row in land])
    out = {f"traj{k}_{kk}": v for k, t in enumerate(trajs) for kk, v in t.items()
           if kk != "robot_type"}
    out.update({f"res_{k}": v for k, v in results.items()})
    np.savez(HERE / "evaluate.npz", n_traj=len(trajs), horizon=H, sim_dt=sp.sim_dt,
             decimation=sp.decimation, landscape_scales=scales, landscape=land,
             landscape_total=total, landscape_argmin=int(np.argmin(total)), **out)


# ----------------------------------------------------------------------------
# 4. FD-Fisher reward (reference active-sysid objective)
# ----------------------------------------------------------------------------
def fisher_golden(rng):
    aso = load("spigym/envs/sysid/active_sysid_openloop.py", ["_reward_fisher_information_matrix"],
               cls="ActiveSysId_OpenLoop")
    n_main, P = 8, 3
    N = n_main * (P + 1)
    root = rng.standard_normal((N, 13)).astype(np.float32)
    dof = rng.standard_normal((N, 12)).astype(np.float32)
    origins = rng.standard_normal((N, 3)).astype(np.float32)
    idx = torch.arange(N).view(n_main, P + 1)
    self = SimpleNamespace(simulator=SimpleNamespace(robot_root_states=torch.tensor(root),
                                                     dof_pos=torch.tensor(dof)),
                           env_origins=torch.tensor(origins), main_idx=idx[:, 0:1],
                           aux_idx=idx[:, 1:], delta_param=0.1, param_dim=P)
    rew = aso["_reward_fisher_information_matrix"](self)
    np.savez(HERE / "fisher.npz", root=root, dof=dof, origins=origins, n_main=n_main, P=P,
             delta=0.1, reward=rew.numpy())


# ----------------------------------------------------------------------------
# 5. candidate-command parametrisations
# ----------------------------------------------------------------------------
class FakeTrial:
    def __init__(self, rng):
        self.rng = rng
        self.names, self.values = [], []

    def suggest_float(self, name, lo, hi):
        v = float(self.rng.uniform(lo, hi))
        self.names.append(name)
        self.values.append(v)
        return v


def commands_golden(rng):
    names = ["sample_commands", "_sample_constant", "_sample_polynomial", "_sample_bezier",
             "_binomial_coefficient"]
    ns = load("spigym/agents/sysid/active_sysid.py", names, cls="ActiveSysId")

    class Sampler:
        pass
    for n in names:
        setattr(Sampler, n, ns[n])
    out = {}
    ranges = np.array([[-1.0, 1.0], [-0.5, 0.5], [-1.0, 1.0], [0.2, 0.4], [0.0, 1.0]] +
                      [[0.0, 1.0]] * 9)
    for mode in ("constant", "polynomial", "bezier"):
        s = Sampler()
        s.default_command = np.array([0.3, 0.0, 0.1, 0.3] + [0.0] * 10, dtype=np.float32)
        s.command_sampling_idxs = [0, 1, 2]
        s.num_steps_per_update = 25
        s.poly_degree = 3
        s.num_bezier_points = 4
        s.command_sampling_mode = mode
        trial = FakeTrial(rng)
        cmds = s.sample_commands(trial, ranges, 4)
        out[f"{mode}_values"] = np.array(trial.values)
        out[f"{mode}_commands"] = cmds
    out["binom"] = np.array([[ns["_binomial_coefficient"](None, n, k) for k in range(8)]
                             for n in range(8)])
    np.savez(HERE / "commands.npz", ranges=ranges, default_command=np.array(
        [0.3, 0.0, 0.1, 0.3] + [0.0] * 10, dtype=np.float32), idxs=np.array([0, 1, 2]),
        steps_per_update=25, poly_degree=3, bezier_points=4, n_updates=4, **out)


# ----------------------------------------------------------------------------
# 3b. evaluate_batch / mass_sweep on trajectories logged with different PD gains
# ----------------------------------------------------------------------------
MIXED_GAINS = ((20.0, 0.5), (25.0, 0.6), (17.0, 0.4))


def evaluate_mixed_golden(rng):
    """Three trajectories, each logged (and stored) with its own Kp / Kd; env batch sizes 16,
    40 and 50 put windows of several files into one chunk, whose gains are its first row's."""
    ev, ml, mo = _eval_functions()
    trajs = []
    for kp, kd in MIXED_GAINS:
        sp_k = gm.SimParams(torque_speed=False, kp=np.full(12, kp), kd=np.full(12, kd))
        trajs += ground_truth(rng, sp_k, n_traj=1)
    sp = gm.SimParams(torque_speed=False)
    H = 5
    with tempfile.TemporaryDirectory() as td:
        paths = []
        for k, t in enumerate(trajs):
            p = Path(td) / f"gt{k}.npz"
            np.savez(p, **t)
            paths.append(p)
        n, ds_np = ev["load_dataset"](paths, H)
    results = {}
    for batch in (16, 40, 50):
        env = make_fake_env(batch, sp)
        ds = ev["to_device"](ds_np, torch.device("cpu"))
        ref_masses = ev["capture_reference_masses"](env.simulator)
        action_buffer = torch.zeros(batch, 12)
        for s in (0.8, 1.0, 1.3):
            ev["apply_base_mass"](env.simulator, ref_masses, float(ref_masses[0]) * float(s))
            r = ev["evaluate_batch"](env, H, action_buffer, ds)
            results[f"b{batch}_s{s}"] = np.array([r.base_pos, r.base_quat, r.joint_pos])
    env = make_fake_env(40, sp)
    ds = ev["to_device"](ds_np, torch.device("cpu"))
    ref_masses = ev["capture_reference_masses"](env.simulator)
    scales = np.linspace(0.5, 2.0, 20)
    land = ml["mass_sweep"](env, ds, H, ref_masses, scales)
    total = np.array([mo["compute_cost"](row) for row in land])
    out = {f"traj{k}_{kk}": v for k, t in enumerate(trajs) for kk, v in t.items()
           if kk != "robot_type"}
    out.update({f"res_{k}": v for k, v in results.items()})
    np.savez(HERE / "evaluate_mixed.npz", n_traj=len(trajs), horizon=H, sim_dt=sp.sim_dt,
             decimation=sp.decimation, landscape_scales=scales, landscape=land,
             landscape_total=total, landscape_argmin=int(np.argmin(total)), **out)


def main():
    if REF is None or not REF.is_dir():
        raise SystemExit("set SPI_REFERENCE to the path of a reference checkout "
                         f"(got {os.environ.get('SPI_REFERENCE')!r})")
    rng = np.random.default_rng(20261203)
    motor_golden(rng)
    dataset_golden(rng)
    evaluate_golden(rng)
    fisher_golden(rng)
    commands_golden(rng)
    evaluate_mixed_golden(rng)
    print("golden vectors written to", HERE)


if __name__ == "__main__":
    main()
