"""Shared test data: seeded ground-truth windows produced by the FP64 oracle."""
import numpy as np

from oracle import dynamics as dyn
from oracle import go2_model as gm
from oracle import sysid as osy
from oracle import windows as ow


def random_theta(rng, n):
    return gm.THETA_PRIOR_LO + (gm.THETA_PRIOR_HI - gm.THETA_PRIOR_LO) * rng.random((n, 13))


def oracle_windows(seed, n_traj=2, T=24, H=5, settle=60, sim=None, causal=True, theta=None):
    """Windows (reference dict + packed init/target/actions) from oracle sine trajectories."""
    sim = sim or gm.SimParams()
    rng = np.random.default_rng(seed)
    amp = rng.uniform(0.1, 0.4, (n_traj, 12))
    freq = rng.uniform(1.0, 3.0, (n_traj, 12))
    ph = rng.uniform(0, 2 * np.pi, (n_traj, 12))
    acts = osy.sine_actions(settle + T + 1, amp, freq, ph, sim.control_dt, sim.action_scale, settle=settle)
    th = gm.THETA_NOMINAL if theta is None else theta
    frames = osy.collect(osy.standing_state(n_traj), acts, th, sim)
    trajs = [{k: (v[settle:] if isinstance(v, np.ndarray) and v.ndim and v.shape[0] == settle + T + 1 else v)
              for k, v in f.items()} for f in frames]
    n, ds = ow.load_dataset(trajs, H, causal=causal)
    init = ow.init_states(ds).astype(np.float32)
    target = ow.target_states(ds).astype(np.float32)
    actions = ds["action_sequences"].astype(np.float32)
    return ds, init, actions, target


def state_error(gpu, ref):
    """max over elements of |gpu - ref| / max(|ref|, 1): relative for large values, absolute below 1."""
    gpu = np.asarray(gpu, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    return float(np.max(np.abs(gpu - ref) / np.maximum(np.abs(ref), 1.0)))
