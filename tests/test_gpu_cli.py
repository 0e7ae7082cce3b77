"""The command-line identification front end on npz files in the reference's collector format."""
import numpy as np
import pytest

from oracle import go2_model as gm
from oracle import sysid as osy

pytestmark = pytest.mark.gpu


def _write_npz(tmp_path, theta, n_traj=2, T=40, settle=60, seed=0):
    rng = np.random.default_rng(seed)
    sim = gm.SimParams(torque_speed=False)
    acts = osy.sine_actions(settle + T, rng.uniform(0.1, 0.4, (n_traj, 12)), rng.uniform(1, 3, (n_traj, 12)),
                            rng.uniform(0, 6.28, (n_traj, 12)), sim.control_dt, sim.action_scale, settle=settle)
    frames = osy.collect(osy.standing_state(n_traj), acts, theta, sim)
    paths = []
    for k, f in enumerate(frames):
        d = {kk: (v[settle:] if isinstance(v, np.ndarray) and v.ndim and v.shape[0] == settle + T else v)
             for kk, v in f.items()}
        p = tmp_path / f"traj{k}.npz"
        np.savez(p, **d)
        paths.append(str(p))
    return paths


def test_landscape_and_identify(built, tmp_path):
    from spi_gb300 import cli
    true = gm.THETA_NOMINAL.copy()
    true[0] = 6.921 * 1.2
    paths = _write_npz(tmp_path, true)
    out = cli.main(["landscape", "--data", *paths, "--horizon", "5", "--out", str(tmp_path)])
    text = (out / "landscape_results.txt").read_text()
    assert "Optimal base mass" in text and len(text.splitlines()) > 25
    out, r = cli.main(["identify", "--data", *paths, "--horizon", "5", "--params", "0", "--samples", "256",
                       "--iterations", "8", "--causal", "--out", str(tmp_path)])
    assert abs(r["best_theta"][0] - true[0]) < 0.05
    assert (out / "optimization_results.txt").exists()
