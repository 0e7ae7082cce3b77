"""The product's npz format and window loader (spi_gb300.data) against the reference's own output.

The golden file tests/golden/dataset.npz holds trajectories written by the reference's
format_data (scripts/data/common.py:83-100) and the windows its load_dataset
(scripts/eval.py:101-171) built from them. These tests run the product code, not the oracle,
on the same inputs; they need no GPU.
"""
import numpy as np

from spi_gb300 import data as sd
from spi_gb300.robot import SimConfig

STATE_KEYS = ("base_positions", "base_orientations", "base_linear_velocities", "base_angular_velocities",
              "joint_positions", "joint_velocities")


def _trajs(g):
    out = []
    for k in range(int(g["n_traj"])):
        pre = f"traj{k}_"
        out.append({key[len(pre):]: g[key] for key in g.files if key.startswith(pre)})
    return out


def test_product_load_dataset_matches_reference(golden):
    g = golden("dataset")
    n, ds = sd.load_dataset(_trajs(g), int(g["horizon"]))
    assert n == int(g["n"])
    for key in g.files:
        if key.startswith("ds_"):
            assert ds[key[3:]].dtype == g[key].dtype, key
            np.testing.assert_array_equal(ds[key[3:]], g[key], err_msg=key)


def test_product_load_dataset_from_npz_files(golden, tmp_path):
    """The same windows when the trajectories come from npz files on disk."""
    g = golden("dataset")
    paths = []
    for k, t in enumerate(_trajs(g)):
        p = tmp_path / f"traj{k}.npz"
        sd.save_npz(p, t)
        paths.append(p)
    n, ds = sd.load_dataset(paths, int(g["horizon"]))
    assert n == int(g["n"])
    for key in g.files:
        if key.startswith("ds_"):
            np.testing.assert_array_equal(ds[key[3:]], g[key], err_msg=key)


def test_product_format_data_matches_reference(golden):
    """format_data from states and actions gives the reference's npz keys and values."""
    g = golden("dataset")
    cfg = SimConfig(sim_dt=0.005, decimation=4)          # the golden trajectories were logged at 50 Hz
    for t in _trajs(g):
        states = np.concatenate([t[k] for k in STATE_KEYS], -1)
        d = sd.format_data(states, t["actions"], cfg)
        for key, want in t.items():
            if key == "joint_torques":                  # the product's collector logs no torques
                continue
            got = np.asarray(d[key])
            if key == "timestamps":
                np.testing.assert_allclose(got, want, rtol=0, atol=1e-12)
            elif key == "sim_duration":
                assert abs(float(got) - float(want)) <= 1e-12
            else:
                assert got.shape == np.asarray(want).shape, key
                np.testing.assert_array_equal(got, want, err_msg=key)
        assert d["robot_type"] == "go2"


def test_eval_weights_chunk_mask():
    """Windows at and after the first motion end of each chunk weigh 0; the normaliser counts
    the non-end windows (scripts/eval.py:279-280, 304)."""
    me = np.zeros(23, dtype=bool)
    me[[6, 14, 22]] = True
    w, n = sd.eval_weights(me, 8)
    want = np.ones(23, dtype=np.float32)
    want[6:8] = 0          # chunk 0..7: end at 6
    want[14:16] = 0        # chunk 8..15: end at 14
    want[22] = 0           # chunk 16..22: end at 22
    np.testing.assert_array_equal(w, want)
    assert n == 20
