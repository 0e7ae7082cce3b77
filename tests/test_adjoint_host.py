"""The hand-written adjoint of the rollout (csrc/adjoint.cuh), built for the host in FP64, against
central finite differences of the same host build of the kernel's dynamics (no GPU needed).

* The equations-of-motion residual r(x, theta, a) the reverse sweep differentiates vanishes at
  the accelerations the forward substep computes (the residual is the forward's model).
* d cost / d theta by the adjoint equals central differences (h = 1e-6 relative) of the FP64
  rollout's cost to 1e-6 of the gradient's size, for both cost modes, at H = 5 and H = 20.
"""
import ctypes

import numpy as np
import pytest

from helpers import oracle_windows, random_theta


@pytest.fixture(scope="module")
def emu(built):
    from spi_gb300 import _lib
    from spi_gb300 import robot as rb
    return _lib.hostemu_lib(), rb.to_struct(rb.SimConfig())


def _qw():
    return np.concatenate([np.full(n, w) for n, w in zip((3, 4, 3, 3, 12, 12), (10, 5, 0.1, 0.1, 1, 0.01))])


def _rollout_cost(lib, robot, init, actions, theta, target, mode):
    W, H = actions.shape[:2]
    tr = np.zeros((W, H, 37))
    rc = lib.spi_hostemu_rollout(ctypes.byref(robot), init.ctypes.data, actions.ctypes.data,
                                 np.ascontiguousarray(theta).ctypes.data, W, H, tr.ctypes.data)
    assert rc == 0
    d = tr[:, -1] - target
    if mode == 1:
        return (_qw() * d * d).sum(1)
    return (10 * np.linalg.norm(d[:, 0:3], axis=1) + 5 * np.linalg.norm(d[:, 3:7], axis=1)
            + np.linalg.norm(d[:, 13:25], axis=1))


def test_residual_vanishes_at_the_forward_accelerations(emu):
    lib, robot = emu
    rng = np.random.default_rng(3)
    _, init, actions, _ = oracle_windows(3, n_traj=2, T=24, H=5)
    th = random_theta(rng, 8)
    for w in range(8):
        out = np.zeros(18)
        x = init[w].astype(np.float64)
        a = actions[w, 0].astype(np.float64)
        assert lib.spi_hostemu_residual(ctypes.byref(robot), x.ctypes.data, th[w].ctypes.data, a.ctypes.data,
                                        out.ctypes.data) == 0
        assert np.abs(out).max() <= 1e-9, np.abs(out).max()


@pytest.mark.parametrize("H,mode", [(5, 1), (20, 1), (20, 0)])
def test_adjoint_matches_central_differences(emu, H, mode):
    lib, robot = emu
    rng = np.random.default_rng(10 + H + mode)
    _, init, actions, target = oracle_windows(4 + H, n_traj=2, T=H + 12, H=H)
    W = 6
    sel = rng.choice(init.shape[0], W, replace=False)
    init = init[sel].astype(np.float64)
    actions = actions[sel].astype(np.float64)
    target = target[sel].astype(np.float64) + 0.01 * rng.standard_normal((W, 37))
    th = random_theta(rng, W)
    cost = np.zeros(W)
    grad = np.zeros((W, 13))
    assert lib.spi_hostemu_grad(ctypes.byref(robot), init.ctypes.data, actions.ctypes.data, th.ctypes.data,
                                target.ctypes.data, _qw().ctypes.data, mode, W, H, cost.ctypes.data,
                                grad.ctypes.data) == 0
    np.testing.assert_allclose(cost, _rollout_cost(lib, robot, init, actions, th, target, mode), rtol=1e-12)
    fd = np.zeros((W, 13))
    for k in range(13):
        h = 1e-6 * max(1.0, abs(th[0, k]))
        tp, tm = th.copy(), th.copy()
        tp[:, k] += h
        tm[:, k] -= h
        fd[:, k] = (_rollout_cost(lib, robot, init, actions, tp, target, mode)
                    - _rollout_cost(lib, robot, init, actions, tm, target, mode)) / (2 * h)
    rel = np.abs(grad - fd).max(1) / np.abs(fd).max(1)
    assert rel.max() <= 1e-6, rel
