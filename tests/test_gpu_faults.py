"""Faults handled on the host or as status codes, with no GPU fault: malformed windows, calls
in the wrong order, non-finite inputs, an over-budget job (tests/test_gpu_server.py)."""
import ctypes

import numpy as np
import pytest
import torch

from oracle import go2_model as gm
from helpers import oracle_windows

pytestmark = pytest.mark.gpu


def test_malformed_windows_are_rejected(built):
    from spi_gb300.engine import Engine
    _, init, actions, target = oracle_windows(1, n_traj=1, T=12, H=4)
    e = Engine()
    with pytest.raises(ValueError):
        e.load_windows(torch.from_numpy(init[:-1]), torch.from_numpy(actions), torch.from_numpy(target))
    with pytest.raises(ValueError):
        e.load_windows(torch.from_numpy(init), torch.from_numpy(actions[..., :11]), torch.from_numpy(target))
    d = torch.zeros(1, device="cuda")
    p = ctypes.c_void_p(d.data_ptr())
    assert e.lib.spi_load_windows(e._h, p, p, p, None, 0, 4, ctypes.c_float(0.0)) == -1
    assert e.lib.spi_load_windows(e._h, p, p, p, None, 8, -1, ctypes.c_float(0.0)) == -1
    assert e.lib.spi_load_windows(e._h, None, p, p, None, 8, 4, ctypes.c_float(0.0)) == -1


def test_calls_out_of_order_return_state_errors(built):
    from spi_gb300.engine import Engine
    e = Engine()
    assert e.lib.spi_run(e._h) == -4                  # no windows yet
    _, init, actions, target = oracle_windows(2, n_traj=1, T=12, H=4)
    e.load_windows(torch.from_numpy(init), torch.from_numpy(actions), torch.from_numpy(target))
    assert e.lib.spi_run(e._h) == -4                  # no theta yet
    assert b"spi_set_theta" in e.lib.spi_last_error()


def test_non_finite_window_state_is_counted_not_fatal(built):
    """A NaN in one window's initial state poisons that window's rollouts: the device counts
    them (spi_sync) and the costs carry the NaN; the engine stays usable."""
    from spi_gb300.engine import Engine
    _, init, actions, target = oracle_windows(3, n_traj=1, T=16, H=4)
    bad = init.copy()
    bad[2, 8] = np.nan
    e = Engine()
    th = torch.from_numpy(np.tile(gm.THETA_NOMINAL.astype(np.float32), (5, 1)))
    e.load_windows(torch.from_numpy(bad), torch.from_numpy(actions), torch.from_numpy(target))
    _, cost = e.evaluate(th)
    assert e.sync() == 5                                            # one window x five theta
    assert np.isnan(cost.cpu().numpy()).all()
    e.load_windows(torch.from_numpy(init), torch.from_numpy(actions), torch.from_numpy(target))
    _, cost = e.evaluate(th)
    assert e.sync() == 5 and np.isfinite(cost.cpu().numpy()).all()   # the count is cumulative
