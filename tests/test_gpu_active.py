"""The reference's finite-difference Fisher objective on the engine (spi_fd_fisher) against the
FP64 oracle's restatement of the reference episode, and the device-CEM excitation search.

Tolerance: the objective is a sum of squared finite differences (s_main - s_aux) / delta of
FP32 states, so FP32 rounding of the states (<= 1e-4 relative) reaches it amplified by
|s| / |s_main - s_aux|. Per-step rewards agree within 2 % of the largest reward of the
candidate's episode and episode objectives within 1 %, well inside the spread between
candidates that the search ranks (tens of percent and more).
"""
import numpy as np
import pytest
import torch

from oracle import fisher as ofi
from oracle import go2_model as gm
from oracle import sysid as osy

pytestmark = pytest.mark.gpu


def _case(C, n, seed):
    from spi_gb300.sensitivity import multisine_actions
    sim = gm.SimParams()
    acts, _ = multisine_actions(C, n, sim.control_dt, sim.action_scale, seed=seed)
    x0 = osy.standing_state(C, z=0.32).astype(np.float32)
    return x0, acts


@pytest.mark.parametrize("param_ids,ksync,delta", [([0, 1], 5, 0.1), (list(range(13)), 1, 0.1),
                                                   ([0, 4, 7, 10], 3, 0.05), ([0, 2], -1, 0.1)])
def test_fd_fisher_matches_oracle_episode(built, param_ids, ksync, delta):
    from spi_gb300.active import fd_fisher
    from spi_gb300.engine import Engine
    C, n = 5, 12
    x0, acts = _case(C, n, seed=len(param_ids) + ksync)
    eng = Engine()
    obj, per = fd_fisher(eng, torch.from_numpy(x0), torch.from_numpy(acts), gm.THETA_NOMINAL.astype(np.float32),
                         param_ids, delta=delta, ksync=ksync, trace=True)
    torch.cuda.synchronize()
    ref_obj, ref_per = ofi.fd_fisher_episode(x0, acts, gm.THETA_NOMINAL, param_ids, delta, ksync, gm.SimParams())
    per = per.cpu().numpy().astype(np.float64)
    obj = obj.cpu().numpy().astype(np.float64)
    scale = np.abs(ref_per).max(1, keepdims=True)
    step_err = float(np.max(np.abs(per - ref_per) / scale))
    obj_err = float(np.max(np.abs(obj - ref_obj) / np.abs(ref_obj)))
    assert step_err <= 2e-2, (step_err, obj_err)
    assert obj_err <= 1e-2, (step_err, obj_err)
    assert np.all(ref_per >= 0) and np.all(np.isfinite(per))


def test_fd_fisher_group_packing_is_independent_of_the_batch(built):
    """A candidate's objective does not depend on which other candidates share its CTA."""
    from spi_gb300.active import fd_fisher
    from spi_gb300.engine import Engine
    x0, acts = _case(7, 10, seed=3)
    eng = Engine()
    ids = [0, 1, 2, 3, 4]
    all7 = fd_fisher(eng, x0, acts, gm.THETA_NOMINAL.astype(np.float32), ids).cpu().numpy()
    sub = fd_fisher(eng, x0[[6, 2]], acts[[6, 2]], gm.THETA_NOMINAL.astype(np.float32), ids).cpu().numpy()
    np.testing.assert_array_equal(sub, all7[[6, 2]])


def test_fd_fisher_rejects_bad_arguments(built):
    from spi_gb300 import _lib
    from spi_gb300.active import fd_fisher
    from spi_gb300.engine import Engine
    x0, acts = _case(2, 4, seed=1)
    eng = Engine()
    with pytest.raises(_lib.SpiError):
        fd_fisher(eng, x0, acts, gm.THETA_NOMINAL.astype(np.float32), [0, 0])          # repeated slot
    with pytest.raises(_lib.SpiError):
        fd_fisher(eng, x0, acts, gm.THETA_NOMINAL.astype(np.float32), [13])            # no such slot
    with pytest.raises(_lib.SpiError):
        fd_fisher(eng, x0, acts, gm.THETA_NOMINAL.astype(np.float32), [0], delta=0.0)


def test_device_search_finds_a_known_optimum(built):
    """spi_search refit from caller costs: a quadratic bowl's minimum is found."""
    from spi_gb300.active import DeviceSearch
    lo, hi = np.zeros(4), np.ones(4)
    target = torch.tensor([0.2, 0.7, 0.4, 0.9], device="cuda")
    s = DeviceSearch(512, lo, hi, elite_frac=0.1, alpha=1.0, min_std_frac=1e-4, seed=7)
    for _ in range(25):
        pop = s.sample()
        cost = ((pop[:, :4] - target) ** 2).sum(1)
        s.refit(cost)
    r = s.read()
    assert r["iteration"] == 25
    np.testing.assert_allclose(r["mu"], target.cpu().numpy(), atol=5e-3)
    assert r["best_cost"] < 1e-3
    s.close()


def test_excitation_search_improves_the_reference_objective(built):
    """The device-CEM search over the group multi-sine family raises the FD-Fisher objective of
    base mass over its first iteration, and its reported best re-scores to the same value."""
    from spi_gb300.active import excitation_search, fd_fisher
    from spi_gb300.data import standing_state
    from spi_gb300.engine import Engine
    eng = Engine()
    r = excitation_search(eng, n_candidates=64, iterations=5, steps=40, param_ids=(0,), seed=3)
    it = r["per_iteration"]
    assert len(it) == 5 and all(np.isfinite(x["best"]) for x in it)
    assert r["best_objective"] >= it[0]["best"]
    assert it[-1]["mean"] > it[0]["mean"]
    acts = r["family"].actions(torch.from_numpy(r["best_params"][None]).cuda(), 40, eng.cfg.control_dt,
                               eng.cfg.action_scale)
    again = fd_fisher(eng, standing_state(1, z=0.32), acts, gm.THETA_NOMINAL.astype(np.float32), (0,))
    assert float(again[0]) == pytest.approx(r["best_objective"], rel=1e-6)
