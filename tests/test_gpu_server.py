"""Continuous-batching server: same results alone and in the mix, equal to the single-job engine."""
import numpy as np
import pytest
import torch

from oracle import go2_model as gm
from helpers import oracle_windows

pytestmark = pytest.mark.gpu


def _job(seed, W, H, N, ids, job_id, iters=4):
    from spi_gb300.server import Server, cem_config
    _, init, actions, target = oracle_windows(seed, n_traj=2, T=W // 2 + H + 2, H=H)
    init, actions, target = (torch.from_numpy(a[:W]).cuda() for a in (init, actions, target))
    c = cem_config(N, ids, gm.THETA_PRIOR_LO[ids], gm.THETA_PRIOR_HI[ids], gm.THETA_NOMINAL, seed=100 + seed,
                   job_id=job_id)
    return Server.make_job(init, actions, target, c, iters), (init, actions, target)


def _run(server, jobs):
    for j, _ in jobs:
        assert server.submit(j) is not None
    return server.run_until_done(len(jobs))


def _server(variant="quad3", **kw):
    from spi_gb300.server import Server
    s = Server(**kw)
    s.set_variant(variant)
    return s


@pytest.mark.parametrize("variant", ["quad3", "lane3"])
def test_same_result_alone_and_in_the_mix(built, variant):
    specs = [(1, 24, 5, 64, [0], 11), (2, 40, 9, 128, [0, 4, 5, 6], 12), (3, 16, 3, 96, list(range(13)), 13)]
    mix = _run(_server(variant, max_slots=8, max_samples=256), [_job(*s, iters=4) for s in specs])
    for s in specs:
        alone = _run(_server(variant, max_slots=8, max_samples=256), [_job(*s, iters=4)])[s[-1]]
        r = mix[s[-1]]
        assert r["iterations"] == 4
        assert np.array_equal(r["best_theta"], alone["best_theta"]) and r["best_cost"] == alone["best_cost"]
        assert np.array_equal(r["mu"], alone["mu"])


@pytest.mark.parametrize("variant", ["quad3", "lane3"])
def test_server_job_equals_engine_cem(built, variant):
    """A server job and the single-job engine CEM agree within the 1e-4 relative cost bar.

    The rollouts are the same code; the two cost-finalize kernels may contract the weighted
    sum into FMAs differently, so the last bits of a cost can differ.
    """
    from spi_gb300.cem import CEM
    from spi_gb300.engine import Engine
    from spi_gb300.server import Server
    ids = [0, 1, 2, 4]
    job, (init, actions, target) = _job(4, 32, 6, 128, ids, 21, iters=5)
    r = _run(_server(variant, max_slots=4, max_samples=128), [(job, None)])[21]
    from spi_gb300.autotune import set_variant
    e = Engine()
    e.load_windows(init, actions, target)
    set_variant(e, variant)
    cem = CEM(e, n_samples=128, param_ids=ids, lo=gm.THETA_PRIOR_LO[ids], hi=gm.THETA_PRIOR_HI[ids],
              nominal=gm.THETA_NOMINAL, seed=104, job_id=21)
    for _ in range(5):
        cem.step()
    ref = cem.read()
    np.testing.assert_allclose(r["mu"], ref["mu"], rtol=1e-6)
    assert abs(ref["best_cost"] - r["best_cost"]) <= 1e-4 * abs(ref["best_cost"])


def test_layout_switch_refused_while_jobs_are_held(built):
    from spi_gb300 import _lib
    s = _server("quad3", max_slots=2, max_samples=64)
    job, keep = _job(8, 16, 4, 64, [0], 41)
    assert s.submit(job) is not None
    with pytest.raises(_lib.SpiError):
        s.set_kernel_layout(1)
    s.run_until_done(1)
    s.set_kernel_layout(1)


def test_admission_respects_budget_and_slots(built):
    from spi_gb300.server import Server
    job, keep = _job(5, 16, 4, 64, [0], 31)
    s = Server(max_slots=2, max_samples=64, hbm_budget_bytes=10 << 20)
    need = s.job_bytes(job)
    assert 0 < need < (10 << 20)
    assert s.submit(job) is not None
    job2, keep2 = _job(6, 16, 4, 64, [0], 32)
    assert s.submit(job2) is not None
    job3, keep3 = _job(7, 16, 4, 64, [0], 33)
    assert s.submit(job3) is None                     # no free slot
    small = Server(max_slots=4, max_samples=64, hbm_budget_bytes=need - 1)
    assert small.submit(job) is None                  # over the HBM budget
