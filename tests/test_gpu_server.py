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


@pytest.mark.parametrize("variant", ["quad3", "lane4"])
def test_same_result_alone_and_in_the_mix(built, variant):
    specs = [(1, 24, 5, 64, [0], 11), (2, 40, 9, 128, [0, 4, 5, 6], 12), (3, 16, 3, 96, list(range(13)), 13)]
    mix = _run(_server(variant, max_slots=8, max_samples=256), [_job(*s, iters=4) for s in specs])
    for s in specs:
        alone = _run(_server(variant, max_slots=8, max_samples=256), [_job(*s, iters=4)])[s[-1]]
        r = mix[s[-1]]
        assert r["iterations"] == 4
        assert np.array_equal(r["best_theta"], alone["best_theta"]) and r["best_cost"] == alone["best_cost"]
        assert np.array_equal(r["mu"], alone["mu"])


def _engine_cem(variant, init, actions, target, n, ids, seed, job_id, iters, cost=None):
    from spi_gb300.autotune import set_variant
    from spi_gb300.cem import CEM
    from spi_gb300.engine import Engine
    e = Engine()
    e.load_windows(init, actions, target)
    set_variant(e, variant)
    if cost is not None:
        e.set_cost(*cost)
    cem = CEM(e, n_samples=n, param_ids=ids, lo=gm.THETA_PRIOR_LO[ids], hi=gm.THETA_PRIOR_HI[ids],
              nominal=gm.THETA_NOMINAL, seed=seed, job_id=job_id)
    cem.run(iters, graph=True)
    return cem.read()


def _assert_same(r, ref):
    assert r["iterations"] == ref["iteration"]
    assert r["best_cost"] == ref["best_cost"], (r["best_cost"], ref["best_cost"])
    assert np.array_equal(r["best_theta"], ref["best_theta"])
    assert np.array_equal(r["mu"], ref["mu"])


@pytest.mark.parametrize("variant", ["quad3", "lane4"])
def test_server_job_equals_engine_cem(built, variant):
    """A server job and the single-job engine CEM give bitwise-identical results: both launch
    the one compiled rollout kernel of items.cu (the engine on a table of one slot) and share
    the finalize, sample and refit code."""
    ids = [0, 1, 2, 4]
    job, (init, actions, target) = _job(4, 32, 6, 128, ids, 21, iters=5)
    r = _run(_server(variant, max_slots=4, max_samples=128), [(job, None)])[21]
    _assert_same(r, _engine_cem(variant, init, actions, target, 128, ids, 104, 21, 5))


@pytest.mark.parametrize("mode,weights", [(0, (10.0, 5.0, 0.1, 0.1, 1.0, 0.01)), (1, (3.0, 2.0, 0.5, 0.2, 4.0, 0.1))])
def test_server_cost_settings_equal_engine_cem(built, mode, weights):
    """The reference's norm cost (mode 0) and non-default squared-error weights: a server job
    equals the engine CEM under the same cost settings bit for bit."""
    from spi_gb300.server import Server
    ids = [0, 3, 5, 9]
    job, (init, actions, target) = _job(6, 29, 5, 96, ids, 31, iters=4)
    srv = Server(max_slots=2, max_samples=128, cost_mode=mode, sq_weights=weights)
    srv.set_variant("lane3")
    r = _run(srv, [(job, None)])[31]
    _assert_same(r, _engine_cem("lane3", init, actions, target, 96, ids, 106, 31, 4, cost=(mode, weights)))


@pytest.mark.parametrize("variant", ["quad3", "lane4"])
def test_served_equals_plain_with_more_jobs_than_slots(built, variant):
    """Eleven jobs of uneven population, ragged window counts, horizons and parameter sets
    through a three-slot server under a small work cap (jobs wait, slots are reused, several
    rounds per tick) equal the same jobs run one at a time on the engine, bit for bit."""
    rng = np.random.default_rng(8)
    specs = []
    for k in range(11):
        W = int(rng.integers(5, 70))
        H = int(rng.integers(2, 9))
        N = int(rng.choice([32, 96, 160, 256]))
        P = int(rng.integers(1, 14))
        ids = sorted(rng.choice(13, P, replace=False).tolist())
        specs.append((20 + k, W, H, N, ids, 40 + k, int(rng.integers(1, 4))))
    jobs = {s[5]: _job(*s[:6], iters=s[6]) for s in specs}
    srv = _server(variant, max_slots=3, max_samples=256)
    srv.set_rounds(3)
    srv.set_work_cap(64)
    pending = list(jobs)
    out = {}
    while len(out) < len(jobs):
        while pending and srv.submit(jobs[pending[0]][0]) is not None:
            pending.pop(0)
        active, _ = srv.stats()
        srv.tick()
        if not active:
            srv.wait()
        for r in srv.poll():
            out[r["job_id"]] = r
    for seed, W, H, N, ids, job_id, iters in specs:
        init, actions, target = jobs[job_id][1]
        _assert_same(out[job_id], _engine_cem(variant, init, actions, target, N, ids, 100 + seed, job_id, iters))


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


@pytest.mark.parametrize("variant", ["quad3", "lane4"])
def test_rounds_per_tick_do_not_change_results(built, variant):
    """Jobs advanced several CEM iterations per tick reach bitwise the same results."""
    specs = [(9, 64, 12, 256, [0, 4], 51), (10, 8, 3, 64, [0], 52), (11, 16, 5, 64, [0, 1, 2], 53)]
    res = {}
    for rounds in (1, 4):
        s = _server(variant, max_slots=8, max_samples=256)
        s.set_rounds(rounds)
        res[rounds] = _run(s, [_job(*sp, iters=9) for sp in specs])
    for sp in specs:
        a, b = res[1][sp[-1]], res[4][sp[-1]]
        assert a["iterations"] == b["iterations"] == 9
        assert np.array_equal(a["best_theta"], b["best_theta"]) and a["best_cost"] == b["best_cost"]
        assert np.array_equal(a["mu"], b["mu"])


@pytest.mark.parametrize("variant", ["quad3", "lane4"])
def test_launch_shape_does_not_change_results(built, variant):
    """A rollout launch capped at one CTA per SM (each warp then takes many work items) and
    three items per claim reach bitwise the same results as one warp per item."""
    specs = [(9, 64, 12, 256, [0, 4], 51), (12, 40, 7, 128, list(range(13)), 54)]
    res = {}
    for shape in ((0, 1), (1, 3)):
        s = _server(variant, max_slots=8, max_samples=256)
        s.config(*shape)
        res[shape] = _run(s, [_job(*sp, iters=3) for sp in specs])
    for sp in specs:
        a, b = res[(0, 1)][sp[-1]], res[(1, 3)][sp[-1]]
        assert a["iterations"] == b["iterations"] == 3
        assert np.array_equal(a["best_theta"], b["best_theta"]) and a["best_cost"] == b["best_cost"]
        assert np.array_equal(a["mu"], b["mu"])


def test_small_job_takes_several_iterations_per_tick(built):
    """Beside a job with 64x its work per iteration, a small job takes 4 iterations per tick."""
    s = _server("lane4", max_slots=4, max_samples=512)
    s.set_rounds(4)
    big, keep_big = _job(12, 128, 16, 512, [0, 4], 61, iters=12)
    small, keep_small = _job(13, 8, 2, 64, [0], 62, iters=12)
    assert s.submit(big) is not None and s.submit(small) is not None
    ticks, done = 0, {}
    while len(done) < 2:
        s.tick()
        ticks += 1
        s.wait()
        for r in s.poll():
            done[r["job_id"]] = ticks
        assert ticks < 40
    assert done[62] <= 12 // 4 + 2 < done[61]


def test_work_cap_runs_shortest_remaining_work_first(built):
    """Past the work cap jobs wait resident; the job with the least remaining work ticks first."""
    s = _server("quad3", max_slots=4, max_samples=256)
    s.set_work_cap(3000)
    big, keep_big = _job(14, 64, 4, 256, [0], 71, iters=8)       # 256 theta x 8 groups = 2048 items
    big2, keep_big2 = _job(15, 64, 4, 256, [0], 72, iters=8)
    assert s.submit(big) is not None
    s.tick()                                             # job 71 starts alone
    small, keep_small = _job(16, 8, 4, 32, [0], 73, iters=8)    # 32 items
    assert s.submit(big2) is not None and s.submit(small) is not None
    order, ticks = [], 0
    while len(order) < 3:
        s.tick()
        ticks += 1
        s.wait()
        order += [r["job_id"] for r in s.poll()]
        assert ticks < 60
    # 71 (less remaining than 72) and the small 73 run together; 72 waits for 71
    assert order.index(73) < order.index(72) and order.index(71) < order.index(72)
