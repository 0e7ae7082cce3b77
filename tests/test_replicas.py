"""Replica mode (replicas only: one independent job per GPU, no data-path collective): the
host bookkeeping -- barrier, slowest-rank time, whole-job rate -- over two gloo ranks on CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from replica_worker import whole_job_rate_worker


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def test_single_process_needs_no_process_group(monkeypatch):
    from spi_gb300 import replicas
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    r = replicas.init()
    assert r.dist is None and r.world == 1 and r.rank == 0
    value, ms = r.whole_job_rate(500.0, 250.0)
    assert ms == 250.0 and value == pytest.approx(2000.0)


def test_whole_job_rate_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    with ctx.Manager() as manager:
        out = manager.dict()
        mp.spawn(whole_job_rate_worker, args=(2, _free_port(), out), nprocs=2, join=True)
        res = dict(out)
    for rank in (0, 1):
        value, ms, rk, world = res[rank]
        assert rk == rank and world == 2
        assert ms == 200.0                              # the slower rank's time on every rank
        assert value == pytest.approx(2 * 1000.0 / 0.2)  # both ranks' units over that time


def test_bench_gpus_2_relaunches_two_ranks():
    """bench.py --gpus 2 started as a plain process runs two ranks itself and reports n_gpus 2
    with the slowest rank's time (the launch check: the same plumbing, a host workload)."""
    import json
    import subprocess
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parent.parent
    env = {k: v for k, v in os.environ.items() if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK")}
    r = subprocess.run([sys.executable, str(root / "bench.py"), "--gpus", "2", "--launch-check", "--steps", "3",
                        "--warmup", "1"], capture_output=True, text=True, timeout=300, env=env, cwd=root)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads([ln for ln in r.stdout.splitlines() if ln.startswith("{")][-1])
    assert line["n_gpus"] == 2
    assert line["value"] == pytest.approx(2 * 8.0 * 3 / (line["slowest_rank_ms"] * 1e-3))
