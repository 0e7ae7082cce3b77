"""Multi-job identification workloads: uneven job mixes, served (batched) vs plain (one job at a time).

* ``c2_specs`` draws jobs the way the uneven-batch workload describes them: population
  U{256..4096}, windows U{16..512}, horizon U{5..50}, parameter dimension U{1..13} on the full
  13-parameter model and priors, FP32, 30 CEM iterations each.
* ``run_served`` admits jobs into the continuous-batching server as they arrive (all at t=0
  for the batch workload, Poisson arrivals for the stream) and ticks until every job is done.
* ``run_plain`` runs the same jobs one after another through the single-job engine (one
  job per launch sequence, CUDA-graph iterations), in arrival order.
Both report aggregate rollout-steps/s and per-job latency (completion - arrival).
"""
from __future__ import annotations

import time
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass

import numpy as np
import torch

from .cem import CEM
from .data import synthetic_windows
from .engine import Engine
from .robot import THETA_NOMINAL, THETA_PRIOR_HI, THETA_PRIOR_LO, SimConfig
from .server import Server, cem_config


@dataclass
class JobSpec:
    job_id: int
    n_samples: int
    n_windows: int
    horizon: int
    param_ids: list
    iterations: int
    seed: int
    theta_true: np.ndarray
    arrival: float = 0.0
    fisher: bool = False      # also score candidate excitations at the identified theta

    @property
    def rollout_steps(self) -> int:
        return self.n_samples * self.n_windows * self.horizon * self.iterations


def c2_specs(n_jobs, seed=0, iterations=30, pop=(256, 4096), windows=(16, 512), horizon=(5, 50), dims=(1, 13)):
    rng = np.random.default_rng(seed)
    specs = []
    for j in range(n_jobs):
        P = int(rng.integers(dims[0], dims[1] + 1))
        ids = sorted(rng.choice(13, P, replace=False).tolist())
        true = THETA_NOMINAL.copy()
        true[ids] = THETA_PRIOR_LO[ids] + (THETA_PRIOR_HI[ids] - THETA_PRIOR_LO[ids]) * rng.random(P)
        specs.append(JobSpec(j, int(rng.integers(pop[0], pop[1] + 1)), int(rng.integers(windows[0], windows[1] + 1)),
                             int(rng.integers(horizon[0], horizon[1] + 1)), ids, iterations, 1000 + j, true))
    return specs


def small_specs(n_jobs, seed=0, iterations=30):
    """Small jobs (population U{64..512}, windows U{8..64}, horizon U{5..20}): each alone leaves
    most of the GPU idle, the regime continuous batching is for."""
    return c2_specs(n_jobs, seed=seed, iterations=iterations, pop=(64, 512), windows=(8, 64), horizon=(5, 20))


def poisson_arrivals(specs, rate, seed=0, fisher_frac=0.0):
    """Poisson arrival times at `rate` jobs/s; a `fisher_frac` share of jobs also asks for an
    excitation score."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, len(specs)))
    for s, a in zip(specs, t):
        s.arrival = float(a)
        s.fisher = bool(rng.random() < fisher_frac)
    return specs


FISHER_CANDIDATES, FISHER_WINDOWS, FISHER_H = 32, 4, 20


class FisherScorer:
    """Excitation scoring at an identified theta (the Fisher request of a job).

    With ``own_stream`` the scorer's engine and its torch work run on a private stream, so that
    a worker thread can score while the caller keeps feeding the server."""

    def __init__(self, cfg: SimConfig | None = None, device=None, own_stream=False):
        from .sensitivity import multisine_actions
        self.stream = torch.cuda.Stream(device=device) if own_stream else None
        self.engine = Engine(cfg, device=device, stream=self.stream)
        c = self.engine.cfg
        acts, _ = multisine_actions(FISHER_CANDIDATES, FISHER_WINDOWS * FISHER_H, c.control_dt, c.action_scale,
                                    seed=11, settle=100)
        self.actions = torch.from_numpy(acts).to(self.engine.device)   # resident on the device

    def score(self, theta):
        from .sensitivity import score_excitations
        if self.stream is not None:
            with torch.cuda.stream(self.stream):
                r = score_excitations(self.engine, theta, self.actions, windows_per_cand=FISHER_WINDOWS,
                                      horizon=FISHER_H, settle=100)
        else:
            r = score_excitations(self.engine, theta, self.actions, windows_per_cand=FISHER_WINDOWS, horizon=FISHER_H,
                                  settle=100)
        return {"best_candidate": r["best"], "logdet": float(r["logdet"][r["best"]])}


class WindowBank:
    """Ground-truth windows per job, generated on the GPU (each job its own theta and seed)."""

    def __init__(self, cfg: SimConfig | None = None, device=None):
        self.engine = Engine(cfg, device=device)
        self.cache = {}

    def get(self, spec: JobSpec):
        key = spec.job_id
        if key not in self.cache:
            init, act, tgt = synthetic_windows(self.engine, spec.theta_true, spec.n_windows, spec.horizon,
                                               n_traj=4, seed=spec.seed)
            dev = self.engine.device
            self.cache[key] = tuple(torch.from_numpy(a).to(dev) for a in (init, act, tgt))
        return self.cache[key]


def _cem_cfg(spec: JobSpec):
    ids = spec.param_ids
    return cem_config(spec.n_samples, ids, THETA_PRIOR_LO[ids], THETA_PRIOR_HI[ids], THETA_NOMINAL,
                      seed=spec.seed, job_id=spec.job_id)


def _summary(specs, latencies, wall, results=None):
    steps = sum(s.rollout_steps for s in specs)
    lat = np.array([latencies[s.job_id] for s in specs])
    out = {"jobs": len(specs), "rollout_steps": int(steps), "wall_s": wall, "rollout_steps_per_s": steps / wall,
           "latency_p50_s": float(np.percentile(lat, 50)), "latency_p99_s": float(np.percentile(lat, 99)),
           "latency_mean_s": float(lat.mean())}
    out["latencies"] = {s.job_id: float(latencies[s.job_id]) for s in specs}
    if results is not None:
        out["results"] = results
    return out


def default_work_cap(device=None):
    """Work items (8-window warps) that keep every SM busy for ~8 waves of resident warps."""
    props = torch.cuda.get_device_properties(device or torch.cuda.current_device())
    return 8 * props.multi_processor_count * 12


def run_served(specs, bank: WindowBank, cfg: SimConfig | None = None, max_slots=64, hbm_budget=150 << 30,
               ctas_per_sm=0, items_per_claim=1, realtime=True, work_cap=None, variant="lane3", rounds=4,
               timeline=True):
    """Continuous batching: admit on arrival while HBM budget, a slot and GPU work capacity are free;
    every tick advances each admitted job by 1 .. `rounds` CEM iterations (more for smaller jobs). Fisher requests are scored on a worker
    thread (own engine and stream) while the server keeps ticking; a job completes when its
    score is in.

    timeline: CUDA events on the server stream around every tick's launches give the GPU time
    of each tick and the idle gaps between consecutive ticks, i.e. how long the GPU waited for
    the host loop (admission, tick set-up, result polling); reported as ``timeline``."""
    max_samples = max(s.n_samples for s in specs)
    server = Server(cfg, max_slots=max_slots, max_samples=max_samples, hbm_budget_bytes=hbm_budget,
                    device=bank.engine.device)
    server.set_variant(variant)
    server.set_rounds(rounds)
    server.config(ctas_per_sm, items_per_claim)
    server.set_work_cap(default_work_cap(bank.engine.device) if work_cap is None else work_cap)
    jobs = {}
    for s in specs:                       # windows ready before the clock starts
        init, act, tgt = bank.get(s)
        jobs[s.job_id] = (Server.make_job(init, act, tgt, _cem_cfg(s), s.iterations), (init, act, tgt))
    pending = sorted(specs, key=lambda s: s.arrival)
    scorer = FisherScorer(cfg, device=bank.engine.device, own_stream=True) if any(s.fisher for s in specs) else None
    if scorer is not None:
        scorer.score(THETA_NOMINAL)       # first-call setup (allocations, attributes) before the clock
    pool = ThreadPoolExecutor(max_workers=1) if scorer is not None else None
    by_id = {s.job_id: s for s in specs}
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    done, lat, results, scoring = 0, {}, {}, []
    qi = 0
    marks = []                            # (event before, event after) each tick's launches

    def _score(job_id, theta, arrival):
        with torch.cuda.device(bank.engine.device):
            out = scorer.score(theta)
        lat[job_id] = time.perf_counter() - t0 - arrival
        return job_id, out

    while done < len(specs):
        now = time.perf_counter() - t0
        while qi < len(pending) and (pending[qi].arrival <= now or not realtime):
            spec = pending[qi]
            if server.submit(jobs[spec.job_id][0]) is None:
                break                     # no slot / budget: wait for a retirement
            qi += 1
        active, _ = server.stats()
        if timeline and active:
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(server.stream)
            server.tick()
            e1.record(server.stream)
            marks.append((e0, e1))
        else:
            server.tick()
        if not active:
            server.wait()
            if qi < len(pending) and realtime:
                time.sleep(max(0.0, min(pending[qi].arrival - (time.perf_counter() - t0), 0.002)))
        for r in server.poll():
            spec = by_id[r["job_id"]]
            if spec.fisher:
                scoring.append(pool.submit(_score, r["job_id"], r["best_theta"], spec.arrival))
            else:
                lat[r["job_id"]] = time.perf_counter() - t0 - spec.arrival
            results[r["job_id"]] = r
            done += 1
    for f in scoring:
        job_id, out = f.result()
        results[job_id]["fisher"] = out
    wall = time.perf_counter() - t0
    if pool is not None:
        pool.shutdown()
    server.close()
    out = _summary(specs, lat, wall, results)
    if timeline and marks:
        torch.cuda.synchronize()
        busy = [a.elapsed_time(b) for a, b in marks]
        gaps = [marks[k][1].elapsed_time(marks[k + 1][0]) for k in range(len(marks) - 1)]
        span = marks[0][0].elapsed_time(marks[-1][1])
        out["timeline"] = {"ticks": len(marks), "gpu_tick_ms_median": float(np.median(busy)),
                           "gpu_busy_ms": float(np.sum(busy)), "gpu_idle_gaps_ms": float(np.sum(gaps)),
                           "max_gap_ms": float(np.max(gaps)) if gaps else 0.0,
                           "idle_fraction": float(np.sum(gaps) / span) if span > 0 else 0.0,
                           "host_loop_ms_per_tick": wall * 1e3 / len(marks),
                           "note": "CUDA events on the server stream before and after each spi_server_tick "
                                   "call; a gap is GPU time between the end of one tick's work and the host "
                                   "loop's next tick call (admission, polling, Fisher hand-off), i.e. GPU time "
                                   "lost to the host loop; the tick call's own table staging (tens of us) counts "
                                   "as tick time. In a real-time stream, jobs that arrive after the GPU frees up "
                                   "also show as gaps"}
    return out


def run_plain(specs, bank: WindowBank, cfg: SimConfig | None = None, graph=True, variant="lane3"):
    """One job at a time through the single-job engine, in arrival order (FIFO), with the
    rollout-kernel variant the server runs (lane layout, 3 CTAs per SM by default)."""
    from .autotune import set_variant
    eng = Engine(cfg, device=bank.engine.device)
    set_variant(eng, variant)
    scorer = FisherScorer(cfg, device=bank.engine.device) if any(s.fisher for s in specs) else None
    if scorer is not None:
        scorer.score(THETA_NOMINAL)       # first-call setup (allocations, attributes) before the clock
    order = sorted(specs, key=lambda s: s.arrival)
    for s in order:
        bank.get(s)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    lat, results = {}, {}
    for s in order:
        now = time.perf_counter() - t0
        if s.arrival > now:
            time.sleep(s.arrival - now)
        init, act, tgt = bank.get(s)
        eng.load_windows(init, act, tgt)
        ids = s.param_ids
        cem = CEM(eng, s.n_samples, ids, THETA_PRIOR_LO[ids], THETA_PRIOR_HI[ids], THETA_NOMINAL, seed=s.seed,
                  job_id=s.job_id)
        cem.run(s.iterations, graph=graph)
        r = cem.read()
        if s.fisher:
            r["fisher"] = scorer.score(r["best_theta"])
        lat[s.job_id] = time.perf_counter() - t0 - s.arrival
        results[s.job_id] = r
    wall = time.perf_counter() - t0
    return _summary(specs, lat, wall, results)
