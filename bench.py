"""Benchmark of the batched candidate-evaluation engine (one JSON line on stdout).

Workload (default, "c1"): full 13-parameter identification of the Go2 model in FP32,
4096 theta samples x 256 logged windows x horizon 20 control steps (4 physics
substeps each) per CEM iteration; ground truth drawn from the parameter priors with a
fixed seed and generated on the GPU (synthetic data: the reference's logged datasets
are not available). One bench step is one CEM iteration: rollouts + windowed cost +
elite refit + resampling, all on the device.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

``--impl reference`` times the reference path's CPU restatement (the FP64 NumPy
oracle; Isaac Gym cannot be installed) on the host cores on a bounded sample of the
same workload. With N > 1 every rank runs an independent replica job (the path has no
cross-job exchange) and rank 0 prints; ``--gpus N`` started as a plain process relaunches
itself under torch.distributed.run with N ranks. ``--launch-check`` runs only that replica
plumbing (ranks, barrier, slowest-rank time) on a fixed host workload, without a GPU.
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
for _p in (ROOT, ROOT / "spi-active_gb300"):
    if str(_p) not in sys.path:
        sys.path.insert(0, str(_p))

METRIC = "rollout-steps/s"
C1 = dict(n_theta=4096, n_windows=256, horizon=20, n_params=13, iterations=30, elite_frac=0.1)


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--workload", choices=("c1", "c2", "c3", "c4", "rollout-case"), default="c1")
    ap.add_argument("--variant", default="lane4", help="rollout-case: rollout-kernel variant")
    ap.add_argument("--c1-variant", default="auto",
                    help="c1: rollout-kernel variant, or auto to time every variant on the workload first (under a "
                         "profiler the timings that pick it are distorted: fix the variant the plain run chose)")
    ap.add_argument("--n-theta", type=int, default=1024, help="rollout-case: theta samples")
    ap.add_argument("--n-windows", type=int, default=256, help="rollout-case: windows")
    ap.add_argument("--horizon", type=int, default=20, help="rollout-case: control steps per window")
    ap.add_argument("--runs", type=int, default=3, help="rollout-case: launches, the last one timed")
    ap.add_argument("--c3-candidates", type=int, default=512, help="c3: candidate excitations scored per step")
    ap.add_argument("--no-serving", action="store_true", help="c1: skip the served-vs-plain job mix")
    ap.add_argument("--mix-jobs", type=int, default=64, help="c1: jobs in each served-vs-plain mix")
    ap.add_argument("--mix-iters", type=int, default=30, help="c1: CEM iterations per job in the mixes")
    ap.add_argument("--c2-jobs", type=int, default=64)
    ap.add_argument("--c4-rate", type=float, default=200.0, help="c4: arrivals per second")
    ap.add_argument("--c4-jobs", type=int, default=64, help="c4: jobs in the stream")
    ap.add_argument("--iters", type=int, default=30, help="c2/c4: CEM iterations per job")
    ap.add_argument("--launch-check", action="store_true",
                    help="replica launch plumbing only: a fixed host workload per rank, no GPU, no rollouts")
    return ap.parse_args()


def relaunch_under_torchrun(n: int) -> int:
    """Start this script again as n ranks of one node (torch.distributed.run on 127.0.0.1)."""
    import socket
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={n}",
           "--master-addr=127.0.0.1", f"--master-port={port}", str(Path(__file__).resolve()), *sys.argv[1:]]
    return subprocess.run(cmd).returncode


def run_launch_check(args):
    """Each rank times the same fixed host workload (a seeded 256 x 256 FP64 matrix power); the
    line reports the whole-job rate over the slowest rank, as the GPU replica path does."""
    from spi_gb300 import replicas
    r = replicas.init("gloo")
    a = np.random.default_rng(r.rank).random((256, 256)) / 256.0
    for _ in range(args.warmup):
        a @ a
    r.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        b = a
        for _ in range(8):
            b = b @ a
    local_ms = (time.perf_counter() - t0) * 1e3
    value, ms = r.whole_job_rate(8.0 * args.steps, local_ms)
    if r.rank == 0:
        print(json.dumps({"metric": "matrix products/s (launch check, no rollouts)", "value": value,
                          "unit": "products/s", "n_gpus": r.world, "steps": args.steps, "warmup": args.warmup,
                          "ms_per_step": ms / max(args.steps, 1), "higher_is_better": True, "scaling": "weak",
                          "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                          "config": {"workload": "launch check: replica ranks over gloo, host workload only"},
                          "slowest_rank_ms": ms}), flush=True)
    r.close()


# --------------------------------------------------------------------------------------
# CPU baseline: the FP64 oracle on the host cores (spawned workers, no GPU in them)
# --------------------------------------------------------------------------------------
def _oracle_chunk(args):
    seed, n_theta, n_windows, horizon = args
    sys.path.insert(0, str(ROOT))
    from oracle import dynamics as dyn
    from oracle import go2_model as gm
    from oracle import sysid as osy
    rng = np.random.default_rng(seed)
    th = gm.THETA_PRIOR_LO + (gm.THETA_PRIOR_HI - gm.THETA_PRIOR_LO) * rng.random((n_theta, 13))
    x0 = np.tile(osy.standing_state(n_windows, z=0.30), (n_theta, 1))
    acts = rng.normal(size=(n_windows, horizon, 12))
    t0 = time.perf_counter()
    dyn.rollout(x0, np.tile(acts, (n_theta, 1, 1)), np.repeat(th, n_windows, 0), gm.SimParams())
    return n_theta * n_windows * horizon, time.perf_counter() - t0


def cpu_baseline(seconds: float, horizon: int):
    """Rollout-steps/s of the FP64 oracle over all host cores on a bounded C1 sample."""
    import multiprocessing as mp
    cores = os.cpu_count() or 1
    per_task = (8, 32, horizon)          # 8 theta x 32 windows x H per task (256 rollouts)
    ctx = mp.get_context("spawn")
    done_steps, tasks = 0, 0
    t0 = time.perf_counter()
    with ctx.Pool(cores) as pool:
        pool.map(_oracle_chunk, [(i, 1, 8, 2) for i in range(cores)])   # import warm-up
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < seconds:
            res = pool.map(_oracle_chunk, [(1000 + tasks + i, *per_task) for i in range(cores)])
            tasks += cores
            done_steps += sum(r[0] for r in res)
        wall = time.perf_counter() - t0
    return {"value": done_steps / wall, "unit": METRIC, "cores": cores, "kind": "port",
            "sample": f"{tasks} tasks x (8 theta x 32 windows x H={horizon}) of the c1 workload, "
                      f"{done_steps} rollout-steps in {wall:.1f} s (FP64 NumPy oracle, spawn pool)"}


# --------------------------------------------------------------------------------------
# GPU clocks during the timed region
# --------------------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() in ("active", "1"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# --------------------------------------------------------------------------------------
def _dist():
    from spi_gb300 import replicas
    r = replicas.init("nccl" if int(os.environ.get("WORLD_SIZE", "1")) > 1 else None)
    return r, r.rank, r.world, r.local


def served_vs_plain(specs, realtime, cfg=None, variant="lane3"):
    """Run the same jobs served (continuous batching) and plain (one job at a time), both on the
    rollout-kernel variant `variant`."""
    from spi_gb300.workloads import WindowBank, run_plain, run_served
    bank = WindowBank(cfg)
    served = run_served(specs, bank, cfg, realtime=realtime, variant=variant)
    plain = run_plain(specs, bank, cfg, variant=variant)
    ratios = []
    for s in specs:
        a, b = served["results"][s.job_id]["best_cost"], plain["results"][s.job_id]["best_cost"]
        ratios.append(a / max(b, 1e-30))
    ratios = np.array(ratios)
    out = {}
    for name, r in (("served", served), ("plain", plain)):
        out[name] = {k: v for k, v in r.items() if k not in ("results", "latencies")}
    out["speedup_rollout_steps"] = served["rollout_steps_per_s"] / plain["rollout_steps_per_s"]
    # Correctness at the 1e-4 relative cost bar: one CEM iteration per job, served and plain. Both
    # paths score the same seeded prior population, so their best costs are comparable directly.
    one = [dataclasses.replace(s, iterations=1, arrival=0.0, fisher=False) for s in specs]
    s1 = run_served(one, bank, cfg, realtime=False, variant=variant)["results"]
    p1 = run_plain(one, bank, cfg, variant=variant)["results"]
    errs = [abs(s1[s.job_id]["best_cost"] - p1[s.job_id]["best_cost"]) / max(abs(p1[s.job_id]["best_cost"]), 1e-30)
            for s in one]
    out["max_rel_cost_err_first_iteration"] = float(max(errs))
    # Served and plain launch the same compiled rollout kernel (the engine as a one-slot table),
    # so each job's search takes the same path in both: every ratio of final best costs is 1.0
    # unless the two diverged.
    out["best_cost_ratio_served_over_plain"] = {"median": float(np.median(ratios)), "min": float(ratios.min()),
                                                "max": float(ratios.max())}
    out["jobs"] = len(specs)
    out["kernel_variant"] = variant
    return out


def serving_mixes(args, variant, ceiling):
    """Served (continuous batching) against plain (one job at a time) on the job mixes the
    throughput / latency half of the metric is stated on, each with its served rate as a
    fraction of the single-job kernel ceiling (`ceiling`: the c1 rollout-steps/s of this run):
    * c2: 64 jobs, population U{256..4096}, windows U{16..512}, horizon U{5..50}, parameters
      U{1..13}, 30 CEM iterations each, all submitted at t = 0;
    * c4: the same size distribution as a Poisson stream at 200 jobs/s with 20 % of the jobs also
      asking for an excitation score, bounded to 64 arrivals (about 0.3 s of arrivals; the full
      60 s stream offers ~100x what one GPU serves and would run for hours);
    * small_jobs: 64 jobs of population U{64..512}, windows U{8..64}, horizon U{5..20}: each
      alone leaves most SMs idle, the regime where batching raises throughput."""
    from spi_gb300.server import Server
    from spi_gb300.workloads import c2_specs, poisson_arrivals, small_specs
    sv = variant if variant in Server.VARIANTS else "lane3"
    n, it = args.mix_jobs, args.mix_iters
    out = {}
    mixes = (
        ("c2", c2_specs(n, seed=2, iterations=it), False,
         f"c2: {n} jobs (pop U{{256..4096}}, W U{{16..512}}, H U{{5..50}}, P U{{1..13}}), {it} CEM iterations "
         "each, all submitted at t=0"),
        ("c4", poisson_arrivals(c2_specs(n, seed=4, iterations=it), args.c4_rate, seed=4, fisher_frac=0.2), True,
         f"c4: Poisson stream at {args.c4_rate:g} jobs/s of the c2 size distribution, {n} arrivals, {it} CEM "
         "iterations each, 20% also score 32 candidate excitations, 150 GB HBM admission budget"),
        ("small_jobs", small_specs(n, seed=3, iterations=it), False,
         f"{n} small jobs (pop U{{64..512}}, W U{{8..64}}, H U{{5..20}}, P U{{1..13}}), {it} CEM iterations each, "
         "all submitted at t=0"),
    )
    for name, specs, realtime, desc in mixes:
        r = served_vs_plain(specs, realtime, variant=sv)
        r["workload"] = desc
        r["served_fraction_of_kernel_ceiling"] = r["served"]["rollout_steps_per_s"] / ceiling
        r["plain_fraction_of_kernel_ceiling"] = r["plain"]["rollout_steps_per_s"] / ceiling
        out[name] = r
    out["kernel_ceiling_rollout_steps_per_s"] = ceiling
    out["note"] = ("the plain engine already puts every (theta, window) pair of a job in one launch, so a job of "
                   "the c2 sizes alone fills the GPU and the served rate is bounded by the same kernel ceiling: "
                   "served / plain cannot approach 5x there; it rises where jobs are small")
    return out


def run_multijob(args):
    import torch
    import __graft_entry__
    __graft_entry__.build()
    from spi_gb300.workloads import c2_specs, poisson_arrivals
    torch.cuda.set_device(0)
    if args.workload == "c2":
        specs = c2_specs(args.c2_jobs, seed=2, iterations=args.iters)
        desc = (f"c2: {args.c2_jobs} uneven jobs (pop U{{256..4096}}, W U{{16..512}}, H U{{5..50}}, "
                f"P U{{1..13}}), {args.iters} CEM iterations each, all submitted at t=0")
        realtime = False
    else:
        specs = poisson_arrivals(c2_specs(args.c4_jobs, seed=4, iterations=args.iters), args.c4_rate, seed=4,
                                 fisher_frac=0.2)
        desc = (f"c4: Poisson stream at {args.c4_rate:g} jobs/s, {args.c4_jobs} jobs from the c2 size "
                f"distribution, {args.iters} CEM iterations each, 20% also score 32 candidate excitations "
                f"(Fisher log det at the identified theta), 150 GB HBM admission budget")
        realtime = True
    with ClockSampler(0) as clocks:
        r = served_vs_plain(specs, realtime)
    served = r["served"]
    line = {"metric": METRIC, "value": served["rollout_steps_per_s"], "unit": METRIC, "n_gpus": 1,
            "steps": len(specs), "warmup": 0, "ms_per_step": served["wall_s"] * 1e3 / len(specs),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": desc, "step": "one identification job"},
            "served_vs_plain": r, "clocks": clocks.summary()}
    print(json.dumps(line), flush=True)


def run_c3(args):
    """C3: score candidate excitations by the Fisher information of forward-mode state
    sensitivities (13 theta directions x 37 states per window), BF16 J^T J on the tensor
    cores, FP64 log det. One step = scoring all candidates once."""
    import torch
    import __graft_entry__
    __graft_entry__.build()
    from spi_gb300.engine import Engine
    from spi_gb300.robot import THETA_NOMINAL
    from spi_gb300.sensitivity import block_weights, fisher, multisine_actions, score_excitations
    torch.cuda.set_device(0)
    eng = Engine()
    cfg = eng.cfg
    n, wpc, H, settle = args.c3_candidates, 8, 20, 100
    acts, _ = multisine_actions(n, wpc * H, cfg.control_dt, cfg.action_scale, seed=3, settle=settle)
    d_acts = torch.from_numpy(acts).cuda()            # the candidates stay resident on the device
    for _ in range(max(args.warmup, 1)):
        r = score_excitations(eng, THETA_NOMINAL, d_acts, windows_per_cand=wpc, horizon=H, settle=settle)
    torch.cuda.synchronize()
    times, parts = [], []
    with ClockSampler(0) as clocks:
        for _ in range(args.steps):
            t0 = time.perf_counter()
            tm = {}
            r = score_excitations(eng, THETA_NOMINAL, d_acts, windows_per_cand=wpc, horizon=H, settle=settle,
                                  timing=tm)
            torch.cuda.synchronize()
            times.append(time.perf_counter() - t0)
            parts.append(tm)
    breakdown = {k: float(np.mean([p[k] for p in parts])) for k in parts[0]}
    # the sensitivity kernel against the FP32 peak: FP operations of the dual-number rollout (the
    # kernel's formulation, one tangent, phase B once) per tangent rollout-step
    from spi_gb300.engine import probe_fp32_peak
    from spi_gb300.flops import dual_flops_per_rollout_step
    dual_fl = dual_flops_per_rollout_step(cfg)
    sens_roof = {"kernel": "sensitivity_kernel", "bound": "fp32",
                 "achieved": n * wpc * H * 13 * dual_fl / (breakdown["sensitivities_ms"] * 1e-3) / 1e12,
                 "peak": probe_fp32_peak() / 1e12, "unit": "TFLOP/s",
                 "flops_per_tangent_rollout_step": dual_fl,
                 "note": "achieved = tangent rollout-steps x FP operations of one dual-number control step "
                         "(csrc/dual.cuh arithmetic, counted on the host; phase B once) / the sensitivity "
                         "phase's device time; peak: the FP32 FMA-loop probe of this GPU"}
    sens_roof["frac"] = sens_roof["achieved"] / sens_roof["peak"]
    # the Fisher reduction alone, tensor cores against CUDA cores, on the last Jacobians
    J, q = r["J"], block_weights((10.0, 5.0, 0.1, 0.1, 1.0, 0.01))
    fisher_ms = {}
    for name, tc in (("tensor_cores_bf16", True), ("cuda_cores_fp32", False)):
        fisher(J, q, tensor_cores=tc)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(10):
            fisher(J, q, tensor_cores=tc)
        e1.record()
        e1.synchronize()
        fisher_ms[name] = e0.elapsed_time(e1) / 10
    t = float(np.mean(times))
    # Fisher roofline: J^T Q J over every candidate, 2 x rows x K x K flops per candidate, J read once
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    f_flops = 2.0 * n * wpc * 37 * 13 * 13
    f_bytes = n * wpc * 37 * 13 * 4
    f_s = fisher_ms["tensor_cores_bf16"] * 1e-3
    bf16_peak = peaks.get("bf16_tflops", 1900.0)
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    fisher_roof = {"kernel": "fisher_mma_kernel", "bound": "hbm", "achieved": f_bytes / f_s / 1e9, "peak": hbm_peak,
                   "unit": "GB/s", "frac": f_bytes / f_s / 1e9 / hbm_peak,
                   "tensor_tflops": f_flops / f_s / 1e12, "tensor_frac": f_flops / f_s / 1e12 / bf16_peak,
                   "note": "13 x 13 Gram matrices over 296 rows per candidate: too small for either roof "
                           "(one warp per candidate, latency-bound); peaks from MEASURED_PEAKS.json"}
    fd_line = fd_fisher_throughput(eng, acts, args)
    grad_line = gradient_throughput(eng, args)
    tangent_steps = n * wpc * H * 13
    primal_steps = n * (settle + wpc * H)
    line = {"metric": "excitation candidates scored/s", "value": n / t, "unit": "candidates/s", "n_gpus": 1,
            "steps": args.steps, "warmup": max(args.warmup, 1), "ms_per_step": t * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (J), bf16 x bf16 -> f32 (J^T J), f64 (log det)",
            "data": "synthetic",
            "config": {"workload": f"c3: {n} multi-sine candidates (12 joints x 3 components, amplitude U(0.05, 0.4) "
                                   f"rad, frequency U(0.5, 4) Hz), {settle}-step settle, {wpc} windows x H={H} "
                                   f"per candidate, 13 x 37 forward-mode sensitivities per window",
                       "step": "score every candidate once (settle trace, sensitivities, Fisher, log det)"},
            "rollout_steps_per_s": (tangent_steps + primal_steps) / t,
            "tangent_rollout_steps_per_step": tangent_steps, "primal_rollout_steps_per_step": primal_steps,
            "fisher_ms": fisher_ms, "fisher_roofline": fisher_roof, "best_candidate": int(r["best"]),
            "gradient": grad_line, "fd_fisher": fd_line, "breakdown_ms": breakdown,
            "sensitivity_roofline": sens_roof,
            "logdet_range": [float(np.min(r["logdet"])), float(np.max(r["logdet"]))],
            "clocks": clocks.summary()}
    print(json.dumps(line), flush=True)


def recorded_dram_bytes(kernel: str):
    """(dram__bytes_read.sum + dram__bytes_write.sum per launch, the ncu command) from the
    kernel's recorded capture on 1024 theta x 256 windows x H=20, or (None, None) without one."""
    rec = ROOT / "profiles" / f"{kernel}_1024x256xH20_dram.txt"
    if not rec.exists():
        return None, None
    vals, cmd = {}, None
    for ln in rec.read_text().splitlines():
        f = ln.split()
        if ln.startswith("command:"):
            cmd = ln[len("command:"):].strip()
        elif len(f) == 2 and f[0] in ("dram__bytes_read.sum", "dram__bytes_write.sum"):
            vals[f[0]] = int(f[1])
    if len(vals) != 2:
        return None, None
    return vals["dram__bytes_read.sum"] + vals["dram__bytes_write.sum"], cmd


def identification_report(cem, eng, theta_true):
    """Per-parameter result of the CEM identification, and which parameters the excitation
    cannot identify. The information check: F = mean_w J_w^T Q J_w at the true theta over the
    loaded windows (forward-mode sensitivities, Q the cost's state weights), so that the cost
    near the truth is about d^T F d for a parameter offset d. With the other parameters refit,
    moving parameter i by r raises the cost by r^2 / (F^-1)_ii; resolution_frac is the offset
    (in units of its prior range) at which that rise equals the best cost reached, i.e. the
    smallest error the windows can tell apart from the achieved fit."""
    import torch
    from spi_gb300.engine import DEFAULT_SQ_WEIGHTS
    from spi_gb300.robot import THETA_NAMES
    from spi_gb300.sensitivity import block_weights, sensitivities
    te = cem.theta_errors(theta_true)
    best = cem.best_cost()
    J, _ = sensitivities(eng, np.asarray(theta_true, np.float32)[None], cem.param_ids)
    q = torch.as_tensor(block_weights(DEFAULT_SQ_WEIGHTS), device=J.device, dtype=torch.float64)
    Jd = J[0].double()                                             # [W, 37, K]
    F = torch.einsum("wik,i,wil->kl", Jd, q, Jd).cpu().numpy() / J.shape[1]
    rng = cem.hi - cem.lo
    Fs = F * np.outer(rng, rng)                                    # in prior-range units
    Finv = np.linalg.pinv(Fs + 1e-12 * np.trace(Fs) * np.eye(len(rng)))
    resolution = np.sqrt(np.maximum(best, 0.0) * np.maximum(np.diag(Finv), 0.0))
    names = [THETA_NAMES[i] for i in cem.param_ids]
    per = {n: {"true": float(t), "est": float(e), "err_frac": float(ef), "std_frac": float(sf),
               "resolution_frac": float(r)}
           for n, t, e, ef, sf, r in zip(names, te["true"], te["est"], te["err_frac"], te["std_frac"], resolution)}
    worst = int(np.argmax(te["err_frac"]))
    return {"best_cost": best, "theta_err": float(te["err_frac"][worst]), "theta_err_param": names[worst],
            "per_param": per,
            "not_identified": [n for n, ef in zip(names, te["err_frac"]) if ef > 0.1],
            "unidentifiable": [n for n, r in zip(names, resolution) if r > 0.1],
            "note": "err_frac = |CEM mean - truth| / prior range; resolution_frac = sqrt(best_cost (F^-1)_ii) / "
                    "prior range from the exact Fisher information at the truth over the loaded windows: above "
                    "0.1 the windows carry too little information on that parameter (e.g. torque-limit scales "
                    "when no motor reaches its limit)"}


def run_rollout_case(args):
    """One rollout-kernel case for profilers: ground-truth windows generated on the GPU (one
    trace-kernel launch), prior theta samples, `--runs` launches of spi_run with the chosen
    variant, the last one timed with CUDA events. Under ncu, skip the first runs - 1 launches of
    the kernel with -s and capture one with -c 1."""
    import torch
    import __graft_entry__
    __graft_entry__.build()
    from spi_gb300 import robot
    from spi_gb300.autotune import set_variant
    from spi_gb300.data import synthetic_windows
    from spi_gb300.engine import Engine
    torch.cuda.set_device(0)
    rng = np.random.default_rng(5)
    lo, hi = robot.THETA_PRIOR_LO, robot.THETA_PRIOR_HI
    e = Engine()
    init, act, tgt = synthetic_windows(e, lo + (hi - lo) * rng.random(13), args.n_windows, args.horizon, seed=77)
    e.load_windows(torch.from_numpy(init), torch.from_numpy(act), torch.from_numpy(tgt))
    e.set_theta(torch.from_numpy((lo + (hi - lo) * rng.random((args.n_theta, 13))).astype(np.float32)))
    set_variant(e, args.variant)
    for _ in range(args.runs - 1):
        e.run()
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0.record(e.stream)
    e.run()
    t1.record(e.stream)
    t1.synchronize()
    _, cost = e.read()
    torch.cuda.synchronize()
    n_bad = e.sync()
    if n_bad:
        raise SystemExit(f"{n_bad} non-finite rollouts")
    ms = t0.elapsed_time(t1)
    steps = args.n_theta * args.n_windows * args.horizon
    print(json.dumps({"metric": METRIC, "value": steps / (ms * 1e-3), "unit": METRIC, "n_gpus": 1, "steps": 1,
                      "warmup": args.runs - 1, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
                      "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                      "config": {"workload": f"rollout-case: {args.n_theta} theta x {args.n_windows} windows x "
                                             f"H={args.horizon}, one spi_run launch timed",
                                 "kernel_variant": args.variant},
                      "median_cost": float(cost.median())}), flush=True)


def fd_fisher_throughput(eng, acts, args, param_ids=tuple(range(13)), delta=0.1, ksync=5):
    """The reference's own excitation objective on the same candidates: the FD-Fisher episode
    (1 main + 13 aux rollouts per candidate, aux at theta + 0.1 on one parameter, resync every 5
    steps, trace(J^T J) of the finite differences after every step) over each candidate's whole
    excitation, one fused launch (spi_fd_fisher)."""
    import torch
    from spi_gb300.active import fd_fisher
    from spi_gb300.data import standing_state
    from spi_gb300.robot import THETA_NOMINAL
    n, T = acts.shape[:2]
    x0 = torch.from_numpy(np.repeat(standing_state(1, z=0.32), n, 0)).cuda()
    a = torch.from_numpy(acts).cuda()
    th = THETA_NOMINAL.astype(np.float32)
    obj = fd_fisher(eng, x0, a, th, param_ids, delta=delta, ksync=ksync)
    torch.cuda.synchronize()
    reps = max(1, min(args.steps, 5))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(eng.stream)
    for _ in range(reps):
        obj = fd_fisher(eng, x0, a, th, param_ids, delta=delta, ksync=ksync)
    e1.record(eng.stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / reps
    o = obj.cpu().numpy()
    rollout_steps = n * (len(param_ids) + 1) * (T + 1)
    return {"workload": f"{n} candidates x (1 main + {len(param_ids)} aux) rollouts x {T + 1} control steps "
                        f"(one zero-action reset step), delta {delta}, resync every {ksync} steps",
            "ms": ms, "candidates_per_s": n / (ms * 1e-3), "rollout_steps_per_s": rollout_steps / (ms * 1e-3),
            "objective_range": [float(np.min(o)), float(np.max(o))], "best_candidate": int(np.argmax(o))}


def gradient_throughput(eng, args, n_theta=512, n_windows=256, horizon=20):
    """d cost / d theta of the squared-error window cost for n_theta prior samples against
    n_windows windows x H = 20 (13 parameters): one hand-written adjoint sweep per rollout
    (spi_adjoint, checkpoints every 5 control steps) against 13 forward-mode tangent sweeps
    (spi_sensitivity). CUDA-event times on the engine stream after a warm-up call of each."""
    import torch
    from spi_gb300 import robot
    from spi_gb300.data import synthetic_windows
    from spi_gb300.engine import COST_SQ
    from spi_gb300.sensitivity import adjoint, tangent_gradient
    rng = np.random.default_rng(12)
    lo, hi = robot.THETA_PRIOR_LO, robot.THETA_PRIOR_HI
    init, act, tgt = synthetic_windows(eng, lo + (hi - lo) * rng.random(13), n_windows, horizon, seed=21)
    eng.load_windows(torch.from_numpy(init), torch.from_numpy(act), torch.from_numpy(tgt))
    eng.set_cost(COST_SQ)
    th = torch.from_numpy((lo + (hi - lo) * rng.random((n_theta, 13))).astype(np.float32)).cuda()
    out = {}
    for name, fn in (("adjoint", lambda: adjoint(eng, th)), ("tangent_13", lambda: tangent_gradient(eng, th))):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        reps = max(1, min(args.steps, 5))
        e0.record(eng.stream)
        for _ in range(reps):
            res = fn()
        e1.record(eng.stream)
        e1.synchronize()
        out[name] = (e0.elapsed_time(e1) / reps, res)
    (ta, (ca, ga)), (tt, (ct, gt)) = out["adjoint"], out["tangent_13"]
    ga, gt = ga.double(), gt.double()
    rel = float(((ga - gt).norm(dim=1) / gt.norm(dim=1).clamp(min=1e-30)).max())
    rollouts = n_theta * n_windows
    return {"workload": f"{n_theta} theta x {n_windows} windows x H={horizon}, 13 parameters, squared-error cost",
            "adjoint_ms": ta, "tangent_13_ms": tt, "speedup_adjoint_over_tangent": tt / ta,
            "adjoint_rollout_gradients_per_s": rollouts / (ta * 1e-3),
            "tangent_rollout_gradients_per_s": rollouts / (tt * 1e-3),
            "max_rel_diff_adjoint_vs_tangent": rel, "nonfinite_rollouts": eng.sync()}


def run_reference(args):
    """The reference arm: the FP64 oracle (the reference path's CPU restatement) on all host
    cores, W warm-up steps then K timed steps. One step is a bounded sample of the C1 workload:
    one task per core of 8 theta x 32 windows x H = 20 rollouts."""
    import multiprocessing as mp
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    H = C1["horizon"]
    per_task = (8, 32, H)
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        pool.map(_oracle_chunk, [(i, 1, 8, 2) for i in range(cores)])   # import warm-up
        task = 0
        for _ in range(args.warmup):
            pool.map(_oracle_chunk, [(1000 + task + i, *per_task) for i in range(cores)])
            task += cores
        step_s, done = [], 0
        for _ in range(args.steps):
            t0 = time.perf_counter()
            res = pool.map(_oracle_chunk, [(1000 + task + i, *per_task) for i in range(cores)])
            step_s.append(time.perf_counter() - t0)
            task += cores
            done += sum(r[0] for r in res)
    total = float(np.sum(step_s))
    value = done / total
    sample = (f"{args.steps} steps x {cores} tasks x (8 theta x 32 windows x H={H}) of the c1 workload, "
              f"{done} rollout-steps in {total:.1f} s (FP64 NumPy oracle, spawn pool, after {args.warmup} "
              f"warm-up steps)")
    line = {"metric": METRIC, "value": value, "unit": METRIC, "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": total * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "c1: 4096 theta x 256 windows x H=20, 13 params, Go2 FP64 NumPy oracle on "
                                   "host cores", "step": f"{cores * 8 * 32 * H} rollout-steps (bounded sample)"},
            "cpu_baseline": {"value": value, "unit": METRIC, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    import __graft_entry__
    if int(os.environ.get("RANK", "0")) == 0:
        __graft_entry__.build()
    ranks, rank, ws, local = _dist()
    ranks.barrier()
    from spi_gb300 import robot
    from spi_gb300.cem import CEM
    from spi_gb300.data import synthetic_windows
    from spi_gb300.engine import Engine, probe_fp32_peak
    from spi_gb300.flops import executed_flops_per_rollout_step, flops_per_rollout_step

    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    cfg = robot.SimConfig()
    N, W, H = C1["n_theta"], C1["n_windows"], C1["horizon"]
    rng = np.random.default_rng(1234 + rank)
    lo, hi = robot.THETA_PRIOR_LO, robot.THETA_PRIOR_HI
    theta_true = lo + (hi - lo) * rng.random(13)
    eng = Engine(cfg, device=dev)
    init, actions, target = synthetic_windows(eng, theta_true, W, H, seed=77 + rank)
    eng.load_windows(torch.from_numpy(init), torch.from_numpy(actions), torch.from_numpy(target))
    cem = CEM(eng, n_samples=N, param_ids=list(range(13)), lo=lo, hi=hi, nominal=robot.THETA_NOMINAL,
              elite_frac=C1["elite_frac"], seed=4321 + rank)
    flush = torch.empty(256 * 1024 * 1024 // 4, device=dev)
    stream = torch.cuda.current_stream(dev)
    # pick the rollout-kernel occupancy variant on this workload (outside the timed region)
    from spi_gb300.autotune import set_variant, tune_engine
    cem.sample()
    if args.c1_variant == "auto":
        variant, variant_ms = tune_engine(eng, use_cache=False)
    else:
        set_variant(eng, args.c1_variant)
        variant, variant_ms = args.c1_variant, None
    cem.sample()             # the tuning runs do not advance the CEM state

    for _ in range(args.warmup):
        cem.step()
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    run_s = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    run_e = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ranks.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        wall0 = time.perf_counter()
        for k in range(args.steps):
            flush.zero_()                                  # L2 flush between timed steps
            starts[k].record(stream)
            cem.step(rollout_events=(run_s[k], run_e[k]))
            ends[k].record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    kern_ms = [s.elapsed_time(e) for s, e in zip(run_s, run_e)]
    n_bad = eng.sync()
    steps_per_iter = N * W * H
    value, total_ms = ranks.whole_job_rate(steps_per_iter * args.steps, float(np.sum(step_ms)), dev)

    # end to end: host buffers through the public API, copies inside the timed region
    e2e = None
    if not args.no_e2e:
        pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory()   # noqa: E731
        h_init, h_act, h_tgt = pin(init), pin(actions), pin(target)
        h_theta = pin(cem.sample_host(args.steps))
        h_cost = torch.empty((N,), dtype=torch.float32).pin_memory()
        d_init = torch.empty_like(h_init, device=dev)
        d_act = torch.empty_like(h_act, device=dev)
        d_tgt = torch.empty_like(h_tgt, device=dev)
        d_theta = torch.empty((N, 13), device=dev)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for k in range(args.steps):
            d_init.copy_(h_init, non_blocking=True)
            d_act.copy_(h_act, non_blocking=True)
            d_tgt.copy_(h_tgt, non_blocking=True)
            d_theta.copy_(h_theta[k], non_blocking=True)
            eng.load_windows(d_init, d_act, d_tgt)
            eng.set_theta(d_theta)
            eng.run()
            _, cost = eng.read()
            h_cost.copy_(cost, non_blocking=True)
        e1.record(stream)
        torch.cuda.synchronize()
        ranks.barrier()
        e2e_value, e2e_ms = ranks.whole_job_rate(steps_per_iter * args.steps, e0.elapsed_time(e1), dev)
        h2d = (init.nbytes + actions.nbytes + target.nbytes + N * 13 * 4)
        e2e = {"value": e2e_value, "unit": METRIC,
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(N * 4),
               "note": "per step: windows + theta H2D from pinned memory, spi_load_windows, "
                       "spi_set_theta, spi_run, spi_read_costs, cost D2H (evaluation only)"}

    fl = flops_per_rollout_step(cfg)
    kmean = float(np.mean(kern_ms))
    peak = probe_fp32_peak()
    achieved = steps_per_iter * fl / (kmean * 1e-3)
    kname = {"lane": "rollout_lane_kernel", "bloc": "rollout_block_kernel"}.get(variant[:4], "rollout_quad_kernel")
    traffic, traffic_cmd = recorded_dram_bytes(kname)
    roof = {"bound": "fp32", "achieved": achieved / 1e12, "peak": peak / 1e12, "unit": "TFLOP/s",
            "frac": achieved / peak, "traffic": traffic,
            "traffic_note": "dram read+write bytes per launch, recorded from one ncu capture of the kernel on "
                            "1024 theta x the same 256 windows x H=20 (" + (traffic_cmd or "no record") + "); the "
                            "window set is read once and theta / partials stay in L2, so traffic does not scale "
                            "with theta",
            "kernel": kname + " (+fill_single_kernel, finalize_costs)",
            "kernel_ms": kmean,
            "flops_per_rollout_step": fl,
            "flops_note": "algorithmic count: the oracle's equations (legs by the articulated-body algorithm), "
                          "instrumented on the host; the kernel condenses each leg through its joint-space "
                          "inertia and executes executed_flops_per_rollout_step for the same result",
            "executed_flops_per_rollout_step": executed_flops_per_rollout_step(cfg),
            "peak_source": "measured FP32 FMA-loop probe on this GPU (no FP32 entry in MEASURED_PEAKS.json)"}
    if rank != 0:
        ranks.close()
        return
    line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "c1", "n_theta": N, "n_windows": W, "horizon": H, "substeps": cfg.decimation,
                       "n_params": 13, "elite_frac": C1["elite_frac"],
                       "step": "one CEM iteration (rollouts + cost + refit + resample)",
                       "l2": "flushed between steps (256 MiB write)", "parallelism": f"replicas x{ws}",
                       "kernel_variant": {"chosen": variant, "tuning_ms": variant_ms}},
            "roofline": roof, "e2e": e2e, "gpu_launches": cem.launches_per_step * args.steps,
            "wall_s": wall, "nonfinite_rollouts": n_bad, "clocks": clocks.summary(),
            "cem": identification_report(cem, eng, theta_true)}
    if ws == 1 and not args.no_serving:
        line["served_vs_plain"] = serving_mixes(args, variant, value)
    if ws == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args.cpu_seconds, H)
    print(json.dumps(line), flush=True)
    ranks.close()


def main():
    args = parse_args()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(relaunch_under_torchrun(args.gpus))
    if args.launch_check:
        run_launch_check(args)
    elif args.impl == "reference":
        run_reference(args)
    elif args.workload == "c3":
        run_c3(args)
    elif args.workload == "rollout-case":
        run_rollout_case(args)
    elif args.workload in ("c2", "c4"):
        run_multijob(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
