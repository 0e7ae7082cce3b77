"""One rollout-kernel case for profilers and quick timings.

    PYTHONPATH=spi-active_gb300 python -m spi_gb300.profile_case [--variant quad3] [--n-theta 1024]
        [--n-windows 256] [--horizon 20] [--runs 2]

Builds the library, generates the ground-truth windows on the GPU (one launch of the trace
kernel, `rollout_kernel<true, 3>`), selects the rollout-kernel variant, and launches
`spi_run` `--runs` times on the same prior samples; the last launch is timed with CUDA
events and printed. Under ncu, skip the first `--runs - 1` launches of the chosen kernel
(and, for quad variants, the trace launch too) with `-s` and capture one with `-c 1`.
"""
from __future__ import annotations

import argparse

import numpy as np
import torch


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--variant", default="quad3")
    ap.add_argument("--n-theta", type=int, default=1024)
    ap.add_argument("--n-windows", type=int, default=256)
    ap.add_argument("--horizon", type=int, default=20)
    ap.add_argument("--runs", type=int, default=2)
    args = ap.parse_args(argv)

    from . import _build
    _build.build()
    from . import robot
    from .autotune import set_variant
    from .data import synthetic_windows
    from .engine import Engine

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
    assert e.sync() == 0, "non-finite rollouts"
    print(f"{args.variant} N={args.n_theta} W={args.n_windows} H={args.horizon}: {t0.elapsed_time(t1):.3f} ms, "
          f"median cost {float(cost.median()):.4g}")


if __name__ == "__main__":
    main()
