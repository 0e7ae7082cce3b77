"""Kernel-variant autotuner for the rollout kernel.

The rollout kernel comes in occupancy variants: the register allocator targets 3, 4 or 5
CTAs of 128 threads per SM (168 / 128 / 96 registers per thread, with more spilling as
registers shrink). Which is fastest depends on the horizon, window tiling and GPU, so the
variant is picked by timing each on the caller's own windows and theta batch. Choices are
cached per (GPU, horizon bucket, work bucket) in the build folder.
"""
from __future__ import annotations

import json
import math
from pathlib import Path

import torch

from . import _lib
from ._build import LIB_DIR

CACHE = LIB_DIR / "autotune.json"
VARIANTS = (3, 4, 5)


def _key(engine):
    name = torch.cuda.get_device_name(engine.device).replace(" ", "_")
    work = engine.N * ((engine.W + 7) // 8)
    return f"{name}|H{2 ** max(0, math.ceil(math.log2(max(engine.H, 1))))}|G{2 ** max(0, math.ceil(math.log2(max(work, 1))))}"


def _load():
    try:
        return json.loads(Path(CACHE).read_text())
    except (OSError, ValueError):
        return {}


def set_variant(engine, min_blocks):
    _lib.check(engine.lib.spi_set_kernel_config(engine._h, int(min_blocks)))
    engine.min_blocks = int(min_blocks)


def tune_engine(engine, reps=3, use_cache=True):
    """Time every variant on the engine's loaded windows and theta batch; keep the fastest.

    Returns (chosen variant, {variant: ms per launch}).
    """
    cache = _load() if use_cache else {}
    key = _key(engine)
    if use_cache and key in cache:
        set_variant(engine, cache[key]["best"])
        return cache[key]["best"], cache[key]["ms"]
    times = {}
    s = engine.stream
    for mb in VARIANTS:
        set_variant(engine, mb)
        engine.run()
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record(s)
        for _ in range(reps):
            engine.run()
        t1.record(s)
        t1.synchronize()
        times[mb] = t0.elapsed_time(t1) / reps
    best = min(times, key=times.get)
    set_variant(engine, best)
    cache[key] = {"best": best, "ms": times}
    try:
        LIB_DIR.mkdir(exist_ok=True)
        Path(CACHE).write_text(json.dumps(cache, indent=1))
    except OSError:
        pass
    return best, times
