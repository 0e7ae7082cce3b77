"""Kernel-variant autotuner for the rollout kernel.

The rollout kernel comes in three lane layouts -- "quad" (four lanes per rollout, one leg
each), "block" (the quad layout with each rollout's base solved once by one warp of the CTA)
and "lane" (one lane per rollout through all four legs) -- and occupancy variants: the
register allocator targets 2..5 CTAs of 128 threads per SM (255 / 168 / 128 / 96 registers
per thread, with more spilling as registers shrink). Which is fastest depends on the
horizon, the window count and the GPU, so the variant is picked by timing each on the caller's
own windows and theta batch. Choices are cached per (GPU, horizon bucket, work bucket,
window-count remainder) in the build folder.
"""
from __future__ import annotations

import json
import math
from pathlib import Path

import torch

from . import _lib
from ._build import LIB_DIR

CACHE = LIB_DIR / "autotune.json"
# (name, layout, min_blocks); layout 0 = SPI_LAYOUT_QUAD, 1 = SPI_LAYOUT_LANE, 2 = SPI_LAYOUT_BLOCK
VARIANTS = (("quad3", 0, 3), ("quad4", 0, 4), ("quad5", 0, 5), ("lane2", 1, 2), ("lane3", 1, 3), ("lane4", 1, 4),
            ("block3", 2, 3), ("block4", 2, 4), ("block5", 2, 5))
_BY_NAME = {v[0]: v for v in VARIANTS}


def _key(engine):
    name = torch.cuda.get_device_name(engine.device).replace(" ", "_")
    work = engine.N * ((engine.W + 7) // 8)
    return (f"{name}|H{2 ** max(0, math.ceil(math.log2(max(engine.H, 1))))}"
            f"|G{2 ** max(0, math.ceil(math.log2(max(work, 1))))}|W%32={engine.W % 32}")


def _load():
    try:
        return json.loads(Path(CACHE).read_text())
    except (OSError, ValueError):
        return {}


def set_variant(engine, name):
    """Select a rollout-kernel variant by name (one of VARIANTS)."""
    _, layout, min_blocks = _BY_NAME[name]
    _lib.check(engine.lib.spi_set_kernel_layout(engine._h, int(layout)))
    _lib.check(engine.lib.spi_set_kernel_config(engine._h, int(min_blocks)))
    engine.variant = name


def tune_engine(engine, reps=3, use_cache=True):
    """Time every variant on the engine's loaded windows and theta batch; keep the fastest.

    Returns (chosen variant, {variant: ms per launch}).
    """
    cache = _load() if use_cache else {}
    key = _key(engine)
    if use_cache and key in cache and cache[key]["best"] in _BY_NAME:
        set_variant(engine, cache[key]["best"])
        return cache[key]["best"], cache[key]["ms"]
    times = {}
    s = engine.stream
    for mb, _, _ in VARIANTS:
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
