"""Launch-setting autotuner for one workload.

Times whole steps of the real workload (a forward frame, or forward +
backward) for each candidate setting on the engine's own stream and keeps the
fastest. The tunables are engine settings that leave every result bit for bit
unchanged:

  sort_ctas_per_sm   residency the radix pass kernel is compiled for (2: 128
                     registers, no spills; 3: 80 registers)

The tile size stays 16x16 and the radix digit 8 bits: the tile size fixes
the reference's key layout (tile id | depth), and a 16-bit tile id takes two
passes at any digit width from 8 to 15 bits.
"""
from __future__ import annotations

from typing import Callable

CANDIDATES = ({"sort_ctas_per_sm": 2}, {"sort_ctas_per_sm": 3})


def tune(make_engine: Callable[[dict], object], enqueue: Callable[[object, int], None], stream,
         frames: int = 20, warmup: int = 3, candidates=CANDIDATES) -> tuple[dict, dict]:
    """make_engine(settings) -> a ready engine (compiled, views set, one frame
    rendered); enqueue(engine, count) enqueues count steps on `stream` (a
    torch.cuda.Stream). Returns (best settings, {label: ms per step})."""
    import torch

    results = {}
    best, best_ms = None, float("inf")
    for cand in candidates:
        eng = make_engine(dict(cand))
        try:
            enqueue(eng, warmup)
            eng.sync()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            enqueue(eng, frames)
            b.record(stream)
            eng.sync()
            ms = a.elapsed_time(b) / frames
        finally:
            eng.close()
        label = ",".join(f"{k}={v}" for k, v in cand.items())
        results[label] = round(ms, 4)
        if ms < best_ms:
            best, best_ms = dict(cand), ms
    return best, results
