"""Launch-setting autotuner for one workload.

Times whole steps of the real workload (a forward frame, or forward +
backward) on the engine's own stream for candidate settings and keeps the
fastest, one axis at a time (each axis tried with the best values found so
far for the others). The tunables are engine settings that leave every
result bit for bit unchanged:

  sort_threads       CTA size of the 4096-key radix passes: 256 threads x 16
                     keys, or 512 threads x 8 keys (twice the warps per SM)
  sort_ctas_per_sm   residency the 256-thread radix pass kernel is compiled
                     for (2: 128 registers, no spills; 3: 80 registers)
  depth_sort_items   keys per thread of the depth sort's radix passes (4, 8,
                     16: partitions of 1024, 2048, 4096 keys); smaller
                     partitions fill the GPU when the Gaussians are few

The tile size stays 16x16 and the radix digit 8 bits: the tile size fixes
the reference's key layout (tile id | depth), and a 13-bit tile id takes two
passes at any digit width from 7 to 12 bits.
"""
from __future__ import annotations

from typing import Callable

AXES = (("sort_threads", (256, 512)), ("sort_ctas_per_sm", (2, 3)), ("depth_sort_items", (16, 8)))


def time_steps(make_engine: Callable[[dict], object], enqueue: Callable[[object, int], None], stream,
               settings: dict, frames: int, warmup: int) -> float:
    """Milliseconds per step of `settings` (CUDA events on `stream`)."""
    import torch

    eng = make_engine(dict(settings))
    try:
        enqueue(eng, warmup)
        eng.sync()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        enqueue(eng, frames)
        b.record(stream)
        eng.sync()
        return a.elapsed_time(b) / frames
    finally:
        eng.close()


def tune(make_engine: Callable[[dict], object], enqueue: Callable[[object, int], None], stream,
         frames: int = 20, warmup: int = 3, axes=AXES) -> tuple[dict, dict]:
    """make_engine(settings) -> a ready engine (compiled, views set, one frame
    rendered); enqueue(engine, count) enqueues count steps on `stream` (a
    torch.cuda.Stream). Returns (best settings, {label: ms per step})."""
    best = {name: values[0] for name, values in axes}
    results: dict[str, float] = {}
    best_ms = None
    for name, values in axes:
        for v in values:
            cand = dict(best, **{name: v})
            label = ",".join(f"{k}={x}" for k, x in cand.items())
            if label not in results:
                results[label] = round(time_steps(make_engine, enqueue, stream, cand, frames, warmup), 4)
            if best_ms is None or results[label] < best_ms:
                best, best_ms = cand, results[label]
    return best, results
