"""Launch-setting autotuner for one workload.

Times whole steps of the real workload (a forward frame, or forward +
backward) on the engine's own stream for candidate settings and keeps the
fastest, one axis at a time (each axis tried with the best values found so
far for the others). The tunables are engine settings that leave every
result bit for bit unchanged:

  key_sort_lookback  the key sort's radix passes: counted (0: every
                     partition's digits counted and scanned first, then a
                     scatter that waits for no other partition) or onesweep
                     with a decoupled look-back (1)
  sort_threads       CTA size of the onesweep key sort's 4096-key passes: 512
                     threads x 8 keys (digits ranked with match-any, twice the
                     warps per SM) or 256 threads x 16 keys (bit ballots);
                     tried only with key_sort_lookback = 1 (the counted
                     passes always run 256 x 16 keys)
  depth_sort_threads the same choice for the depth sort's passes
  depth_sort_items   keys per thread of the depth sort's 256-thread passes
                     (16, 8, 4: partitions of 4096, 2048, 1024 keys); smaller
                     partitions fill the GPU when the Gaussians are few
  sort_ctas_per_sm   residency the 256 x 16-key pass kernels are compiled
                     for: 0 the defaults (counted scatter 3 CTAs per SM at 80
                     registers, onesweep 2 at 128), 2 both at 2

For a training step (forward + backward, TRAIN_AXES) the blend's settings:

  blend_round           list entries the blend stages per round (its batch
                        depth): 128, 64 or 256
  blend_backward_round  the same for the blend adjoint: 64, 32 or 128
  blend_persistent      one CTA per tile (0), or persistent CTAs taking
                        (view, tile) items from a queue over all views (1)

Forward images are bit for bit the same under every setting; the adjoint's
gradients are sums of float atomics, whose order no setting fixes.

The tile size stays 16x16 and the radix digit 8 bits: the tile size fixes
the reference's key layout (tile id | depth), and a 13-bit tile id takes two
passes at any digit width from 7 to 12 bits.
"""
from __future__ import annotations

from typing import Callable

AXES = (("key_sort_lookback", (0, 1)), ("sort_threads", (256, 512)), ("depth_sort_threads", (256, 512)),
        ("depth_sort_items", (16, 8)), ("sort_ctas_per_sm", (0, 2)))
TRAIN_AXES = (("blend_backward_round", (64, 32, 128)), ("blend_round", (128, 64, 256)), ("blend_persistent", (0, 1)))
# axes that change nothing under the given settings: not tried there
INERT = {"sort_threads": lambda s: s.get("key_sort_lookback", 0) == 0}


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
         frames: int = 20, warmup: int = 3, axes=AXES, base: dict | None = None) -> tuple[dict, dict]:
    """make_engine(settings) -> a ready engine (compiled, views set, one frame
    rendered); enqueue(engine, count) enqueues count steps on `stream` (a
    torch.cuda.Stream). base: settings kept as they are. Returns (best
    settings, {label: ms per step})."""
    best = dict(base or {}, **{name: values[0] for name, values in axes})
    results: dict[str, float] = {}
    best_ms = None
    for name, values in axes:
        if name in INERT and INERT[name](best):
            continue
        for v in values:
            cand = dict(best, **{name: v})
            label = ",".join(f"{k}={x}" for k, x in cand.items() if k in dict(axes))
            if label not in results:
                results[label] = round(time_steps(make_engine, enqueue, stream, cand, frames, warmup), 4)
            if best_ms is None or results[label] < best_ms:
                best, best_ms = cand, results[label]
    return best, results
