"""Benchmark of the Gaussian-splatting hot path: forward frames per second on the
bench workload (cfg1: 1,000,000 Gaussians, 1920x1080, SH degree 3, 16x16 tiles).

A step is one forward frame: preprocess -> tile-count scan -> key duplication ->
radix sort -> tile ranges -> blend, with the Gaussians resident in device memory.

  value  frames/s over --steps frames enqueued back to back (CUDA graph replay),
         CUDA events on the engine's stream, max over ranks; the timed region
         of --steps frames runs 5 times and value is the median region
         (timed_regions_ms lists all five)
  e2e    frames/s through the C ABI with host buffers: per step the camera is
         uploaded from pinned host memory, the frame rendered and the RGBA8 image
         read back into pinned host memory (tpd_render_async / tpd_wait_render,
         two frames in flight)
  roofline  one radix pass of the key sort (its counting and scatter kernels,
         or its onesweep kernel): algorithmic bytes K*24 per pass over the
         pass's average duration, from CUDA events recorded between stages
         during a second timed region
  general_sort  the standalone radix sort on the frame's keys in random order,
         all key bits, sort GB/s by the fixed formula K*(8 + 24*ceil(B/8))
  cpu_baseline  the oracle's FP32 transcription of the reference shaders (same
         4-way radix sort and pass count) on the host cores
  fwd_bwd  training steps/s on cfg2 (200,000 Gaussians, 800x800): forward +
         backward as one captured graph per step (tpd_step_async)
  batched  views/s on cfg3 (500,000 Gaussians, 64 views of mixed sizes):
         forward + backward of all 64 views as one graph per step, against
         the plain pipeline rendering and differentiating one view per call;
         stages_ms splits the step by stage
  large  views/s on cfg4 (6,000,000 Gaussians, 8 views of 3840x2160),
         forward + backward per step, with the key count and the device
         memory the engine holds
  autotune  the launch setting picked for the workload (torpedo_gb300.autotune)
         and the per-frame time of each candidate; train_ms_per_step the
         training-step candidates (blend batch depths, persistent tile
         scheduler) tuned on cfg2 and on cfg3, whose picks those runs use

--impl reference times that CPU transcription alone (rank 0; other ranks exit).
Launched with torchrun for N > 1: every rank renders the workload independently
(replicas; weak scaling).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "fwd FPS at 1M Gaussians 1080p (cfg1); sort GB/s vs HBM in roofline"
UNIT = "frames/s"
REGIONS = 5  # timed regions of --steps frames each; value is their median
FRAME_STAGES = ("preprocess", "depth_sort", "keygen", "key_sort", "ranges", "blend")


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Clocks:
    """Samples nvidia-smi clocks / throttle reasons while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-i", str(self.gpu), "-lms", "100"], stdout=open(self.path, "w"),
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict | None:
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in Path(self.path).read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), float(parts[3]), parts[5:9]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return None
        # samples under load: power well above idle
        pmax = max(r[2] for r in rows)
        load = [r for r in rows if r[2] >= 0.5 * pmax] or rows
        sm = sorted(r[0] for r in load)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in load for i, v in enumerate(r[3]) if v.lower() == "active"})
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": max(r[1] for r in rows), "reasons": reasons,
                "samples": len(rows), "samples_under_load": len(load)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def cpu_frames(records, oc, budget_s: float, threads: int, max_frames: int):
    """Times the oracle's FP32 transcription on whole frames (camera constants
    oc, an oracle camera) until the budget is spent."""
    from oracle import oracle as O

    times = []
    k = 0
    t_all = time.perf_counter()
    while len(times) < max_frames:
        t0 = time.perf_counter()
        _, k = O.frame_f32(records, oc, threads=threads)
        times.append(time.perf_counter() - t0)
        if time.perf_counter() - t_all > budget_s:
            break
    return times, k


def oracle_workload(cfg_name: str):
    """Records and camera constants of a one-view workload built by the oracle
    alone (its own seeded generator and camera maths, equal bit for bit to the
    product's): the reference arm loads nothing of the product library."""
    from oracle import oracle as O
    from torpedo_gb300.configs import CONFIGS, FAR, FOV, NEAR, UP

    cfg = CONFIGS[cfg_name]
    if cfg.views != 1:
        raise SystemExit(f"--impl reference times one-view workloads; {cfg_name} has {cfg.views} views")
    w, h = cfg.sizes[0]
    recs = O.synthetic_records(int(cfg.name[3:]), cfg.n, cfg.mean_box)
    return cfg, recs, O.orbit_camera((0.0, 0.0, -5.0), w, h, FOV, NEAR, FAR, UP)


def run_reference(args):
    world, rank, local = dist_setup()
    if rank != 0:
        return
    cfg, recs, oc = oracle_workload(args.config)
    threads = os.cpu_count() or 1
    # warm-up frames, then timed frames; the run is capped at ~3 minutes of CPU time
    per_frame = cpu_frames(recs, oc, 0.0, threads, 1)[0][0]
    warm = max(0, min(args.warmup, int(20 / max(per_frame, 1e-3))))
    if warm:
        cpu_frames(recs, oc, 1e9, threads, warm)
    steps = max(3, min(args.steps, int(150 / max(per_frame, 1e-3))))
    times, k = cpu_frames(recs, oc, 1e9, threads, steps)
    total = sum(times)
    value = len(times) / total
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world,
        "steps": len(times), "warmup": warm, "ms_per_step": round(1000 * total / len(times), 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(cfg, oc.width, oc.height, k),
        "cpu_baseline": {"value": round(value, 4), "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{len(times)} whole {cfg.name} frames of the FP32 transcription of the "
                                   f"reference shaders (4-way radix sort, {ref_passes(oc.width, oc.height)} passes "
                                   f"over K={k} keys), OpenMP over workgroups"},
        "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference's Vulkan/Slang path cannot run here (no Vulkan, no slangc, no software renderer); "
                "this arm times the oracle's line-by-line FP32 transcription of its shaders",
    }
    print(json.dumps(line), flush=True)


def ref_passes(width: int, height: int) -> int:
    from oracle import oracle as O

    return O.radix_pass_count(width, height)


def workload_config(cfg, width, height, keys):
    return {"workload": f"{cfg.name}: {cfg.n:,} Gaussians, {width}x{height}, SH degree 3, 16x16 tiles, "
                        f"means U[-{cfg.mean_box:g},{cfg.mean_box:g}]^3, camera (0,0,-5) fov 60",
            "n_gaussians": cfg.n, "image": [width, height], "keys": int(keys), "views": 1,
            "l2": "inputs larger than L2: 240 MB of records and >= 100 MB of keys per frame",
            "parallelism": "replicas"}


def general_sort(eng, K, key_bits, stream, steps):
    """The standalone radix sort (tpd_sort_pairs) on the frame's K keys in random
    order, all key_bits bits (8-bit passes): sort GB/s by the fixed formula
    K * (8 + 24 * ceil(B / 8)) bytes over the measured time."""
    import numpy as np
    import torch

    import torpedo_gb300 as T
    from torpedo_gb300 import _lib as L

    dev = torch.device("cuda", torch.cuda.current_device())
    with torch.cuda.stream(stream):
        keys = torch.empty(K, dtype=torch.int64, device=dev)
        vals = torch.empty(K, dtype=torch.int32, device=dev)
        lib = T.load()
        assert lib.tpd_read_buffer(eng._h, L.TPD_BUF_KEYS, keys.data_ptr(), 0, K * 8, 1) == 0
        assert lib.tpd_read_buffer(eng._h, L.TPD_BUF_VALUES, vals.data_ptr(), 0, K * 4, 1) == 0
        g = torch.Generator(device=dev)
        g.manual_seed(0)
        perm = torch.randperm(K, device=dev, generator=g)
        keys0, vals0 = keys[perm].contiguous(), vals[perm].contiguous()
        reps = max(3, min(20, steps // 10))
        times = []
        for _ in range(reps + 2):
            k, v = keys0.clone(), vals0.clone()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            T.sort_pairs(k, v, key_bits)
            b.record(stream)
            b.synchronize()
            times.append(a.elapsed_time(b))
        ms = float(np.median(times[2:]))
    hbm, _ = peaks()
    alg = K * (8 + 24 * math.ceil(key_bits / 8))
    return {"keys": K, "key_bits": key_bits, "passes": math.ceil(key_bits / 8), "ms": round(ms, 4),
            "algorithmic_GBps": round(alg / (ms / 1000) / 1e9, 1), "frac_of_hbm": round(alg / (ms / 1000) / 1e9 / hbm, 4),
            "keys_per_s": round(K / (ms / 1000), 1),
            "input": "the frame's keys in a seeded random order; timed with CUDA events, median"}


def kernels_per_frame(views: int, tile_passes: int, counted: bool = True) -> int:
    """Kernel launches of one frame: frame_begin, preprocess, depth-sort passes
    (a pass whose digit is the same for every key launches and returns), the
    depth-order scan fused with keygen, tile-id sort passes (counted passes: a
    counting and a scatter kernel each; the last scatter also writes the tile
    ranges), blend."""
    depth_passes = math.ceil((32 + (views - 1).bit_length()) / 8)
    return 4 + depth_passes + tile_passes * (2 if counted else 1)


def _params(sc, dev):
    import numpy as np
    import torch

    return [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in
            (sc.means, sc.log_scales, sc.quats, sc.opacity_logits, sc.sh)]


def train_rate(cfg_name, stream, local, steps, warmup, settings, stage_steps=0):
    """Forward + backward steps (one captured graph each) on every view of a
    config at once; returns (ms per step, stats, views, pixels, stages, extra):
    with stage_steps > 0 also the per-stage ms of a step (another engine with
    stage timing runs that many steps eagerly, CUDA events between stages),
    and the device memory the engine holds (cudaMemGetInfo before and after)."""
    import torch

    import torpedo_gb300 as T
    from torpedo_gb300 import configs

    dev = torch.device("cuda", local)
    cfg = configs.CONFIGS[cfg_name]
    sc = configs.scene(cfg)
    cams = configs.cameras(cfg)
    params = _params(sc, dev)
    pixels = sum(c.width * c.height for c in cams)
    gen = torch.Generator(device=dev)
    gen.manual_seed(int(cfg.name[3:]))
    dimg = torch.randn(pixels * 3, generator=gen, device=dev)
    grads = [torch.empty_like(p) for p in params]
    torch.cuda.synchronize(dev)
    free0 = torch.cuda.mem_get_info(dev)[0]

    def engine(**extra):
        e = T.GaussianEngine(device=local, stream=stream.cuda_stream, **settings, **extra)
        e.compile_params(*params)
        if len(cams) == 1:
            e.set_camera(cams[0])
        else:
            e.set_views(cams)
        e.raster_frame()
        return e

    eng = engine()
    try:
        eng.step_async(dimg, grads, max(3, warmup))
        eng.sync()
        held = free0 - torch.cuda.mem_get_info(dev)[0]
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        eng.step_async(dimg, grads, steps)
        b.record(stream)
        st = eng.sync()
        ms = a.elapsed_time(b) / steps
    finally:
        eng.close()
    stages = None
    if stage_steps:
        eng = engine(stage_timing=True)
        try:
            eng.step_async(dimg, grads, 1)
            eng.sync()
            eng.stage_times(reset=True)
            eng.step_async(dimg, grads, stage_steps)
            eng.sync()
            tot, nfr = eng.stage_times()
            stages = {k: round(v / max(1, nfr), 4) for k, v in tot.items() if k != "ranges"}
        finally:
            eng.close()
    return ms, st, len(cams), pixels, stages, {"device_bytes_held": int(held)}


def train_tune(cfg_name, stream, local, base, frames=4, warmup=2):
    """The training-step autotuner (torpedo_gb300.autotune.TRAIN_AXES: the
    blend's batch depths and its persistent form) on a config's forward +
    backward step; returns (settings, {candidate: ms per step})."""
    import torch

    import torpedo_gb300 as T
    from torpedo_gb300 import autotune, configs

    dev = torch.device("cuda", local)
    cfg = configs.CONFIGS[cfg_name]
    sc = configs.scene(cfg)
    cams = configs.cameras(cfg)
    params = _params(sc, dev)
    gen = torch.Generator(device=dev)
    gen.manual_seed(int(cfg.name[3:]))
    dimg = torch.randn(sum(c.width * c.height for c in cams) * 3, generator=gen, device=dev)
    grads = [torch.empty_like(p) for p in params]

    def make(settings):
        e = T.GaussianEngine(device=local, stream=stream.cuda_stream, **settings)
        e.compile_params(*params)
        if len(cams) == 1:
            e.set_camera(cams[0])
        else:
            e.set_views(cams)
        e.raster_frame()
        return e

    return autotune.tune(make, lambda e, k: e.step_async(dimg, grads, k), stream, frames=frames, warmup=warmup,
                         axes=autotune.TRAIN_AXES, base=base)


def plain_views_rate(cfg_name, local, passes, settings):
    """The plain pipeline on the same views: per view set_camera, raster_frame
    and backward, each call returning when its work is done (one engine per
    image size, so no view reallocates buffers). Returns views/s."""
    import torch

    import torpedo_gb300 as T
    from torpedo_gb300 import configs

    dev = torch.device("cuda", local)
    cfg = configs.CONFIGS[cfg_name]
    sc = configs.scene(cfg)
    cams = configs.cameras(cfg)
    params = _params(sc, dev)
    engines = {}
    grads = [torch.empty_like(p) for p in params]
    gen = torch.Generator(device=dev)
    gen.manual_seed(int(cfg.name[3:]))
    dimgs = [torch.randn(c.width * c.height * 3, generator=gen, device=dev) for c in cams]
    try:
        for c in cams:
            if (c.width, c.height) not in engines:
                e = T.GaussianEngine(device=local, **settings)
                e.compile_params(*params)
                engines[(c.width, c.height)] = e

        def one_pass():
            for c, d in zip(cams, dimgs):
                e = engines[(c.width, c.height)]
                e.set_camera(c)
                e.raster_frame()
                e.backward(d, *grads)

        one_pass()  # warm-up: sizes the key buffers of every engine
        best = None
        for _ in range(passes):  # the fastest pass: host round trips make single passes noisy
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            one_pass()
            torch.cuda.synchronize(dev)
            dt = time.perf_counter() - t0
            best = dt if best is None else min(best, dt)
    finally:
        for e in engines.values():
            e.close()
    return len(cams) / best


def run_train_only(args):
    """cfg2 forward + backward steps alone (one JSON line), e.g. for a profiler."""
    import torch

    torch.cuda.set_device(0)
    stream = torch.cuda.Stream(torch.device("cuda", 0))
    settings = {"sort_ctas_per_sm": args.sort_ctas or 2, "sort_threads": args.sort_threads or 512,
                "depth_sort_items": args.depth_sort_items or 16, "depth_sort_threads": args.depth_sort_threads or 256}
    ms, st, _, _, _, _ = train_rate("cfg2", stream, 0, args.steps, args.warmup, settings)
    print(json.dumps({"fwd_bwd": {"config": "cfg2", "value": round(1000.0 / ms, 3), "unit": "it/s",
                                  "ms_per_step": round(ms, 4), "keys": int(st["keys"]), "settings": settings}}))


def run_ours(args):
    import numpy as np
    import torch

    import torpedo_gb300 as T
    from torpedo_gb300 import configs

    world, rank, local = dist_setup()
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    # a dedicated stream: the engine launches on it and the timing events are recorded on it
    stream = torch.cuda.Stream(dev)
    assert stream.cuda_stream != 0

    cfg = configs.CONFIGS[args.config]
    sc = configs.scene(cfg)
    cam = configs.cameras(cfg)[0]

    def make_engine(settings, stage_timing=False):
        e = T.GaussianEngine(device=local, stream=stream.cuda_stream, stage_timing=stage_timing, **settings)
        e.compile(sc.records)
        e.set_camera(cam)
        e.raster_frame()
        return e

    if args.no_autotune:
        settings, tuned = {}, None  # the engine's defaults
    elif args.sort_ctas:
        settings, tuned = {"sort_ctas_per_sm": args.sort_ctas, "sort_threads": args.sort_threads,
                           "depth_sort_items": args.depth_sort_items,
                           "depth_sort_threads": args.depth_sort_threads}, None
    else:
        from torpedo_gb300 import autotune

        settings, tuned = autotune.tune(make_engine, lambda e, k: e.raster_frames_async(k), stream)
    eng = make_engine(settings)
    st = eng.raster_frame()
    launches_per_frame = kernels_per_frame(1, int(st["sort_passes"]), not settings.get("key_sort_lookback", 0))

    def barrier():
        torch.cuda.synchronize(dev)
        if dist:
            dist.barrier()

    def max_over_ranks(x: float) -> float:
        if not dist:
            return x
        t = torch.tensor([x], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    # warm-up
    eng.raster_frames_async(max(3, args.warmup))
    eng.sync()

    clocks = Clocks(local)
    barrier()
    clocks.start()
    time.sleep(0.3)
    # timed regions: value is the median of REGIONS regions of exactly
    # args.steps frames each, every region bracketed by barrier + synchronize
    # and timed with CUDA events on the engine's stream, max over ranks
    region_ms = []
    for _ in range(REGIONS):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        barrier()
        e0.record(stream)
        eng.raster_frames_async(args.steps)
        e1.record(stream)
        st = eng.sync()
        barrier()
        region_ms.append(max_over_ranks(e0.elapsed_time(e1)))
    clk = clocks.stop()
    ms = sorted(region_ms)[len(region_ms) // 2]
    value = world * args.steps / (ms / 1000.0)

    # stage-timed region: live per-stage durations for the roofline
    eng_t = make_engine(settings, stage_timing=True)
    eng_t.stage_times(reset=True)
    barrier()
    eng_t.raster_frames_async(args.steps)
    eng_t.sync()
    stage_ms, nfr = eng_t.stage_times()
    eng_t.close()
    stage_avg = {k: v / max(1, nfr) for k, v in stage_ms.items() if k in FRAME_STAGES}

    # end to end through the C ABI with host buffers
    e2e = None
    if not args.no_e2e:
        # two frames in flight through the public API: per step the camera goes
        # up from pinned host memory and the RGBA8 image comes back into pinned
        # host memory (its copy overlaps the next frame)
        img_host = [torch.empty(cam.width * cam.height * 4, dtype=torch.uint8, pin_memory=True) for _ in range(2)]
        barrier()
        t0 = time.perf_counter()
        for i in range(args.steps):
            eng.set_camera(cam)
            eng.render_async(img_host[i % 2], rgba8=True)
            if i >= 1:
                eng.wait_render()
        eng.wait_render()
        barrier()
        dt = max_over_ranks(time.perf_counter() - t0)
        e2e = {"value": round(world * args.steps / dt, 3), "unit": UNIT, "h2d_bytes_per_step": 160,
               "d2h_bytes_per_step": cam.width * cam.height * 4,
               "api": "set_camera + tpd_render_async (RGBA8 into pinned host memory) + tpd_wait_render, "
                      "two frames in flight"}

    K = int(st["keys"])
    passes = int(st["sort_passes"])  # tile-id passes of the key sort
    key_bits = int(st["key_bits"])
    hbm, peak_kind = peaks()
    sort_formula = K * (8 + 24 * math.ceil(key_bits / 8))
    pass_ms = stage_avg["key_sort"] / passes
    achieved = K * 24 / (pass_ms / 1000.0) / 1e9
    # DRAM bytes per key of one pass, from the committed ncu capture of the
    # pass's kernels (read + write), times K
    counted = not settings.get("key_sort_lookback")
    traffic = None
    tfile = ROOT / "profiles" / "radix_pass_traffic.json"
    if tfile.exists():
        t = json.loads(tfile.read_text())
        per_key = t.get("counted" if counted else "onesweep")
        traffic = int(per_key * K) if per_key else None
    pass_kernel = ("partition_count_kernel (chunk_scan_kernel in the first pass) + scatter_kernel "
                   "(one counted 8-bit tile-id radix pass of the key sort)"
                   if counted else "onesweep_kernel (one 8-bit tile-id radix pass of the key sort)")
    general = general_sort(eng, K, key_bits, stream, args.steps) if not args.no_general_sort else None
    eng.close()

    # blend: evaluated (pixel, entry) pairs of this workload, counted on the CPU
    # by the oracle's rules (oracle/count_blend_pairs.py) and committed
    blend = None
    pfile = ROOT / "profiles" / f"blend_pairs_{cfg.name}.json"
    if pfile.exists():
        pc = json.loads(pfile.read_text())
        if int(pc["keys"]) == K:
            sm_count = torch.cuda.get_device_properties(dev).multi_processor_count
            fp32_peak = sm_count * 128 * 2 * float(json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
                                                   .get("sm_max_mhz", 2070.0)) * 1e6 / 1e12 \
                if (ROOT / "MEASURED_PEAKS.json").exists() else sm_count * 128 * 2 * 2.07e9 / 1e12
            pairs_s = pc["evaluated_pairs"] / (stage_avg["blend"] / 1000.0)
            blend = {"kernel": "blend_kernel", "bound": "sm fp32 / issue", "evaluated_pairs": pc["evaluated_pairs"],
                     "contributing_pairs": pc["contributing_pairs"], "ms": round(stage_avg["blend"], 4),
                     "pairs_per_s": round(pairs_s, 1), "achieved_tflops": round(pairs_s * 20 / 1e12, 2),
                     "peak_tflops": round(fp32_peak, 1), "frac": round(pairs_s * 20 / 1e12 / fp32_peak, 4),
                     "note": "20 FP32 operations per evaluated pair; peak = SMs x 128 FP32 lanes x 2 x max SM clock"}

    fwd_bwd = batched = large = None
    tuned_train = {}
    if not args.no_train:
        settings2, tuned_train["cfg2"] = train_tune("cfg2", stream, local, settings, frames=20, warmup=3)
        ms2, st2, _, _, _, _ = train_rate("cfg2", stream, local, 50, 3, settings2)
        fwd_bwd = {"config": "cfg2: 200,000 Gaussians (means N(0,1)^3), one 800x800 view, dL/dimage ~ N(0,1)",
                   "value": round(1000.0 / ms2, 3), "unit": "it/s", "ms_per_step": round(ms2, 4),
                   "keys": int(st2["keys"]), "settings": settings2,
                   "step": "forward frame + backward to means, log-scales, quaternions, opacity logits, SH; "
                           "one captured CUDA graph per step"}
        settings3, tuned_train["cfg3"] = train_tune("cfg3", stream, local, settings)
        ms3, st3, views3, pixels3, stages3, _ = train_rate("cfg3", stream, local, 5, 2, settings3, stage_steps=2)
        plain = plain_views_rate("cfg3", local, 3, settings3)
        batched = {"config": "cfg3: 500,000 Gaussians (means N(0,1)^3), 64 views on a sphere of radius 5, sizes "
                             "from {640x480, 1280x720, 1920x1080} (seed 3), dL/dimage ~ N(0,1)",
                   "views_per_s": round(views3 * 1000.0 / ms3, 2), "ms_per_step": round(ms3, 3),
                   "keys": int(st3["keys"]), "pixels": pixels3,
                   "plain_views_per_s": round(plain, 2), "batched_over_plain": round(views3 * 1000.0 / ms3 / plain, 3),
                   "plain": "one view per call: set_camera, raster_frame, backward, each waiting for its work; "
                            "fastest of 3 passes over the 64 views",
                   "stages_ms": stages3, "settings": settings3,
                   "stages_note": "per step, from 2 eager steps with CUDA events between stages (no graph)"}
        if not args.no_large:
            ms4, st4, views4, pixels4, _, ex4 = train_rate("cfg4", stream, local, 3, 1, settings3)
            large = {"config": "cfg4: 6,000,000 Gaussians (means U[-10,10]^3), 8 views of 3840x2160, "
                               "dL/dimage ~ N(0,1)",
                     "views_per_s": round(views4 * 1000.0 / ms4, 2), "ms_per_step": round(ms4, 3),
                     "keys": int(st4["keys"]), "key_capacity": int(st4["key_capacity"]), "pixels": pixels4,
                     "device_bytes_held": ex4["device_bytes_held"],
                     "step": "forward + backward of the 8 views as one captured graph per step"}

    line = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": max(3, args.warmup), "ms_per_step": round(ms / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded cfg1 generator)",
        "config": workload_config(cfg, cam.width, cam.height, K),
        "roofline": {"bound": "hbm", "kernel": pass_kernel,
                     "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                     "frac": round(achieved / hbm, 4), "traffic": traffic, "peak_kind": f"{peak_kind} copy bandwidth",
                     "bytes_per_launch": K * 24, "avg_launch_ms": round(pass_ms, 5),
                     "basis": "K * 24 B per 8-bit pass: the per-pass term of the fixed sort formula "
                              "K * (8 + 24 * ceil(B / 8)) for 64-bit keys and 32-bit values",
                     "moved_bytes_per_launch": K * 16,
                     "moved_GBps": round(K * 16 / (pass_ms / 1000.0) / 1e9, 1),
                     "moved_frac": round(K * 16 / (pass_ms / 1000.0) / 1e9 / hbm, 4),
                     "moved_note": "the pass itself reads and writes 32-bit tile ids and 32-bit values "
                                   "(16 B per key); the depth half of the keys is ordered by the depth presort",
                     "time_note": "avg_launch_ms = the key-sort stage / its passes; with counted passes the first "
                                  "pass's per-partition digit counts are added by keygen_scan_kernel as it writes "
                                  "the keys (their cost is in the keygen stage, about 0.005 ms at 1080p), and that "
                                  "pass's counting launch only scans them"},
        "frame_sort": {"keys": K, "key_bits": key_bits, "tile_passes": passes,
                       "depth_sort_ms": round(stage_avg["depth_sort"], 4), "key_sort_ms": round(stage_avg["key_sort"], 4),
                       "formula_GBps": round(sort_formula / ((stage_avg["depth_sort"] + stage_avg["key_sort"]) / 1000) / 1e9, 1),
                       "frac_of_hbm": round(sort_formula / ((stage_avg["depth_sort"] + stage_avg["key_sort"]) / 1000) / 1e9
                                            / hbm, 4),
                       "note": "Gaussians sorted by depth first (N items), then the K keys on their tile-id bits "
                               "only; GB/s by the fixed formula K * (8 + 24 * ceil(B / 8)) bytes over that time: "
                               "algorithmic credit for passes the presort makes unnecessary, not bandwidth"},
        "general_sort": general,
        "blend": blend,
        "stages_ms": {k: round(v, 4) for k, v in stage_avg.items()},
        "gpu_launches": launches_per_frame * args.steps,
        "clocks": clk,
        "autotune": {"settings": settings, "ms_per_frame": tuned, "train_ms_per_step": tuned_train},
        "fwd_bwd": fwd_bwd,
        "batched": batched,
        "large": large,
        "timed_regions_ms": [round(x, 4) for x in region_ms],
    }
    if e2e:
        line["e2e"] = e2e
    if rank == 0 and world == 1 and args.cpu_baseline_s > 0:
        from oracle import oracle as O

        threads = os.cpu_count() or 1
        oc = O.camera(cam.view, cam.projview(), cam.width, cam.height, focal=(cam.proj[0, 0], cam.proj[1, 1]))
        times, k = cpu_frames(sc.records, oc, args.cpu_baseline_s, threads, 50)
        line["cpu_baseline"] = {"value": round(len(times) / sum(times), 4), "unit": UNIT, "cores": threads,
                                "kind": "port",
                                "sample": f"{len(times)} whole frames of the FP32 transcription of the reference "
                                          f"shaders (4-way radix sort), K={k}"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", default="cfg1")
    ap.add_argument("--cpu-baseline-s", type=float, default=15.0)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-general-sort", action="store_true")
    ap.add_argument("--sort-ctas", type=int, default=0,
                    help="radix pass kernel residency (2 or 3 CTAs per SM); 0 = autotune")
    ap.add_argument("--sort-threads", type=int, default=0, help="with --sort-ctas: radix CTA size (256 or 512)")
    ap.add_argument("--depth-sort-items", type=int, default=0, help="with --sort-ctas: depth sort keys per thread")
    ap.add_argument("--depth-sort-threads", type=int, default=0, help="with --sort-ctas: depth sort CTA size (256 or 512)")
    ap.add_argument("--no-autotune", action="store_true", help="the engine's default settings (e.g. for a profiler)")
    ap.add_argument("--no-train", action="store_true", help="skip the cfg2, cfg3 and cfg4 forward+backward measurements")
    ap.add_argument("--no-large", action="store_true", help="skip the cfg4 forward+backward measurement")
    ap.add_argument("--train-only", action="store_true", help="only the cfg2 forward+backward steps (profiling)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.train_only:
        run_train_only(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
