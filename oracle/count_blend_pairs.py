"""Counts the blend's work measure for a workload on the CPU: the (pixel, list
entry) pairs evaluated until each pixel terminates, and those that add colour,
by the FP32 transcription's rules over the oracle's own per-tile lists (which
equal the CUDA pipeline's bit for bit). Writes profiles/blend_pairs_<cfg>.json,
which bench.py reads to express the blend kernel's throughput as pairs/s.

    python oracle/count_blend_pairs.py cfg1
"""
from __future__ import annotations

import json
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


def count(cfg_name: str) -> dict:
    from oracle import build
    from oracle import oracle as O
    from torpedo_gb300 import configs

    build.build()
    sc = configs.scene(cfg_name)
    cams = configs.cameras(cfg_name)
    total_ev = total_co = 0
    keys = 0
    t0 = time.time()
    for cam in cams:
        oc = O.camera(cam.view, cam.projview(), cam.width, cam.height, focal=(cam.proj[0, 0], cam.proj[1, 1]))
        s32 = O.preprocess_f32(sc.records, oc)
        offs, k = O.scan_tiles(s32)
        skeys, svals = O.stable_sort(*O.keygen(s32, offs, k, cam.width, cam.height))
        n_tiles = ((cam.width + 15) // 16) * ((cam.height + 15) // 16)
        rng = O.tile_ranges(skeys, n_tiles)
        ev, co = O.blend_pair_count(s32, svals, rng, cam.width, cam.height)
        total_ev += ev
        total_co += co
        keys += int(k)
    return {"config": cfg_name, "views": len(cams), "keys": keys, "evaluated_pairs": total_ev,
            "contributing_pairs": total_co, "cpu_seconds": round(time.time() - t0, 1),
            "command": f"python oracle/count_blend_pairs.py {cfg_name}",
            "rules": "per pixel, list entries in order until T*(1-alpha) < 1e-4 (that entry counted) or the "
                     "list ends; contributing = alpha >= 1/255 and not terminating (blend.slang:24-105)"}


if __name__ == "__main__":
    name = sys.argv[1] if len(sys.argv) > 1 else "cfg1"
    out = count(name)
    (ROOT / "profiles").mkdir(exist_ok=True)
    path = ROOT / "profiles" / f"blend_pairs_{name}.json"
    path.write_text(json.dumps(out, indent=1) + "\n")
    print(json.dumps(out))
