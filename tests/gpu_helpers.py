"""Shared plumbing of the GPU parity tests: render through the C ABI, read the
engine's buffers back, and run the oracle on the same inputs."""
from __future__ import annotations

import numpy as np

import torpedo_gb300 as T
from oracle import oracle as O
from torpedo_gb300 import _lib as L


def ocam(cam: T.Camera):
    return O.camera(cam.view, cam.projview(), cam.width, cam.height, focal=(cam.proj[0, 0], cam.proj[1, 1]))


def render(records, cams, entity_index=None, n_entities=1, transforms=None, **kw):
    eng = T.GaussianEngine(**kw)
    eng.compile(records, entity_index, n_entities)
    if transforms is not None:
        for e, m in enumerate(transforms):
            eng.transform_host.transform(e, m)
    if len(cams) == 1:
        eng.set_camera(cams[0])
    else:
        eng.set_views(cams)
    stats = eng.raster_frame()
    return eng, stats


def gpu_state(eng: T.GaussianEngine, stats: dict) -> dict:
    n = eng.n
    v = stats["views"]
    k = stats["keys"]
    out = {
        "splats": eng.read_buffer(L.TPD_BUF_SPLATS, np.uint32, v * n * 12).reshape(v * n, 12),
        "offsets": eng.read_buffer(L.TPD_BUF_OFFSETS, np.uint32, v * n),
        "keys": eng.read_buffer(L.TPD_BUF_KEYS, np.uint64, k),
        "vals": eng.read_buffer(L.TPD_BUF_VALUES, np.uint32, k),
        "ranges": eng.read_buffer(L.TPD_BUF_RANGES, np.uint32, stats["tiles"] * 2).reshape(-1, 2),
        "images": eng.read_image(),
        "final_T": eng.read_buffer(L.TPD_BUF_FINAL_T, np.float32, eng.pixels),
        "n_contrib": eng.read_buffer(L.TPD_BUF_N_CONTRIB, np.uint32, eng.pixels),
        "K": k,
    }
    return out


def oracle_frame(records, cam, sh_degree=3, band3_compat=True, ent_idx=None, transforms=None, f64=True):
    oc = ocam(cam)
    s32 = O.preprocess_f32(records, oc, sh_degree, band3_compat, ent_idx, transforms)
    offs, k = O.scan_tiles(s32)
    keys, vals = O.keygen(s32, offs, k, cam.width, cam.height)
    skeys, svals = O.stable_sort(keys, vals)
    n_tiles = ((cam.width + 15) // 16) * ((cam.height + 15) // 16)
    rng = O.tile_ranges(skeys, n_tiles)
    # key offsets in depth order (the engine scans tile counts after sorting the
    # Gaussians by (depth bits, index); culled ones, depth key 0xFFFFFFFF, go
    # last here and are dropped by the engine's depth sort)
    dkey = np.where(s32[:, 3] > 0, s32[:, 6], np.uint32(0xFFFFFFFF)).astype(np.uint32)
    order = np.argsort(dkey, kind="stable")
    cnt = s32[order, 3].astype(np.uint64)
    doffs = (np.cumsum(cnt) - cnt).astype(np.uint32)
    out = dict(s32=s32, offsets=offs, depth_offsets=doffs, K=k, keys_unsorted=keys, vals_unsorted=vals, keys=skeys,
               vals=svals, ranges=rng)
    if f64:
        s64, rect, frag = O.preprocess_f64(records, oc, sh_degree, band3_compat, ent_idx, transforms)
        img64, T64, nc64, pfrag = O.blend_f64(s64, svals, rng, cam.width, cam.height)
        out.update(s64=s64, rect=rect, frag=frag, img64=img64, T64=T64, nc64=nc64, pfrag=pfrag)
    return out
