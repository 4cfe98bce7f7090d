"""ctypes wrapper of the CPU oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() (as the
checker) and bench.py's CPU-baseline legs. The product never imports this.
See tpd_oracle.h for what each function restates; shader maths is "parity
unpinned" (the reference's Slang/Vulkan path cannot run here and ships no
golden vectors), host camera / pass-count inputs are pinned by the fixtures
in tests/golden/.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
_lib = None


class OrcCamera(C.Structure):
    _fields_ = [("view", C.c_float * 16), ("projview", C.c_float * 16), ("focal", C.c_float * 2),
                ("width", C.c_uint32), ("height", C.c_uint32)]


class OrcParams64(C.Structure):
    _fields_ = [("means", C.c_void_p), ("log_scales", C.c_void_p), ("quats", C.c_void_p),
                ("opacity_logits", C.c_void_p), ("sh", C.c_void_p)]


def load():
    global _lib
    if _lib is None:
        from . import build as _b  # noqa: F401  (oracle/build.py)
        path = _b.build()
        lib = C.CDLL(str(path))
        P = C.c_void_p
        sig = {
            "orc_preprocess_f32": (None, [P, C.c_uint32, P, P, C.POINTER(OrcCamera), C.c_uint32, C.c_int, P]),
            "orc_preprocess_f64": (None, [P, C.c_uint32, P, P, C.POINTER(OrcCamera), C.c_uint32, C.c_int, P, P, P]),
            "orc_scan_tiles": (C.c_uint64, [P, C.c_uint32, P]),
            "orc_keygen": (None, [P, P, C.c_uint32, C.c_uint32, C.c_uint32, P, P]),
            "orc_stable_sort_pairs": (None, [P, P, C.c_uint64]),
            "orc_radix4_sort": (None, [P, P, C.c_uint64, C.c_uint32, C.c_int]),
            "orc_higher_msb": (C.c_uint32, [C.c_uint32]),
            "orc_radix_pass_count": (C.c_uint32, [C.c_uint32, C.c_uint32]),
            "orc_tile_ranges": (None, [P, C.c_uint64, C.c_uint32, P]),
            "orc_blend_f32": (None, [P, P, P, C.c_uint32, C.c_uint32, P, P, P, C.c_int]),
            "orc_blend_f64": (None, [P, P, P, C.c_uint32, C.c_uint32, P, P, P, P]),
            "orc_blend_pair_count": (None, [P, P, P, C.c_uint32, C.c_uint32, P, P, C.c_int]),
            "orc_frame_f32": (C.c_uint64, [P, C.c_uint32, C.POINTER(OrcCamera), C.c_uint32, P, C.c_int, C.c_uint32]),
            "orc_render_params_f64": (None, [C.POINTER(OrcParams64), C.c_uint32, C.POINTER(OrcCamera), C.c_uint32,
                                             C.c_int, P, P, P]),
            "orc_backward_f64": (None, [C.POINTER(OrcParams64), C.c_uint32, C.POINTER(OrcCamera), C.c_uint32, C.c_int,
                                        P, P, P, P, P, P, P, P, P]),
            "orc_look_at": (None, [P, P, P, P]),
            "orc_perspective": (None, [C.c_uint32, C.c_uint32, C.c_float, C.c_float, C.c_float, P]),
            "orc_mat4_mul": (None, [P, P, P]),
            "orc_synthetic_scene": (None, [C.c_uint64, C.c_uint32, C.c_float, P]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def _c(a, dtype):
    return np.ascontiguousarray(np.asarray(a, dtype=dtype))


def look_at(eye, center, up) -> np.ndarray:
    """Camera::lookAt with the reference's accurate arithmetic: 4x4 row-major float32."""
    e, c, u = (_c(v, np.float32).reshape(3) for v in (eye, center, up))
    out = np.zeros((4, 4), np.float32)
    load().orc_look_at(e.ctypes.data, c.ctypes.data, u.ctypes.data, out.ctypes.data)
    return out


def perspective(width: int, height: int, fov_y_degrees: float, near: float, far: float) -> np.ndarray:
    """PerspectiveCamera's reversed-Z projection: 4x4 row-major float32."""
    out = np.zeros((4, 4), np.float32)
    load().orc_perspective(width, height, fov_y_degrees, near, far, out.ctypes.data)
    return out


def mat4_mul(a, b) -> np.ndarray:
    """math::mul(a, b) with the reference's accurate dot product."""
    a, b = _c(a, np.float32), _c(b, np.float32)
    out = np.zeros((4, 4), np.float32)
    load().orc_mat4_mul(a.ctypes.data, b.ctypes.data, out.ctypes.data)
    return out


def orbit_camera(eye, width: int, height: int, fov_y_degrees=60.0, near=0.2, far=100.0, up=(0.0, -1.0, 0.0)):
    """Camera constants of a view at `eye` looking at the origin, as updateCameraBuffer packs them."""
    view = look_at(eye, (0.0, 0.0, 0.0), up)
    proj = perspective(width, height, fov_y_degrees, near, far)
    return camera(view, mat4_mul(proj, view), width, height, focal=(proj[0, 0], proj[1, 1]))


def synthetic_records(seed: int, n: int, mean_box: float = 0.0) -> np.ndarray:
    """The seeded synthetic scene of the workloads as (n, 60) float32 records."""
    rec = np.zeros((n, 60), np.float32)
    load().orc_synthetic_scene(seed, n, float(mean_box), rec.ctypes.data)
    return rec


def camera(view, projview, width: int, height: int, focal=None) -> OrcCamera:
    """Camera constants as updateCameraBuffer packs them; focal defaults to (proj[0,0], proj[1,1]) given separately."""
    c = OrcCamera()
    c.view[:] = list(_c(view, np.float32).reshape(16))
    c.projview[:] = list(_c(projview, np.float32).reshape(16))
    f = focal if focal is not None else (1.0, 1.0)
    c.focal[0], c.focal[1] = float(f[0]), float(f[1])
    c.width, c.height = width, height
    return c


def preprocess_f32(recs, cam: OrcCamera, sh_degree=3, band3_compat=True, ent_idx=None, transforms=None):
    recs = _c(recs, np.float32)
    n = recs.shape[0]
    out = np.zeros((n, 12), np.uint32)
    ei = _c(ent_idx, np.uint32) if ent_idx is not None else None
    tr = _c(transforms, np.float32) if transforms is not None else None
    load().orc_preprocess_f32(recs.ctypes.data, n, ei.ctypes.data if ei is not None else None,
                              tr.ctypes.data if tr is not None else None, C.byref(cam), sh_degree,
                              1 if band3_compat else 0, out.ctypes.data)
    return out


def preprocess_f64(recs, cam: OrcCamera, sh_degree=3, band3_compat=True, ent_idx=None, transforms=None):
    recs = _c(recs, np.float32)
    n = recs.shape[0]
    sp = np.zeros((n, 12), np.float64)
    rect = np.zeros((n, 4), np.uint32)
    frag = np.zeros(n, np.uint8)
    ei = _c(ent_idx, np.uint32) if ent_idx is not None else None
    tr = _c(transforms, np.float32) if transforms is not None else None
    load().orc_preprocess_f64(recs.ctypes.data, n, ei.ctypes.data if ei is not None else None,
                              tr.ctypes.data if tr is not None else None, C.byref(cam), sh_degree,
                              1 if band3_compat else 0, sp.ctypes.data, rect.ctypes.data, frag.ctypes.data)
    return sp, rect, frag.astype(bool)


def scan_tiles(splats_u32):
    s = _c(splats_u32, np.uint32)
    offs = np.zeros(s.shape[0], np.uint32)
    total = load().orc_scan_tiles(s.ctypes.data, s.shape[0], offs.ctypes.data)
    return offs, int(total)


def keygen(splats_u32, offsets, total, width, height):
    s = _c(splats_u32, np.uint32)
    o = _c(offsets, np.uint32)
    keys = np.zeros(total, np.uint64)
    vals = np.zeros(total, np.uint32)
    load().orc_keygen(s.ctypes.data, o.ctypes.data, s.shape[0], width, height, keys.ctypes.data, vals.ctypes.data)
    return keys, vals


def stable_sort(keys, vals):
    k = _c(keys, np.uint64).copy()
    v = _c(vals, np.uint32).copy()
    load().orc_stable_sort_pairs(k.ctypes.data, v.ctypes.data, k.shape[0])
    return k, v


def radix4_sort(keys, vals, passes, threads=0):
    k = _c(keys, np.uint64).copy()
    v = _c(vals, np.uint32).copy()
    load().orc_radix4_sort(k.ctypes.data, v.ctypes.data, k.shape[0], passes, threads)
    return k, v


def higher_msb(n: int) -> int:
    return int(load().orc_higher_msb(n))


def radix_pass_count(width: int, height: int) -> int:
    return int(load().orc_radix_pass_count(width, height))


def tile_ranges(keys, n_tiles):
    k = _c(keys, np.uint64)
    r = np.zeros((n_tiles, 2), np.uint32)
    load().orc_tile_ranges(k.ctypes.data, k.shape[0], n_tiles, r.ctypes.data)
    return r


def blend_f32(splats_u32, vals, ranges, width, height, threads=0):
    s = _c(splats_u32, np.uint32)
    v = _c(vals, np.uint32)
    r = _c(ranges, np.uint32)
    img = np.zeros((height, width, 3), np.float32)
    T = np.zeros((height, width), np.float32)
    nc = np.zeros((height, width), np.uint32)
    load().orc_blend_f32(s.ctypes.data, v.ctypes.data if v.size else None, r.ctypes.data, width, height,
                         img.ctypes.data, T.ctypes.data, nc.ctypes.data, threads)
    return img, T, nc


def blend_pair_count(splats_u32, vals, ranges, width, height, threads=0):
    """(evaluated, contributing) (pixel, entry) pairs of the FP32 blend's rules."""
    s = _c(splats_u32, np.uint32)
    v = _c(vals, np.uint32)
    r = _c(ranges, np.uint32)
    ev, co = C.c_uint64(0), C.c_uint64(0)
    load().orc_blend_pair_count(s.ctypes.data, v.ctypes.data if v.size else None, r.ctypes.data, width, height,
                                C.byref(ev), C.byref(co), threads)
    return int(ev.value), int(co.value)


def blend_f64(splat64, vals, ranges, width, height):
    s = _c(splat64, np.float64)
    v = _c(vals, np.uint32)
    r = _c(ranges, np.uint32)
    img = np.zeros((height, width, 3), np.float64)
    T = np.zeros((height, width), np.float64)
    nc = np.zeros((height, width), np.uint32)
    frag = np.zeros((height, width), np.uint8)
    load().orc_blend_f64(s.ctypes.data, v.ctypes.data if v.size else None, r.ctypes.data, width, height,
                         img.ctypes.data, T.ctypes.data, nc.ctypes.data, frag.ctypes.data)
    return img, T, nc, frag.astype(bool)


def frame_f32(recs, cam: OrcCamera, sh_degree=3, threads=0, tile_rows_limit=0):
    recs = _c(recs, np.float32)
    h = cam.height
    gy = (cam.height + 15) // 16
    if tile_rows_limit and tile_rows_limit < gy:
        h = tile_rows_limit * 16
    img = np.zeros((h, cam.width, 3), np.float32)
    k = load().orc_frame_f32(recs.ctypes.data, recs.shape[0], C.byref(cam), sh_degree, img.ctypes.data, threads,
                             tile_rows_limit)
    return img, int(k)


def _params64(means, log_scales, quats, logits, sh):
    arrs = [_c(a, np.float64) for a in (means, log_scales, quats, logits, sh)]
    p = OrcParams64(*[a.ctypes.data for a in arrs])
    return p, arrs


def render_params_f64(params, cam: OrcCamera, vals, ranges, sh_degree=3, band3_compat=True):
    p, keep = _params64(*params)
    n = keep[0].shape[0]
    img = np.zeros((cam.height, cam.width, 3), np.float64)
    v = _c(vals, np.uint32)
    r = _c(ranges, np.uint32)
    load().orc_render_params_f64(C.byref(p), n, C.byref(cam), sh_degree, 1 if band3_compat else 0,
                                 v.ctypes.data if v.size else None, r.ctypes.data, img.ctypes.data)
    return img


def backward_f64(params, cam: OrcCamera, vals, ranges, dL_dimage, sh_degree=3, band3_compat=True):
    p, keep = _params64(*params)
    n = keep[0].shape[0]
    g = [np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, 4)), np.zeros(n), np.zeros((n, 48))]
    g2d = np.zeros((n, 9))
    v = _c(vals, np.uint32)
    r = _c(ranges, np.uint32)
    d = _c(dL_dimage, np.float64)
    load().orc_backward_f64(C.byref(p), n, C.byref(cam), sh_degree, 1 if band3_compat else 0,
                            v.ctypes.data if v.size else None, r.ctypes.data, d.ctypes.data,
                            *[a.ctypes.data for a in g], g2d.ctypes.data)
    return g, g2d
