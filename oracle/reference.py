"""The reference's own compute shaders run on the CPU (oracle/_ref/libtpdref.so,
built by oracle/build_ref.py from the reference's Slang source where the
reference tree is present).

TEST INFRASTRUCTURE ONLY: tests/golden/make_golden.py records golden vectors
with it, and tests check against it when it is built. The product never uses
it.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import build_ref

_lib = None


def available() -> bool:
    return build_ref.LIB.exists() or build_ref.available()


def load():
    global _lib
    if _lib is None:
        lib = C.CDLL(str(build_ref.build()))
        P = C.c_void_p
        lib.ref_frame_run.restype = P
        lib.ref_frame_run.argtypes = [P, C.c_uint32, P, P, C.c_uint32, P, P, P, C.c_uint32, C.c_uint32, C.c_uint32]
        lib.ref_frame_keys.restype = C.c_uint64
        lib.ref_frame_keys.argtypes = [P]
        lib.ref_frame_oob.restype = C.c_uint64
        lib.ref_frame_oob.argtypes = [P]
        lib.ref_frame_passes.restype = C.c_uint32
        lib.ref_frame_passes.argtypes = [P]
        lib.ref_frame_copy.argtypes = [P, P, P, P, P, P, P]
        lib.ref_frame_free.argtypes = [P]
        _lib = lib
    return _lib


def frame(records, view, projview, focal, width: int, height: int, sh_degree: int = 3, ent_idx=None,
          transforms=None) -> dict:
    """One frame of the reference's shaders: splats after project (n x 12
    words), offsets after prefix (n), sorted keys and values (K), ranges
    (tiles x 2), the stored image (h x w x 4 float32), K, the radix pass count
    and the number of out-of-range buffer accesses (0 for a sound run)."""
    lib = load()
    recs = np.ascontiguousarray(records, np.float32)
    n = recs.shape[0]
    v = np.ascontiguousarray(view, np.float32).reshape(16)
    pv = np.ascontiguousarray(projview, np.float32).reshape(16)
    fo = np.ascontiguousarray(focal, np.float32).reshape(2)
    ei = np.ascontiguousarray(ent_idx, np.uint32) if ent_idx is not None else None
    tr = np.ascontiguousarray(transforms, np.float32) if transforms is not None else None
    n_ent = tr.reshape(-1, 16).shape[0] if tr is not None else 0
    f = lib.ref_frame_run(recs.ctypes.data if n else None, n, ei.ctypes.data if ei is not None else None,
                          tr.ctypes.data if tr is not None else None, n_ent, v.ctypes.data, pv.ctypes.data,
                          fo.ctypes.data, width, height, sh_degree)
    try:
        k = int(lib.ref_frame_keys(f))
        tiles = ((width + 15) // 16) * ((height + 15) // 16)
        out = dict(splats=np.zeros((n, 12), np.uint32), offsets=np.zeros(n, np.uint32), keys=np.zeros(k, np.uint64),
                   vals=np.zeros(k, np.uint32), ranges=np.zeros((tiles, 2), np.uint32),
                   image=np.zeros((height, width, 4), np.float32))
        lib.ref_frame_copy(f, *[out[x].ctypes.data if out[x].size else None
                                for x in ("splats", "offsets", "keys", "vals", "ranges", "image")])
        out.update(K=k, passes=int(lib.ref_frame_passes(f)), oob=int(lib.ref_frame_oob(f)))
        return out
    finally:
        lib.ref_frame_free(f)
