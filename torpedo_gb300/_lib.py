"""ctypes binding of libtpdsplat.so (the C ABI declared in include/tpdsplat.h).

The library is built in-tree by torpedo_gb300.build. There is no fallback: if
the shared library is missing, loading raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_LIB_PATH = Path(__file__).resolve().parent / "_build" / "libtpdsplat.so"

TPD_OK, TPD_ERR_ARG, TPD_ERR_OOM, TPD_ERR_TIMEOUT, TPD_ERR_DEVICE, TPD_ERR_STATE, TPD_ERR_CAPACITY, TPD_ERR_IO = range(8)
TPD_IMAGE_RGB32F, TPD_IMAGE_RGBA8 = 0, 1
STAGES = ("preprocess", "depth_sort", "keygen", "key_sort", "ranges", "blend", "backward_setup", "blend_backward",
          "preprocess_backward")
# device status bits (TPD_DEVSTAT_*) and the status word's offset in a stage workspace
DEVSTAT_KEY_OVERFLOW, DEVSTAT_LOOKBACK_TIMEOUT, DEVSTAT_BAD_INPUT, DEVSTAT_BAD_INDEX = 0x1, 0x2, 0x8, 0x10
WORKSPACE_STATUS_OFFSET = 0
(TPD_BUF_RECORDS, TPD_BUF_SPLATS, TPD_BUF_OFFSETS, TPD_BUF_KEYS, TPD_BUF_VALUES, TPD_BUF_RANGES, TPD_BUF_IMAGE,
 TPD_BUF_FINAL_T, TPD_BUF_N_CONTRIB, TPD_BUF_G2D) = range(10)


class Settings(C.Structure):
    _fields_ = [
        ("sh_degree", C.c_uint32),
        ("band3_compat", C.c_uint32),
        ("device", C.c_int32),
        ("stream", C.c_void_p),
        ("use_graph", C.c_uint32),
        ("spin_limit", C.c_uint32),
        ("initial_key_capacity", C.c_uint64),
        ("timeout_s", C.c_double),
        ("test_never_publish", C.c_uint32),
        ("stage_timing", C.c_uint32),
        ("sort_ctas_per_sm", C.c_uint32),
        ("depth_sort_items", C.c_uint32),
        ("sort_threads", C.c_uint32),
        ("depth_sort_threads", C.c_uint32),
        ("blend_round", C.c_uint32),
        ("blend_backward_round", C.c_uint32),
        ("blend_persistent", C.c_uint32),
        ("key_sort_lookback", C.c_uint32),
        ("keep_backward_state", C.c_uint32),
        ("reserved", C.c_uint32 * 1),
    ]


class FrameStats(C.Structure):
    _fields_ = [
        ("keys", C.c_uint64),
        ("key_capacity", C.c_uint64),
        ("visible", C.c_uint32),
        ("tiles", C.c_uint32),
        ("key_bits", C.c_uint32),
        ("sort_passes", C.c_uint32),
        ("status", C.c_uint32),
        ("retries", C.c_uint32),
        ("views", C.c_uint32),
        ("reserved", C.c_uint32 * 5),
    ]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_ if f != "reserved"}


class View(C.Structure):
    _fields_ = [("view", C.c_float * 16), ("proj", C.c_float * 16), ("width", C.c_uint32), ("height", C.c_uint32)]


_P = C.c_void_p
_F = C.POINTER(C.c_float)
_U32 = C.c_uint32

# name -> (restype, argtypes); exactly the declarations of include/tpdsplat.h
SIGNATURES = {
    "tpd_version": (C.c_char_p, []),
    "tpd_status_string": (C.c_char_p, [C.c_int]),
    "tpd_settings_init": (None, [C.POINTER(Settings)]),
    "tpd_create": (C.c_int, [C.POINTER(Settings), C.POINTER(_P)]),
    "tpd_destroy": (None, [_P]),
    "tpd_last_error": (C.c_char_p, [_P]),
    "tpd_compile": (C.c_int, [_P, _P, _U32, _P, _U32]),
    "tpd_compile_params_device": (C.c_int, [_P, _P, _P, _P, _P, _P, _U32]),
    "tpd_set_transform": (C.c_int, [_P, _U32, _F]),
    "tpd_set_camera": (C.c_int, [_P, _F, _F, _U32, _U32]),
    "tpd_set_views": (C.c_int, [_P, C.POINTER(View), _U32]),
    "tpd_raster_frame": (C.c_int, [_P, C.POINTER(FrameStats)]),
    "tpd_raster_frames_async": (C.c_int, [_P, _U32]),
    "tpd_sync": (C.c_int, [_P, C.POINTER(FrameStats)]),
    "tpd_stage_times": (C.c_int, [_P, C.POINTER(C.c_double), C.POINTER(C.c_uint64), C.c_int]),
    "tpd_read_image": (C.c_int, [_P, _P, _U32, C.c_int]),
    "tpd_backward": (C.c_int, [_P, _P, _P, _P, _P, _P, _P]),
    "tpd_step_async": (C.c_int, [_P, _P, _P, _P, _P, _P, _P, _U32]),
    "tpd_render_async": (C.c_int, [_P, _P, _U32, C.c_int]),
    "tpd_wait_render": (C.c_int, [_P, _P]),
    "tpd_get_buffer": (C.c_int, [_P, _U32, C.POINTER(_P), C.POINTER(C.c_uint64)]),
    "tpd_read_buffer": (C.c_int, [_P, _U32, _P, C.c_uint64, C.c_uint64, C.c_int]),
    "tpd_get_stream": (_P, [_P]),
    "tpd_key_bits_for_tiles": (_U32, [_U32]),
    "tpd_sort_workspace_size": (C.c_size_t, [_U32]),
    "tpd_sort_pairs": (C.c_int, [_P, _P, _P, _P, _U32, _U32, _P, C.c_size_t, _P, C.POINTER(C.c_int)]),
    "tpd_scan_workspace_size": (C.c_size_t, [_U32]),
    "tpd_scan_tiles": (C.c_int, [_P, _U32, _P, _P, _P, C.c_size_t, _P]),
    "tpd_scan_tiles_static": (C.c_int, [_P, _U32, _P, _P, _P, _P]),
    "tpd_test_set_never_publish": (None, [_U32]),
    "tpd_look_at": (None, [_F, _F, _F, _F]),
    "tpd_perspective": (None, [_U32, _U32, C.c_float, C.c_float, C.c_float, _F]),
    "tpd_mat4_mul": (None, [_F, _F, _F]),
    "tpd_synthetic_scene": (None, [C.c_uint64, _U32, C.c_float, _F, _F, _F, _F, _F, _P]),
    "tpd_random_points": (None, [C.c_uint64, _U32, C.c_float, _F, C.c_float, C.c_float, C.c_float, C.c_float, _P]),
    "tpd_load_ply": (C.c_int, [C.c_char_p, _P, C.POINTER(_U32)]),
}

_lib = None


def lib_path() -> Path:
    return _LIB_PATH


def load() -> C.CDLL:
    """Loads libtpdsplat.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not _LIB_PATH.exists():
        raise RuntimeError(
            f"{_LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
            "(torpedo_gb300.build.build()); there is no CPU fallback")
    lib = C.CDLL(str(_LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class TpdError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"tpdsplat error {code} ({status_string(code)}): {msg}")
        self.code = code


def status_string(code: int) -> str:
    return load().tpd_status_string(code).decode()


def fptr(a) -> C.POINTER(C.c_float):
    """float* of a contiguous float32 numpy array."""
    return a.ctypes.data_as(_F)
