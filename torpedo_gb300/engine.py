"""Python mirror of the reference's GaussianEngine over the C ABI.

Reference interface (paths relative to the reference project root):
  GaussianEngine::compile / rasterFrame / draw / getTransformHost
      torpedo/volumetric/include/torpedo/volumetric/GaussianEngine.h:23-27
  TransformHost::transform        torpedo/rendering/src/TransformHost.cpp:3-12
  Camera::lookAt                  torpedo/rendering/src/Camera.cpp:3-16
  PerspectiveCamera projection    torpedo/extension/src/PerspectiveCamera.cpp:9-23
  GaussianPoint::random/fromModel torpedo/volumetric/src/GaussianGeometry.cpp:8-127

Names follow the reference (compile, raster_frame, transform host); errors
raise TpdError like the reference's exceptions.
"""
from __future__ import annotations

import ctypes as C
from collections import deque
from dataclasses import dataclass

import numpy as np

from . import _lib as L


def _check(code: int, handle=None):
    if code != L.TPD_OK:
        msg = L.load().tpd_last_error(handle).decode() if handle else ""
        raise L.TpdError(code, msg)


def _f32(a, shape=None) -> np.ndarray:
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float32))
    if shape is not None:
        a = a.reshape(shape)
    return a


# ---------------------------------------------------------------- cameras

def look_at(eye, center, up) -> np.ndarray:
    """Camera::lookAt: row-major world->view matrix (y down)."""
    out = np.zeros(16, np.float32)
    L.load().tpd_look_at(L.fptr(_f32(eye, 3)), L.fptr(_f32(center, 3)), L.fptr(_f32(up, 3)), L.fptr(out))
    return out.reshape(4, 4)


def perspective(width: int, height: int, fov_y_degrees: float = 0.0, near: float = 0.01, far: float = 100.0):
    """PerspectiveCamera projection (reversed Z). fov_y_degrees <= 0: fy = sqrt(3)."""
    out = np.zeros(16, np.float32)
    L.load().tpd_perspective(width, height, float(fov_y_degrees), float(near), float(far), L.fptr(out))
    return out.reshape(4, 4)


def mat4_mul(a, b) -> np.ndarray:
    """math::mul with the reference's compensated dot product."""
    out = np.zeros(16, np.float32)
    L.load().tpd_mat4_mul(L.fptr(_f32(a, 16)), L.fptr(_f32(b, 16)), L.fptr(out))
    return out.reshape(4, 4)


def key_bits_for_tiles(tiles: int) -> int:
    return int(L.load().tpd_key_bits_for_tiles(tiles))


@dataclass
class Camera:
    view: np.ndarray   # 4x4 row-major
    proj: np.ndarray   # 4x4 row-major
    width: int
    height: int

    @staticmethod
    def orbit(eye, width: int, height: int, center=(0.0, 0.0, 0.0), up=(0.0, -1.0, 0.0), fov_y_degrees: float = 60.0,
              near: float = 0.2, far: float = 100.0) -> "Camera":
        return Camera(look_at(eye, center, up), perspective(width, height, fov_y_degrees, near, far), width, height)

    def projview(self) -> np.ndarray:
        return mat4_mul(self.proj, self.view)


# ---------------------------------------------------------------- scenes

@dataclass
class Scene:
    records: np.ndarray      # (n, 60) float32, the 240-byte GaussianPoint records
    means: np.ndarray | None = None
    log_scales: np.ndarray | None = None
    quats: np.ndarray | None = None
    opacity_logits: np.ndarray | None = None
    sh: np.ndarray | None = None

    @property
    def n(self) -> int:
        return int(self.records.shape[0])


def synthetic_scene(seed: int, n: int, mean_box: float = 0.0) -> Scene:
    """Seeded scene: means ~ N(0,1)^3 (mean_box <= 0) or U[-b, b]^3, log-scales ~ N(-4, .5),
    unit quaternions, opacity = sigmoid(N(0,1)), SH ~ N(0, .2)."""
    m = np.zeros((n, 3), np.float32)
    ls = np.zeros((n, 3), np.float32)
    q = np.zeros((n, 4), np.float32)
    lo = np.zeros(n, np.float32)
    sh = np.zeros((n, 48), np.float32)
    rec = np.zeros((n, 60), np.float32)
    L.load().tpd_synthetic_scene(seed, n, float(mean_box), L.fptr(m), L.fptr(ls), L.fptr(q), L.fptr(lo), L.fptr(sh),
                                 rec.ctypes.data)
    return Scene(rec, m, ls, q, lo, sh)


def random_points(seed: int, n: int, radius: float = 1.0, center=(0.0, 0.0, 0.0), min_scale: float = 0.1,
                  max_scale: float = 1.0, min_opacity: float = 0.1, max_opacity: float = 1.0) -> np.ndarray:
    """GaussianPoint::random, seeded."""
    rec = np.zeros((n, 60), np.float32)
    L.load().tpd_random_points(seed, n, radius, L.fptr(_f32(center, 3)), min_scale, max_scale, min_opacity,
                               max_opacity, rec.ctypes.data)
    return rec


def load_ply(path: str) -> np.ndarray:
    """GaussianPoint::fromModel: 3DGS PLY -> (n, 60) records."""
    lib = L.load()
    n = C.c_uint32(0)
    _check(lib.tpd_load_ply(str(path).encode(), None, C.byref(n)))
    rec = np.empty((n.value, 60), np.float32)  # every record is written in full
    _check(lib.tpd_load_ply(str(path).encode(), rec.ctypes.data, C.byref(n)))
    return rec


# ---------------------------------------------------------------- engine

class TransformHost:
    """Per-entity model matrices (TransformHost::transform)."""

    def __init__(self, engine: "GaussianEngine"):
        self._engine = engine

    def transform(self, entity: int, model) -> None:
        e = self._engine
        _check(L.load().tpd_set_transform(e._h, entity, L.fptr(_f32(model, 16))), e._h)


class GaussianEngine:
    """tpd::GaussianEngine over libtpdsplat.

    compile(records) uploads the point cloud, set_camera / set_views choose the
    view(s), raster_frame() renders synchronously, read_image() returns the
    image(s) (the draw() step without a swapchain).
    """

    def __init__(self, sh_degree: int = 3, band3_compat: bool = True, device: int = 0, stream: int | None = None,
                 use_graph: bool = True, spin_limit: int = 0, initial_key_capacity: int = 0, timeout_s: float = 60.0,
                 test_never_publish: bool = False, stage_timing: bool = False, sort_ctas_per_sm: int = 0,
                 depth_sort_items: int = 0, sort_threads: int = 0, depth_sort_threads: int = 0, blend_round: int = 0,
                 blend_backward_round: int = 0, blend_persistent: bool = False, key_sort_lookback: bool = False,
                 keep_backward_state: int = 0):
        lib = L.load()
        s = L.Settings()
        lib.tpd_settings_init(C.byref(s))
        s.sh_degree = sh_degree
        s.band3_compat = 1 if band3_compat else 0
        s.device = device
        s.stream = stream
        s.use_graph = 1 if use_graph else 0
        s.spin_limit = spin_limit
        s.initial_key_capacity = initial_key_capacity
        s.timeout_s = timeout_s
        s.test_never_publish = 1 if test_never_publish else 0
        s.stage_timing = 1 if stage_timing else 0
        s.sort_ctas_per_sm = sort_ctas_per_sm
        s.depth_sort_items = depth_sort_items
        s.sort_threads = sort_threads
        s.depth_sort_threads = depth_sort_threads
        s.blend_round = blend_round
        s.blend_backward_round = blend_backward_round
        s.blend_persistent = 1 if blend_persistent else 0
        s.key_sort_lookback = 1 if key_sort_lookback else 0
        s.keep_backward_state = keep_backward_state
        h = C.c_void_p()
        _check(lib.tpd_create(C.byref(s), C.byref(h)))
        self._h = h
        self.device = device
        self._views: list[Camera] = []
        self._render_dst: deque = deque()  # destinations of outstanding renders, kept alive until waited for
        self.n = 0
        self.transform_host = TransformHost(self)

    # reference name
    def get_transform_host(self) -> TransformHost:
        return self.transform_host

    def close(self):
        if getattr(self, "_h", None):
            L.load().tpd_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def compile(self, records, entity_index=None, n_entities: int = 1) -> None:
        rec = _f32(records)
        if rec.ndim != 2 or rec.shape[1] != 60:
            raise ValueError("records must be (n, 60) float32")
        ent = None
        if entity_index is not None:
            ent = np.ascontiguousarray(np.asarray(entity_index, dtype=np.uint32))
        _check(L.load().tpd_compile(self._h, rec.ctypes.data, rec.shape[0], ent.ctypes.data if ent is not None else None,
                                    n_entities), self._h)
        self.n = rec.shape[0]

    def compile_params(self, means, log_scales, quats, opacity_logits, sh) -> None:
        """Raw parameters as contiguous float32 CUDA tensors on this engine's device."""
        import torch

        for t in (means, log_scales, quats, opacity_logits, sh):
            if not (t.is_cuda and t.dtype == torch.float32 and t.is_contiguous()):
                raise ValueError("parameters must be contiguous float32 CUDA tensors")
        n = means.shape[0]
        _check(L.load().tpd_compile_params_device(self._h, means.data_ptr(), log_scales.data_ptr(), quats.data_ptr(),
                                                  opacity_logits.data_ptr(), sh.data_ptr(), n), self._h)
        self.n = n

    def set_camera(self, cam: Camera) -> None:
        _check(L.load().tpd_set_camera(self._h, L.fptr(_f32(cam.view, 16)), L.fptr(_f32(cam.proj, 16)), cam.width,
                                       cam.height), self._h)
        self._views = [cam]

    def set_views(self, cams: list[Camera]) -> None:
        arr = (L.View * len(cams))()
        for i, c in enumerate(cams):
            arr[i].view[:] = list(_f32(c.view, 16))
            arr[i].proj[:] = list(_f32(c.proj, 16))
            arr[i].width = c.width
            arr[i].height = c.height
        _check(L.load().tpd_set_views(self._h, arr, len(cams)), self._h)
        self._views = list(cams)

    def raster_frame(self) -> dict:
        st = L.FrameStats()
        _check(L.load().tpd_raster_frame(self._h, C.byref(st)), self._h)
        return st.as_dict()

    def raster_frames_async(self, count: int) -> None:
        """Enqueues count frames back to back (no host wait); sync() waits."""
        _check(L.load().tpd_raster_frames_async(self._h, count), self._h)

    def sync(self) -> dict:
        st = L.FrameStats()
        _check(L.load().tpd_sync(self._h, C.byref(st)), self._h)
        return st.as_dict()

    def stage_times(self, reset: bool = False) -> tuple[dict, int]:
        """Accumulated per-stage GPU ms (engine created with stage_timing=True) and the frame count."""
        ms = (C.c_double * len(L.STAGES))()
        fr = C.c_uint64()
        _check(L.load().tpd_stage_times(self._h, ms, C.byref(fr), 1 if reset else 0), self._h)
        return {k: ms[i] for i, k in enumerate(L.STAGES)}, int(fr.value)

    @property
    def pixels(self) -> int:
        return sum(c.width * c.height for c in self._views)

    def read_image(self, rgba8: bool = False):
        """Host copy of the image(s): list of (H, W, 3) float32 or (H, W, 4) uint8, one per view."""
        n = self.pixels
        flat = np.zeros(n * 4, np.uint8) if rgba8 else np.zeros(n * 3, np.float32)
        _check(L.load().tpd_read_image(self._h, flat.ctypes.data, L.TPD_IMAGE_RGBA8 if rgba8 else L.TPD_IMAGE_RGB32F, 0),
               self._h)
        out, off = [], 0
        for c in self._views:
            k = c.width * c.height
            if rgba8:
                out.append(flat[off * 4:(off + k) * 4].reshape(c.height, c.width, 4))
            else:
                out.append(flat[off * 3:(off + k) * 3].reshape(c.height, c.width, 3))
            off += k
        return out

    def read_image_device(self, out) -> None:
        """Copies the packed RGB float image(s) into a contiguous float32 CUDA tensor of pixels*3 elements."""
        import torch

        if not (out.is_cuda and out.is_contiguous() and out.dtype == torch.float32
                and out.numel() == self.pixels * 3):
            raise ValueError("out must be a contiguous float32 CUDA tensor of pixels * 3 elements")
        _check(L.load().tpd_read_image(self._h, out.data_ptr(), L.TPD_IMAGE_RGB32F, 1), self._h)

    def buffer(self, which: int) -> tuple[int, int]:
        p = C.c_void_p()
        b = C.c_uint64()
        _check(L.load().tpd_get_buffer(self._h, which, C.byref(p), C.byref(b)), self._h)
        return int(p.value or 0), int(b.value)

    def read_buffer(self, which: int, dtype, count: int | None = None, offset_elems: int = 0) -> np.ndarray:
        """Host copy of an internal buffer (TPD_BUF_*) as a numpy array of dtype."""
        dt = np.dtype(dtype)
        _, size = self.buffer(which)
        if count is None:
            count = size // dt.itemsize - offset_elems
        out = np.zeros(count, dt)
        if count:
            _check(L.load().tpd_read_buffer(self._h, which, out.ctypes.data, offset_elems * dt.itemsize,
                                            count * dt.itemsize, 0), self._h)
        return out

    def stream_handle(self) -> int:
        return int(L.load().tpd_get_stream(self._h) or 0)

    def backward(self, dL_dimage, g_means=None, g_log_scales=None, g_quats=None, g_logits=None, g_sh=None):
        """Gradients w.r.t. raw parameters (torch CUDA tensors, allocated when not given)."""
        import torch

        n = self.n
        dev = dL_dimage.device
        mk = lambda t, shape: t if t is not None else torch.empty(shape, dtype=torch.float32, device=dev)
        g_means, g_log_scales, g_quats = mk(g_means, (n, 3)), mk(g_log_scales, (n, 3)), mk(g_quats, (n, 4))
        g_logits, g_sh = mk(g_logits, (n,)), mk(g_sh, (n, 48))
        dimg = dL_dimage.contiguous()
        torch.cuda.current_stream(dev).synchronize()
        _check(L.load().tpd_backward(self._h, dimg.data_ptr(), g_means.data_ptr(), g_log_scales.data_ptr(),
                                     g_quats.data_ptr(), g_logits.data_ptr(), g_sh.data_ptr()), self._h)
        return g_means, g_log_scales, g_quats, g_logits, g_sh

    def render_async(self, dst, rgba8: bool = True) -> None:
        """Renders the current view(s) and copies the image into dst (a pinned
        host or CUDA tensor of pixels * 4 bytes for RGBA8, pixels * 3 floats
        otherwise) without waiting; wait_render() waits for the oldest of at
        most two outstanding renders and returns its stats."""
        fmt = L.TPD_IMAGE_RGBA8 if rgba8 else L.TPD_IMAGE_RGB32F
        on_device = 1 if getattr(dst, "is_cuda", False) else 0
        _check(L.load().tpd_render_async(self._h, dst.data_ptr(), fmt, on_device), self._h)
        self._render_dst.append(dst)  # the copy into dst lands before the matching wait_render returns

    def wait_render(self) -> dict:
        st = L.FrameStats()
        _check(L.load().tpd_wait_render(self._h, C.byref(st)), self._h)
        if self._render_dst:
            self._render_dst.popleft()
        return st.as_dict()

    def step_async(self, dL_dimage, grads, count: int = 1):
        """count training steps (forward frame + backward) enqueued on the engine's
        stream without host waits; grads = (g_means, g_log_scales, g_quats,
        g_logits, g_sh) CUDA tensors, overwritten each step. Call sync() to wait."""
        import torch

        dimg = dL_dimage.contiguous()
        ptrs = [g.data_ptr() for g in grads]
        torch.cuda.current_stream(dimg.device).synchronize()  # inputs written on torch's stream
        _check(L.load().tpd_step_async(self._h, dimg.data_ptr(), *ptrs, count), self._h)
        self._step_refs = (dimg, tuple(grads))  # kept alive while the steps run


def sort_pairs(keys, vals, key_bits: int):
    """Stable radix sort of CUDA tensors keys (int64 holding u64) / vals (int32 holding u32) on the low key_bits."""
    import torch

    n = keys.numel()
    lib = L.load()
    ws = torch.empty(int(lib.tpd_sort_workspace_size(n)), dtype=torch.uint8, device=keys.device)
    ka, va = torch.empty_like(keys), torch.empty_like(vals)
    alt = C.c_int(0)
    stream = torch.cuda.current_stream(keys.device).cuda_stream
    _check(lib.tpd_sort_pairs(keys.data_ptr(), vals.data_ptr(), ka.data_ptr(), va.data_ptr(), n, key_bits,
                              ws.data_ptr(), ws.numel(), stream, C.byref(alt)))
    _check_workspace_status(ws, n)
    return (ka, va) if alt.value else (keys, vals)


def _check_workspace_status(ws, n: int) -> None:
    """Raises TpdError when the device status word a stage call left in its
    workspace is not 0 (waits for the stream)."""
    import torch

    if n == 0:
        return
    st = int(ws[L.WORKSPACE_STATUS_OFFSET:L.WORKSPACE_STATUS_OFFSET + 4].view(torch.int32).item())
    if st:
        raise L.TpdError(L.TPD_ERR_TIMEOUT if st & L.DEVSTAT_LOOKBACK_TIMEOUT else L.TPD_ERR_DEVICE,
                         f"device status 0x{st & 0xFFFFFFFF:x}: the result is invalid")


def scan_tiles(splats_u32):
    """Exclusive scan of the tiles word of (n, 12) int32 CUDA splats -> (offsets, total)."""
    import torch

    n = splats_u32.shape[0]
    lib = L.load()
    ws = torch.empty(int(lib.tpd_scan_workspace_size(n)), dtype=torch.uint8, device=splats_u32.device)
    offs = torch.empty(n, dtype=torch.int32, device=splats_u32.device)
    tot = torch.zeros(1, dtype=torch.int32, device=splats_u32.device)
    stream = torch.cuda.current_stream(splats_u32.device).cuda_stream
    _check(lib.tpd_scan_tiles(splats_u32.data_ptr(), n, offs.data_ptr(), tot.data_ptr(), ws.data_ptr(), ws.numel(),
                              stream))
    _check_workspace_status(ws, n)
    return offs, tot
