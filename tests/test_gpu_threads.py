"""Engines are independent of each other: two engines created and driven
from two host threads at once on the same device (each thread's first frame
racing through the once-per-device kernel set-up) render the same frames as
one engine on one thread, bit for bit, and a training step's stage timing
splits the step into its forward and backward stages."""
import threading

import numpy as np
import pytest

import torpedo_gb300 as T
from torpedo_gb300 import configs

pytestmark = pytest.mark.gpu


def _render(recs, cam, frames, out, slot, barrier):
    try:
        eng = T.GaussianEngine()
        eng.compile(recs)
        eng.set_camera(cam)
        barrier.wait()
        imgs = []
        for _ in range(frames):
            eng.raster_frame()
            imgs.append(eng.read_image()[0].copy())
        eng.close()
        out[slot] = imgs
    except Exception as exc:  # reported by the main thread
        out[slot] = exc


def test_two_engines_two_threads_same_device(cuda):
    recs = configs.scene("cfg0").records
    cams = [T.Camera.orbit((0.0, 0.0, -5.0), 256, 256), T.Camera.orbit((3.0, 0.0, -4.0), 320, 200)]
    out = [None, None]
    barrier = threading.Barrier(2)
    threads = [threading.Thread(target=_render, args=(recs, cams[i], 4, out, i, barrier)) for i in range(2)]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=300)
    for i in range(2):
        assert not isinstance(out[i], Exception), out[i]
        assert out[i] is not None
        eng = T.GaussianEngine()
        eng.compile(recs)
        eng.set_camera(cams[i])
        eng.raster_frame()
        ref = eng.read_image()[0]
        eng.close()
        for img in out[i]:
            np.testing.assert_array_equal(img, ref)


def test_step_stage_times_cover_the_backward(cuda):
    torch = cuda
    sc = configs.scene("cfg2", 20_000)
    dev = torch.device("cuda")
    params = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in
              (sc.means, sc.log_scales, sc.quats, sc.opacity_logits, sc.sh)]
    cam = T.Camera.orbit((0.0, 0.0, -5.0), 256, 256)
    eng = T.GaussianEngine(stage_timing=True)
    eng.compile_params(*params)
    eng.set_camera(cam)
    eng.raster_frame()
    dimg = torch.randn(256 * 256 * 3, device=dev)
    grads = [torch.empty_like(p) for p in params]
    eng.stage_times(reset=True)
    eng.step_async(dimg, grads, 3)
    eng.sync()
    ms, frames = eng.stage_times()
    eng.close()
    assert frames == 3
    for k in ("preprocess", "depth_sort", "keygen", "key_sort", "blend", "backward_setup", "blend_backward",
              "preprocess_backward"):
        assert ms[k] > 0.0, (k, ms)
