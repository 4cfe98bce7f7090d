"""Frames that keep the adjoint's inputs (per-pixel final transmittance and
last contributor) only when asked: keep_backward_state 0 (default: once a
backward has been called on the engine), 1 (always) and 2 (never). Whatever
the setting, a read of those buffers and a backward see the last rendered
frame: the engine renders it again from that frame's own view constants when
it kept nothing, so a camera set after the frame does not enter. Checked
against an engine whose frames always keep them: images and the kept buffers
bit for bit, gradients within the reordering of their float atomic sums."""
import numpy as np
import pytest

import torpedo_gb300 as T
from torpedo_gb300 import _lib as L
from torpedo_gb300 import configs

pytestmark = pytest.mark.gpu

N = 3000
W, H = 96, 80


def _engine(torch, keep, use_graph=True):
    sc = configs.scene("cfg2", N)
    dev = torch.device("cuda")
    params = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in
              (sc.means, sc.log_scales, sc.quats, sc.opacity_logits, sc.sh)]
    eng = T.GaussianEngine(keep_backward_state=keep, use_graph=use_graph)
    eng.compile_params(*params)
    return eng


def _state(eng):
    return (eng.read_buffer(L.TPD_BUF_FINAL_T, np.float32, eng.pixels).view(np.uint32),
            eng.read_buffer(L.TPD_BUF_N_CONTRIB, np.uint32, eng.pixels))


def _grads(torch, eng, dimg):
    return [t.cpu().numpy() for t in eng.backward(torch.from_numpy(dimg).cuda().reshape(-1))]


def _same_gradient(g, g_ref):
    """Equal up to the order of the adjoint's float atomic additions."""
    for a, b in zip(g, g_ref):
        np.testing.assert_allclose(a, b, rtol=1e-5, atol=1e-6 * float(np.abs(b).max(initial=0.0)))


@pytest.mark.parametrize("keep", [0, 2])
@pytest.mark.parametrize("use_graph", [True, False])
def test_state_and_backward_match_frames_that_keep_it(cuda, keep, use_graph):
    torch = cuda
    cam_a = T.Camera.orbit((0.0, 0.0, -5.0), W, H)
    cam_b = T.Camera.orbit((1.5, -0.5, -4.5), W, H)
    dimg = np.random.default_rng(4).normal(size=(H, W, 3)).astype(np.float32)

    ref = _engine(torch, 1, use_graph)
    ref.set_camera(cam_a)
    ref.raster_frame()
    ref.raster_frame()  # (a graph replay when graphs are on)
    st_ref = _state(ref)
    img_ref = ref.read_image()[0]
    g_ref = _grads(torch, ref, dimg)

    eng = _engine(torch, keep, use_graph)
    eng.set_camera(cam_a)
    eng.raster_frame()
    eng.raster_frame()
    np.testing.assert_array_equal(eng.read_image()[0].view(np.uint32), img_ref.view(np.uint32))
    eng.set_camera(cam_b)  # set but not rendered: the last frame is still cam_a's
    st = _state(eng)
    for a, b in zip(st, st_ref):
        np.testing.assert_array_equal(a, b)
    _same_gradient(_grads(torch, eng, dimg), g_ref)

    # later frames: keep 0 now keeps the state (a backward was called), keep 2 never does;
    # either way the next backward is the gradient of the frame just rendered
    eng.set_camera(cam_a)
    eng.raster_frame()
    _same_gradient(_grads(torch, eng, dimg), g_ref)


def test_step_async_keeps_state(cuda):
    """A training step's frame keeps the adjoint's inputs whatever the setting."""
    torch = cuda
    cam = T.Camera.orbit((0.0, 0.0, -5.0), W, H)
    dimg = torch.from_numpy(np.random.default_rng(5).normal(size=(H, W, 3)).astype(np.float32)).cuda().reshape(-1)
    ref = _engine(torch, 1)
    ref.set_camera(cam)
    ref.raster_frame()
    st_ref = _state(ref)
    eng = _engine(torch, 2)
    eng.set_camera(cam)
    eng.raster_frame()
    grads = (torch.empty((N, 3), device="cuda"), torch.empty((N, 3), device="cuda"), torch.empty((N, 4), device="cuda"),
             torch.empty((N,), device="cuda"), torch.empty((N, 48), device="cuda"))
    eng.step_async(dimg, grads, 1)
    eng.sync()
    for a, b in zip(_state(eng), st_ref):
        np.testing.assert_array_equal(a, b)
