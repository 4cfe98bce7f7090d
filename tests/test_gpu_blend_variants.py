"""The blend's launch settings change no result: the forward image is bit for
bit the same for every batch depth (64, 128, 256 list entries per round)
with one CTA per tile or persistent CTAs on the tile queue, on one view and
on five views of mixed sizes; the adjoint's gradients agree with the default
within float-atomic reordering for every adjoint batch depth (32, 64, 128)
and either launch form, and a persistent adjoint run twice on one frame gives
the same gradients (its queue starts again)."""
import numpy as np
import pytest

import torpedo_gb300 as T
from tests import gpu_helpers as H
from torpedo_gb300 import configs

pytestmark = pytest.mark.gpu


def _views():
    eyes = configs.fibonacci_sphere(5)
    sizes = [(160, 120), (128, 72), (192, 108), (100, 64), (64, 64)]
    return [T.Camera.orbit(tuple(float(x) for x in eyes[i]), *sizes[i]) for i in range(5)]


@pytest.mark.parametrize("views", ["one", "five"])
def test_forward_image_is_the_same_for_every_setting(cuda, views):
    recs = configs.scene("cfg3", 30_000).records
    cams = [T.Camera.orbit((0.0, 0.0, -5.0), 256, 256)] if views == "one" else _views()
    eng, _ = H.render(recs, cams)
    ref = [im.copy() for im in eng.read_image()]
    eng.close()
    for rnd in (64, 128, 256):
        for persistent in (False, True):
            eng, _ = H.render(recs, cams, blend_round=rnd, blend_persistent=persistent)
            imgs = eng.read_image()
            eng.close()
            for a, b in zip(imgs, ref):
                np.testing.assert_array_equal(a, b, err_msg=f"round {rnd} persistent {persistent}")


def _grads(torch, params, cams, dimg, **settings):
    eng = T.GaussianEngine(**settings)
    eng.compile_params(*params)
    if len(cams) == 1:
        eng.set_camera(cams[0])
    else:
        eng.set_views(cams)
    eng.raster_frame()
    g1 = [t.cpu().numpy().astype(np.float64) for t in eng.backward(dimg)]
    g2 = [t.cpu().numpy().astype(np.float64) for t in eng.backward(dimg)]
    eng.close()
    return g1, g2


def test_adjoint_gradients_agree_for_every_setting(cuda):
    torch = cuda
    sc = configs.scene("cfg2", 20_000)
    dev = torch.device("cuda")
    params = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in
              (sc.means, sc.log_scales, sc.quats, sc.opacity_logits, sc.sh)]
    cams = _views()
    pixels = sum(c.width * c.height for c in cams)
    dimg = torch.from_numpy(np.random.default_rng(5).normal(size=pixels * 3).astype(np.float32)).to(dev)
    ref, _ = _grads(torch, params, cams, dimg)
    for rnd in (32, 64, 128):
        for persistent in (False, True):
            g1, g2 = _grads(torch, params, cams, dimg, blend_backward_round=rnd, blend_persistent=persistent)
            for a, b, c in zip(g1, g2, ref):
                scale = np.abs(c).max() + 1e-12
                assert np.abs(a - c).max() <= 1e-5 * scale, (rnd, persistent)
                assert np.abs(b - c).max() <= 1e-5 * scale, (rnd, persistent, "second backward")
