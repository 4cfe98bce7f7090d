"""The hand-written backward against the FP64 oracle's analytic gradient (itself
checked against central finite differences in test_oracle.py), through the C
ABI and through the torch.autograd.Function wrapper.

Bar: relative error <= 1e-3 (tests/tolerances.py), measured per parameter
group as ||g_gpu - g_64|| / ||g_64|| and per element against a floor of 1e-3
of the group's largest gradient."""
import numpy as np
import pytest

import torpedo_gb300 as T
from oracle import oracle as O
from tests import gpu_helpers as H
from tests import tolerances as tol
from torpedo_gb300 import configs
from torpedo_gb300 import _lib as L

pytestmark = pytest.mark.gpu

NAMES = ["means", "log_scales", "quats", "opacity_logits", "sh"]


def _setup(cuda, n, w, h, seed=2, compat=True, eye=(0.0, 0.0, -5.0)):
    torch = cuda
    sc = configs.scene("cfg2", n)
    cam = T.Camera.orbit(eye, w, h)
    dev = torch.device("cuda")
    params = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in
              (sc.means, sc.log_scales, sc.quats, sc.opacity_logits, sc.sh)]
    dimg = np.random.default_rng(seed).normal(size=(h, w, 3)).astype(np.float32)
    return sc, cam, params, dimg


def _compare(g_gpu, g64, vis):
    for name, a, b in zip(NAMES, g_gpu, g64):
        a = np.asarray(a, np.float64).reshape(len(a), -1)[vis]
        b = np.asarray(b, np.float64).reshape(len(b), -1)[vis]
        nb = np.linalg.norm(b)
        if nb == 0:
            assert np.abs(a).max(initial=0) == 0
            continue
        rel = np.linalg.norm(a - b) / nb
        assert rel <= tol.GRAD_REL, (name, rel)
        floor = 1e-3 * np.abs(b).max()
        el = np.abs(a - b) / (np.abs(b) + floor)
        assert np.quantile(el, 0.999) <= 10 * tol.GRAD_REL, (name, np.quantile(el, 0.999))


@pytest.mark.parametrize("compat", [True, False])
def test_backward_vs_fp64_oracle(cuda, compat):
    torch = cuda
    sc, cam, params, dimg = _setup(cuda, 2000, 64, 64, compat=compat)
    eng = T.GaussianEngine(band3_compat=compat)
    eng.compile_params(*params)
    eng.set_camera(cam)
    stats = eng.raster_frame()
    g = [t.cpu().numpy() for t in eng.backward(torch.from_numpy(dimg).cuda().reshape(-1))]
    vals = eng.read_buffer(L.TPD_BUF_VALUES, np.uint32, stats["keys"])
    rng = eng.read_buffer(L.TPD_BUF_RANGES, np.uint32, stats["tiles"] * 2).reshape(-1, 2)
    splats = eng.read_buffer(L.TPD_BUF_SPLATS, np.uint32, sc.n * 12).reshape(sc.n, 12)
    eng.close()
    p64 = [a.astype(np.float64) for a in (sc.means, sc.log_scales, sc.quats, sc.opacity_logits, sc.sh)]
    g64, _ = O.backward_f64(p64, H.ocam(cam), vals, rng, dimg.astype(np.float64), band3_compat=compat)
    vis = splats[:, 7] != 0
    assert vis.sum() > 100
    _compare(g, g64, vis)


def test_backward_800x800_subscene(cuda):
    """A larger frame at the cfg2 image size (800x800)."""
    torch = cuda
    sc, cam, params, dimg = _setup(cuda, 20_000, 800, 800, seed=3)
    eng = T.GaussianEngine()
    eng.compile_params(*params)
    eng.set_camera(cam)
    stats = eng.raster_frame()
    g = [t.cpu().numpy() for t in eng.backward(torch.from_numpy(dimg).cuda().reshape(-1))]
    vals = eng.read_buffer(L.TPD_BUF_VALUES, np.uint32, stats["keys"])
    rng = eng.read_buffer(L.TPD_BUF_RANGES, np.uint32, stats["tiles"] * 2).reshape(-1, 2)
    splats = eng.read_buffer(L.TPD_BUF_SPLATS, np.uint32, sc.n * 12).reshape(sc.n, 12)
    eng.close()
    p64 = [a.astype(np.float64) for a in (sc.means, sc.log_scales, sc.quats, sc.opacity_logits, sc.sh)]
    g64, _ = O.backward_f64(p64, H.ocam(cam), vals, rng, dimg.astype(np.float64))
    _compare(g, g64, splats[:, 7] != 0)


def test_autograd_function(cuda):
    torch = cuda
    from torpedo_gb300.autograd import rasterize

    sc, cam, params, dimg = _setup(cuda, 1500, 64, 64, seed=4)
    leaves = [p.clone().requires_grad_(True) for p in params]
    eng = T.GaussianEngine()
    img = rasterize(*leaves, eng, [cam])
    loss = (img * torch.from_numpy(dimg).cuda().reshape(-1)).sum()
    loss.backward()
    eng2 = T.GaussianEngine()
    eng2.compile_params(*params)
    eng2.set_camera(cam)
    eng2.raster_frame()
    direct = eng2.backward(torch.from_numpy(dimg).cuda().reshape(-1))
    for a, b in zip(leaves, direct):
        torch.testing.assert_close(a.grad, b, rtol=1e-4, atol=1e-6)
    eng.close()
    eng2.close()


@pytest.mark.parametrize("views", [1, 3])
def test_step_async_graph_matches_backward(cuda, views):
    """tpd_step_async (forward + backward captured as one graph per step) gives
    the gradients of tpd_raster_frame + tpd_backward on the same views; the
    adjoint sums with float atomics, so the bar is 1e-5 relative."""
    torch = cuda
    sc = configs.scene("cfg2", 20_000)
    eyes = configs.fibonacci_sphere(views)
    sizes = [(96, 80), (64, 64), (120, 72)]
    cams = [T.Camera.orbit(tuple(float(x) for x in eyes[v]), *sizes[v % 3]) for v in range(views)]
    dev = torch.device("cuda")
    params = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in
              (sc.means, sc.log_scales, sc.quats, sc.opacity_logits, sc.sh)]
    pixels = sum(c.width * c.height for c in cams)
    dimg = torch.from_numpy(np.random.default_rng(5).normal(size=pixels * 3).astype(np.float32)).to(dev)
    eng = T.GaussianEngine(use_graph=True)
    eng.compile_params(*params)
    if views == 1:
        eng.set_camera(cams[0])
    else:
        eng.set_views(cams)
    eng.raster_frame()
    ref = [t.cpu().numpy() for t in eng.backward(dimg)]
    grads = [torch.full_like(p, float("nan")) for p in params]
    eng.step_async(dimg, grads, count=3)
    eng.sync()
    eng.close()
    for name, a, b in zip(NAMES, [g.cpu().numpy() for g in grads], ref):
        nb = np.linalg.norm(b)
        assert np.all(np.isfinite(a)), name
        assert np.linalg.norm(a - b) <= 1e-5 * nb + 1e-12, (name, np.linalg.norm(a - b) / max(nb, 1e-30))
