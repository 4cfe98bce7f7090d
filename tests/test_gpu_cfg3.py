"""cfg3 at full size, the batched training workload: 500,000 Gaussians
(means N(0,1)^3), 64 views on a sphere of radius 5 with sizes drawn from
640x480, 1280x720 and 1920x1080, about 194M keys in one batched frame.

Checked:
- every view's segment of the batched key array, its values and its tile
  ranges bit-exact against the oracle's keygen + std::stable_sort of that view
  (the reference sorts one view per frame, GaussianEngine.cpp:621-712; tile
  ids here are offset by the view's tile base);
- the images of three views (one of each size) within 1e-3 of the FP64 oracle
  on a band of tile rows, outside pixels whose FP64 decisions lie at a
  threshold;
- the batched backward with dL/dimage on three views only equals the sum of
  those views' single-view backwards."""
import numpy as np
import pytest

import torpedo_gb300 as T
from oracle import oracle as O
from tests import gpu_helpers as H
from tests.tolerances import IMAGE_ABS
from torpedo_gb300 import configs
from torpedo_gb300 import _lib as L

pytestmark = pytest.mark.gpu

BAND_ROWS = 4  # tile rows of each checked image compared with FP64


@pytest.fixture(scope="module")
def cfg3(cuda):
    sc = configs.scene("cfg3")
    cams = configs.cameras("cfg3")
    eng, stats = H.render(sc.records, cams)
    yield sc, cams, eng, stats
    eng.close()


def _checked_views(cams):
    """The first view of each image size."""
    seen, out = set(), []
    for v, c in enumerate(cams):
        if (c.width, c.height) not in seen:
            seen.add((c.width, c.height))
            out.append(v)
    return out


def test_cfg3_batched_lists_bit_exact_per_view(cfg3):
    sc, cams, eng, stats = cfg3
    K = stats["keys"]
    assert stats["views"] == 64 and K > 100_000_000
    keys = eng.read_buffer(L.TPD_BUF_KEYS, np.uint64, K)
    vals = eng.read_buffer(L.TPD_BUF_VALUES, np.uint32, K)
    ranges = eng.read_buffer(L.TPD_BUF_RANGES, np.uint32, stats["tiles"] * 2).reshape(-1, 2)
    pos = 0
    tile_base = 0
    for v, cam in enumerate(cams):
        oc = H.ocam(cam)
        s32 = O.preprocess_f32(sc.records, oc)
        offs, k = O.scan_tiles(s32)
        ok, ov = O.stable_sort(*O.keygen(s32, offs, k, cam.width, cam.height))
        n_tiles = ((cam.width + 15) // 16) * ((cam.height + 15) // 16)
        orng = O.tile_ranges(ok, n_tiles).astype(np.int64)
        seg = slice(pos, pos + k)
        np.testing.assert_array_equal(keys[seg], ok + (np.uint64(tile_base) << np.uint64(32)), err_msg=f"view {v}")
        np.testing.assert_array_equal(vals[seg], ov, err_msg=f"view {v}")
        got = ranges[tile_base:tile_base + n_tiles].astype(np.int64)
        nonempty = orng[:, 1] > orng[:, 0]
        np.testing.assert_array_equal(got[nonempty], orng[nonempty] + pos, err_msg=f"view {v}")
        assert np.all(got[~nonempty] == 0)
        pos += k
        tile_base += n_tiles
    assert pos == K


def test_cfg3_images_vs_fp64_on_a_band(cfg3):
    sc, cams, eng, stats = cfg3
    imgs = eng.read_image()
    for v in _checked_views(cams):
        cam = cams[v]
        oc = H.ocam(cam)
        s32 = O.preprocess_f32(sc.records, oc)
        offs, k = O.scan_tiles(s32)
        ok, ov = O.stable_sort(*O.keygen(s32, offs, k, cam.width, cam.height))
        gx = (cam.width + 15) // 16
        rng = O.tile_ranges(ok, gx * ((cam.height + 15) // 16))
        # a band of tile rows through the middle of the view; other tiles are left empty
        r0 = ((cam.height + 15) // 16) // 2 - BAND_ROWS // 2
        band = np.zeros_like(rng)
        band[r0 * gx:(r0 + BAND_ROWS) * gx] = rng[r0 * gx:(r0 + BAND_ROWS) * gx]
        s64, _, _ = O.preprocess_f64(sc.records, oc)
        img64, _, _, pfrag = O.blend_f64(s64, ov, band, cam.width, cam.height)
        rows = slice(r0 * 16, min(cam.height, (r0 + BAND_ROWS) * 16))
        err = np.abs(imgs[v][rows].astype(np.float64) - img64[rows]).max(axis=2)[~pfrag[rows]]
        assert err.max() <= IMAGE_ABS, (v, err.max())
        assert float(imgs[v][rows].sum()) > 0


def test_cfg3_batched_gradient_equals_sum_of_views(cuda):
    torch = cuda
    sc = configs.scene("cfg3")
    cams = configs.cameras("cfg3")
    dev = torch.device("cuda")
    params = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in
              (sc.means, sc.log_scales, sc.quats, sc.opacity_logits, sc.sh)]
    picked = _checked_views(cams)
    gen = np.random.default_rng(3)
    dimgs = [np.zeros((c.height, c.width, 3), np.float32) for c in cams]
    for v in picked:
        dimgs[v] = gen.normal(size=dimgs[v].shape).astype(np.float32)
    eng = T.GaussianEngine()
    eng.compile_params(*params)
    eng.set_views(cams)
    eng.raster_frame()
    flat = torch.from_numpy(np.concatenate([d.reshape(-1) for d in dimgs])).to(dev)
    gb = [t.cpu().numpy().astype(np.float64) for t in eng.backward(flat)]
    eng.close()
    acc = None
    for v in picked:
        e = T.GaussianEngine()
        e.compile_params(*params)
        e.set_camera(cams[v])
        e.raster_frame()
        g = [t.cpu().numpy().astype(np.float64) for t in e.backward(torch.from_numpy(dimgs[v].reshape(-1)).to(dev))]
        e.close()
        acc = g if acc is None else [a + b for a, b in zip(acc, g)]
    for a, b in zip(gb, acc):
        scale = np.abs(b).max() + 1e-12
        assert np.abs(a - b).max() <= 1e-4 * scale
