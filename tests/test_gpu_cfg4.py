"""cfg4 at full size: 6,000,000 Gaussians (means U[-10,10]^3), 8 views of
3840x2160 on a sphere of radius 5 (the cameras sit inside the cloud, so some
Gaussians cover more than 10,000 tiles), about 166M keys in one batched frame.

Checked: every view's segment of the batched key array, its values and its
tile ranges bit-exact against the oracle's keygen + std::stable_sort of that
view (tile ids offset by the view's tile base); view 0's image bit-identical to
a single-view frame; one forward + backward step with finite gradients."""
import numpy as np
import pytest

import torpedo_gb300 as T
from oracle import oracle as O
from tests import gpu_helpers as H
from torpedo_gb300 import configs
from torpedo_gb300 import _lib as L

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cfg4(cuda):
    sc = configs.scene("cfg4")
    cams = configs.cameras("cfg4")
    eng, stats = H.render(sc.records, cams)
    yield sc, cams, eng, stats
    eng.close()


def test_cfg4_batched_lists_bit_exact_per_view(cfg4):
    sc, cams, eng, stats = cfg4
    K = stats["keys"]
    assert stats["views"] == 8 and K > 100_000_000
    keys = eng.read_buffer(L.TPD_BUF_KEYS, np.uint64, K)
    vals = eng.read_buffer(L.TPD_BUF_VALUES, np.uint32, K)
    ranges = eng.read_buffer(L.TPD_BUF_RANGES, np.uint32, stats["tiles"] * 2).reshape(-1, 2)
    pos = 0
    tile_base = 0
    for cam in cams:
        oc = H.ocam(cam)
        s32 = O.preprocess_f32(sc.records, oc)
        offs, k = O.scan_tiles(s32)
        ok, ov = O.stable_sort(*O.keygen(s32, offs, k, cam.width, cam.height))
        n_tiles = ((cam.width + 15) // 16) * ((cam.height + 15) // 16)
        orng = O.tile_ranges(ok, n_tiles).astype(np.int64)
        seg = slice(pos, pos + k)
        expect = ok + (np.uint64(tile_base) << np.uint64(32))
        np.testing.assert_array_equal(keys[seg], expect)
        np.testing.assert_array_equal(vals[seg], ov)
        got = ranges[tile_base:tile_base + n_tiles].astype(np.int64)
        nonempty = orng[:, 1] > orng[:, 0]
        np.testing.assert_array_equal(got[nonempty], orng[nonempty] + pos)
        assert np.all(got[~nonempty] == 0)
        pos += k
        tile_base += n_tiles
    assert pos == K


def test_cfg4_view0_equals_single_view_frame(cfg4):
    sc, cams, eng, stats = cfg4
    batched = eng.read_image()[0]
    e1, s1 = H.render(sc.records, [cams[0]])
    single = e1.read_image()[0]
    e1.close()
    np.testing.assert_array_equal(batched, single)
    assert np.isfinite(batched).all()


def test_cfg4_forward_backward_step(cuda):
    torch = cuda
    sc = configs.scene("cfg4")
    cams = configs.cameras("cfg4")
    dev = torch.device("cuda")
    params = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in
              (sc.means, sc.log_scales, sc.quats, sc.opacity_logits, sc.sh)]
    eng = T.GaussianEngine()
    eng.compile_params(*params)
    eng.set_views(cams)
    st = eng.raster_frame()
    pixels = sum(c.width * c.height for c in cams)
    dimg = torch.randn(pixels * 3, device=dev, generator=torch.Generator(device=dev).manual_seed(4))
    grads = [torch.full_like(p, float("nan")) for p in params]
    eng.step_async(dimg, grads, 1)
    eng.sync()
    eng.close()
    assert st["keys"] > 100_000_000
    for g in grads:
        assert torch.isfinite(g).all()
    assert float(grads[0].abs().sum()) > 0
