"""The bench workload at full size (1,000,000 Gaussians, 1920x1080): keys,
values and ranges bit-exact against the oracle's keygen + std::stable_sort,
size-independent properties (sortedness, permutation, partition of the key
array by the ranges, sum of tile counts = K), and the image against the FP64
oracle on a band of tile rows."""
import numpy as np
import pytest

from oracle import oracle as O
from tests import gpu_helpers as H
from tests import tolerances as tol
from torpedo_gb300 import configs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def full(cuda):
    recs = configs.scene("cfg1").records
    cam = configs.cameras("cfg1")[0]
    eng, stats = H.render(recs, [cam])
    g = H.gpu_state(eng, stats)
    eng.close()
    o = H.oracle_frame(recs, cam, f64=False)
    return recs, cam, stats, g, o


def test_fullsize_keys_values_ranges_bit_exact(full):
    recs, cam, stats, g, o = full
    assert stats["keys"] == o["K"] and stats["keys"] > 5_000_000
    np.testing.assert_array_equal(g["splats"], o["s32"])
    np.testing.assert_array_equal(g["keys"], o["keys"])
    np.testing.assert_array_equal(g["vals"], o["vals"])
    np.testing.assert_array_equal(g["ranges"], o["ranges"])


def test_fullsize_properties(full):
    recs, cam, stats, g, o = full
    k = g["keys"]
    assert np.all(k[1:] >= k[:-1])
    # values are a permutation of the unsorted values
    assert np.array_equal(np.sort(g["vals"]), np.sort(o["vals_unsorted"]))
    r = g["ranges"]
    ne = r[:, 1] > r[:, 0]
    assert int((r[ne, 1] - r[ne, 0]).sum()) == stats["keys"]
    assert int(g["splats"][:, 3].astype(np.uint64).sum()) == stats["keys"]
    assert np.all(r[~ne] == 0)


def test_fullsize_image_band_vs_fp64(full):
    recs, cam, stats, g, o = full
    oc = H.ocam(cam)
    s64, _, _ = O.preprocess_f64(recs, oc)
    rows = 6  # tile rows 0..5 (96 pixel rows)
    img64, _, _, frag = O.blend_f64(s64, o["vals"], o["ranges"], cam.width, rows * 16)
    img = g["images"][0][: rows * 16]
    err = np.abs(img.astype(np.float64) - img64).max(axis=2)
    assert err[~frag].max(initial=0.0) <= tol.IMAGE_ABS
