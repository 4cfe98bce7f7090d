"""Every radix pass variant gives the same frame, bit for bit.

The engine settings key_sort_lookback, sort_threads, depth_sort_threads,
depth_sort_items and sort_ctas_per_sm choose the key sort's form (counted
passes at 3 or 2 CTAs per SM, or onesweep passes with a look-back) and
among five compiled onesweep kernels (512 x 8 keys with match-any ranking;
256 x 16 keys at 2 or 3 CTAs per SM, 256 x 8 and 256 x 4 keys with
bit-ballot ranking) for the depth presort and the onesweep key sort.
The default settings are checked against the oracle stage by stage in
test_gpu_pipeline.py; here each other choice must reproduce the default
frame exactly: sorted keys and values, tile ranges, image, final
transmittance and contributor counts.
"""
import numpy as np
import pytest

import torpedo_gb300 as T
from tests import gpu_helpers as H
from torpedo_gb300 import configs

pytestmark = pytest.mark.gpu

VARIANTS = [
    dict(sort_ctas_per_sm=2),
    dict(key_sort_lookback=True),
    dict(key_sort_lookback=True, sort_threads=256),
    dict(key_sort_lookback=True, sort_threads=256, sort_ctas_per_sm=3),
    dict(depth_sort_threads=512),
    dict(depth_sort_items=8),
    dict(depth_sort_items=4),
    dict(sort_threads=256, depth_sort_threads=512, depth_sort_items=8),
]


def _scenes():
    cams = configs.cameras("cfg1")
    return {
        "cfg1_200k": (configs.scene("cfg1", 200_000).records, [cams[0]]),
        "cfg0": (configs.scene("cfg0").records, [configs.cameras("cfg0")[0]]),
        "views3_60k": (configs.scene("cfg1", 60_000).records,
                       [cams[0], T.Camera.orbit((0.9, 0.3, -4.5), 640, 360), T.Camera.orbit((-1.2, 0.5, -3.8), 333, 217)]),
    }


_ref = {}


def _state(name, recs, cams, **kw):
    eng, stats = H.render(recs, cams, **kw)
    try:
        assert stats["status"] == 0
        return H.gpu_state(eng, stats)
    finally:
        eng.close()


@pytest.mark.parametrize("variant", VARIANTS, ids=lambda v: ",".join(f"{k}={x}" for k, x in v.items()))
@pytest.mark.parametrize("scene", ["cfg1_200k", "cfg0", "views3_60k"])
def test_variant_matches_default_frame(cuda, scene, variant):
    recs, cams = _scenes()[scene]
    if scene not in _ref:
        _ref[scene] = _state(scene, recs, cams)
    ref = _ref[scene]
    got = _state(scene, recs, cams, **variant)
    assert got["K"] == ref["K"]
    for key in ("keys", "vals", "ranges", "n_contrib"):
        np.testing.assert_array_equal(got[key], ref[key], err_msg=key)
    np.testing.assert_array_equal(got["final_T"].view(np.uint32), ref["final_T"].view(np.uint32))
    for a, b in zip(got["images"], ref["images"]):
        np.testing.assert_array_equal(a.view(np.uint32), b.view(np.uint32))
