"""Failure detection without a GPU fault: bounded device waits end with an error
status the host reads, capacity overflow grows the key buffers and re-runs the
frame, and degenerate inputs render cleanly. Nothing here traps or hangs the
GPU: the look-back test makes partition 0 of the tile scan skip its
publication (a flag that nothing sets), so successors spin until their
iteration limit, record the timeout and finish."""
import numpy as np
import pytest

import torpedo_gb300 as T
from tests import gpu_helpers as H
from torpedo_gb300 import configs
from torpedo_gb300 import _lib as L

pytestmark = pytest.mark.gpu


def test_lookback_spin_limit_reports_timeout_and_context_survives(cuda):
    recs = configs.scene("cfg0").records
    cam = configs.cameras("cfg0")[0]
    eng = T.GaussianEngine(test_never_publish=True, spin_limit=2000, use_graph=False)
    eng.compile(recs)
    eng.set_camera(cam)
    with pytest.raises(T.TpdError) as ei:
        eng.raster_frame()
    assert ei.value.code == L.TPD_ERR_TIMEOUT
    eng.close()
    # the context is still usable: a normal frame renders and matches the oracle
    eng2, stats = H.render(recs, [cam])
    g = H.gpu_state(eng2, stats)
    eng2.close()
    o = H.oracle_frame(recs, cam, f64=False)
    np.testing.assert_array_equal(g["keys"], o["keys"])


def test_key_capacity_overflow_grows_and_reruns(cuda):
    recs = configs.scene("cfg0").records
    cam = configs.cameras("cfg0")[0]
    eng = T.GaussianEngine(initial_key_capacity=1000)
    eng.compile(recs)
    eng.set_camera(cam)
    stats = eng.raster_frame()
    assert stats["retries"] >= 1 and stats["key_capacity"] >= stats["keys"]
    g = H.gpu_state(eng, stats)
    eng.close()
    o = H.oracle_frame(recs, cam, f64=False)
    np.testing.assert_array_equal(g["keys"], o["keys"])
    np.testing.assert_array_equal(g["vals"], o["vals"])


def test_empty_scene_renders_black(cuda):
    cam = configs.cameras("cfg0")[0]
    eng = T.GaussianEngine()
    eng.compile(np.zeros((0, 60), np.float32))
    eng.set_camera(cam)
    stats = eng.raster_frame()
    assert stats["keys"] == 0
    assert np.all(eng.read_image()[0] == 0)
    eng.close()


def test_all_culled_and_degenerate_inputs(cuda):
    cam = configs.cameras("cfg0")[0]
    recs = configs.scene("cfg0", 64).records.copy()
    recs[:, 2] = -10.0          # all behind the camera
    recs[0, 0:3] = np.nan       # NaN mean
    recs[1, 8:11] = 0.0         # zero scale: det = 0.3^2, still finite
    recs[2, 4:8] = 0.0          # zero quaternion
    eng, stats = H.render(recs, [cam])
    assert stats["keys"] == 0
    assert np.all(eng.read_image()[0] == 0)
    eng.close()


def test_calls_out_of_order_are_rejected(cuda):
    eng = T.GaussianEngine()
    with pytest.raises(T.TpdError) as ei:
        eng.raster_frame()
    assert ei.value.code == L.TPD_ERR_STATE
    with pytest.raises(T.TpdError):
        eng.compile(np.zeros((4, 60), np.float32), entity_index=[0, 1, 2, 9], n_entities=3)
    eng.close()
