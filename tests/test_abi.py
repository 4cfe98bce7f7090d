"""The C-ABI library loads and exports every entry point include/tpdsplat.h
declares; host-only entry points behave (no device work here)."""
import ctypes as C
import re
from pathlib import Path

import numpy as np

import torpedo_gb300 as T
from torpedo_gb300 import _lib as L

HEADER = Path(__file__).resolve().parent.parent / "include" / "tpdsplat.h"


def declared():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^TPD_API [^;]*?\b(tpd_\w+)\s*\(", text, re.M)))


def test_every_declared_symbol_is_exported():
    names = declared()
    assert len(names) >= 25
    lib = C.CDLL(str(L.lib_path()))
    for n in names:
        assert hasattr(lib, n), n


def test_binding_covers_header():
    assert set(declared()) == set(L.SIGNATURES)


def test_host_entry_points():
    lib = T.load()
    assert lib.tpd_version().startswith(b"tpdsplat")
    assert lib.tpd_status_string(0) == b"ok"
    s = L.Settings()
    lib.tpd_settings_init(C.byref(s))
    assert s.sh_degree == 3 and s.band3_compat == 1 and s.use_graph == 1
    assert lib.tpd_sort_workspace_size(1 << 20) > lib.tpd_sort_workspace_size(1)
    assert lib.tpd_scan_workspace_size(0) > 0


def test_synthetic_scene_is_seeded_and_activated():
    a = T.synthetic_scene(7, 100)
    b = T.synthetic_scene(7, 100)
    np.testing.assert_array_equal(a.records, b.records)
    r = a.records
    np.testing.assert_allclose(r[:, 3], 1 / (1 + np.exp(-a.opacity_logits.astype(np.float64))), rtol=1e-6)
    np.testing.assert_allclose(r[:, 8:11], np.exp(a.log_scales.astype(np.float64)), rtol=1e-6)
    np.testing.assert_allclose(np.linalg.norm(r[:, 4:8], axis=1), 1.0, rtol=1e-6)
    assert np.all(r[:, 11] == 1.0)
    box = T.synthetic_scene(1, 1000, mean_box=3.0)
    assert np.abs(box.means).max() <= 3.0


def test_random_points_layout():
    r = T.random_points(3, 50, radius=10.0, min_scale=0.005, max_scale=0.2)
    assert r.shape == (50, 60)
    assert np.all(np.abs(r[:, 0:3]) <= 10.0)
    assert np.all((r[:, 8:11] >= 0.005) & (r[:, 8:11] <= 0.2))
    assert np.all(r[:, 4:8] == np.array([0, 0, 0, 1], np.float32))
    assert np.all(r[:, 15:] == 0)
