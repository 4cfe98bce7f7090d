"""Stage-by-stage parity of the CUDA pipeline (through the C ABI) with the oracle.

  preprocess   bit-exact vs the FP32 transcription; <= 1e-5 scaled relative
               error vs FP64 (tests/tolerances.py); tile counts exact except
               the FP64 oracle's edge set, which is counted and reported
  scan         K exact; key offsets exact (scanned in depth order over the
               visible items: the depth sort drops the culled ones, which the
               oracle's order puts last)
  keygen+sort  keys and values bit-exact vs keygen + std::stable_sort
  ranges       bit-exact
  blend        <= 1e-3 max-abs per channel vs FP64, outside flagged pixels
"""
import numpy as np
import pytest

import torpedo_gb300 as T
from tests import gpu_helpers as H
from tests import kat
from tests import tolerances as tol
from torpedo_gb300 import configs

pytestmark = pytest.mark.gpu


def _scene(name):
    if name == "cfg0":
        return configs.scene("cfg0").records, configs.cameras("cfg0")[0]
    if name == "cfg1_200k":
        return configs.scene("cfg1", 200_000).records, configs.cameras("cfg1")[0]
    if name == "cfg2_50k":
        return configs.scene("cfg2", 50_000).records, configs.cameras("cfg2")[0]
    if name == "odd_size":
        return configs.scene("cfg0").records, T.Camera.orbit((0.3, -0.2, -4.0), 173, 91)
    if name == "kat_single":
        r, c, _ = kat.single_isotropic()
        return r, c
    if name == "kat_two":
        return kat.two_depths()
    if name == "kat_edge":
        return kat.tile_edge()
    if name == "kat_culled":
        return kat.culled()
    if name == "kat_screen_filling":
        return kat.screen_filling()
    if name == "kat_tiny_view":
        return kat.tiny_view()
    if name == "kat_wide_row":
        return kat.wide_row()
    raise KeyError(name)


SCENES = ["cfg0", "cfg1_200k", "cfg2_50k", "odd_size", "kat_single", "kat_two", "kat_edge", "kat_culled",
          "kat_screen_filling", "kat_tiny_view", "kat_wide_row"]
_cache = {}


@pytest.fixture(params=SCENES)
def frame(request, cuda):
    name = request.param
    if name not in _cache:
        recs, cam = _scene(name)
        eng, stats = H.render(recs, [cam])
        g = H.gpu_state(eng, stats)
        eng.close()
        o = H.oracle_frame(recs, cam)
        _cache[name] = (recs, cam, stats, g, o)
    return _cache[name]


def test_splats_bit_exact_vs_fp32_transcription(frame):
    recs, cam, stats, g, o = frame
    np.testing.assert_array_equal(g["splats"], o["s32"])


def test_splats_vs_fp64(frame):
    recs, cam, stats, g, o = frame
    s = g["splats"]
    vis = (s[:, 7] != 0) & (o["s64"][:, 7] != 0) & ~o["frag"]
    if vis.any():
        err = tol.splat_rel_error(s.view(np.float32)[vis], o["s64"][vis], cam.width, cam.height)
        assert err.max() <= tol.PREPROCESS_REL, err.max()
    tiles_match = s[:, 3] == o["s64"][:, 3].astype(np.uint32)
    assert np.all(tiles_match | o["frag"])
    edge = int((~tiles_match).sum())
    print(f"tile-count edge cases: {edge} of {len(s)} (flagged {int(o['frag'].sum())})")


def test_scan_offsets_and_total(frame):
    recs, cam, stats, g, o = frame
    assert stats["keys"] == o["K"]
    vis = int((o["s32"][:, 3] > 0).sum())
    assert stats["visible"] == vis
    # the culled items close the oracle's depth order with offset K; the engine
    # keeps only the visible prefix
    assert np.all(o["depth_offsets"][vis:] == o["K"])
    np.testing.assert_array_equal(g["offsets"][:vis], o["depth_offsets"][:vis])


def test_sorted_keys_and_values_bit_exact(frame):
    recs, cam, stats, g, o = frame
    np.testing.assert_array_equal(g["keys"], o["keys"])
    np.testing.assert_array_equal(g["vals"], o["vals"])


def test_tile_ranges_bit_exact(frame):
    recs, cam, stats, g, o = frame
    np.testing.assert_array_equal(g["ranges"], o["ranges"])


def test_image_vs_fp64(frame):
    recs, cam, stats, g, o = frame
    img = g["images"][0]
    err = np.abs(img.astype(np.float64) - o["img64"]).max(axis=2)
    ok = ~o["pfrag"]
    assert err[ok].max(initial=0.0) <= tol.IMAGE_ABS, err[ok].max()
    print(f"pixels flagged near a blend threshold: {int(o['pfrag'].sum())} of {err.size}; "
          f"max err elsewhere {err[ok].max(initial=0.0):.2e}")


def test_final_T_and_contributors(frame):
    recs, cam, stats, g, o = frame
    T_ = g["final_T"].reshape(cam.height, cam.width)
    nc = g["n_contrib"].reshape(cam.height, cam.width)
    ok = ~o["pfrag"]
    assert np.abs(T_[ok] - o["T64"][ok]).max(initial=0.0) <= 1e-3
    assert np.mean(nc[ok] == o["nc64"][ok]) >= 0.999


def test_thin_rotated_needles(cuda):
    """Long, thin, rotated Gaussians (kat.thin_rotated): the case where the
    blend's per-block cull is easiest to get wrong. Their FP32 conics carry
    up to 2e-3 relative error against FP64 (condition numbers near 3e4), the
    reference's own FP32 arithmetic, so the blend is checked against an FP64
    blend of the exact FP32 splats instead: a contributing pair that the cull
    dropped would change the contributor count, T and colour of the pixels
    along a needle's edge, far more than the few pixels where an FP32 decision
    near a threshold goes the other way."""
    from oracle import oracle as O

    recs, cam = kat.thin_rotated()
    eng, stats = H.render(recs, [cam])
    g = H.gpu_state(eng, stats)
    eng.close()
    o = H.oracle_frame(recs, cam, f64=False)
    np.testing.assert_array_equal(g["splats"], o["s32"])
    np.testing.assert_array_equal(g["keys"], o["keys"])
    np.testing.assert_array_equal(g["vals"], o["vals"])
    np.testing.assert_array_equal(g["ranges"], o["ranges"])
    s = o["s32"]
    s64 = s.view(np.float32).astype(np.float64)
    s64[:, 3] = s[:, 3].astype(np.float64)
    img64, T64, nc64, pfrag = O.blend_f64(s64, o["vals"], o["ranges"], cam.width, cam.height)
    ok = ~pfrag
    err = np.abs(g["images"][0].astype(np.float64) - img64).max(axis=2)[ok]
    T_ = g["final_T"].reshape(cam.height, cam.width).astype(np.float64)[ok]
    nc = g["n_contrib"].reshape(cam.height, cam.width)[ok]
    n = err.size
    print(f"thin needles: K={stats['keys']}, pixels > 1e-3: {int((err > 1e-3).sum())} of {n}, "
          f"max {err.max():.2e}; contributor counts equal: {np.mean(nc == nc64[ok]):.5f}")
    assert (err > tol.IMAGE_ABS).sum() <= n // 1000
    assert (np.abs(T_ - T64[ok]) > 1e-3).sum() <= n // 1000
    assert np.mean(nc == nc64[ok]) >= 0.999


@pytest.mark.parametrize("deg", [0, 1, 2, 3])
@pytest.mark.parametrize("compat", [True, False])
def test_sh_degrees_and_band3_mode(cuda, deg, compat):
    recs, cam = _scene("cfg0")
    eng, stats = H.render(recs, [cam], sh_degree=deg, band3_compat=compat)
    g = H.gpu_state(eng, stats)
    eng.close()
    o = H.oracle_frame(recs, cam, sh_degree=deg, band3_compat=compat, f64=False)
    np.testing.assert_array_equal(g["splats"], o["s32"])
    np.testing.assert_array_equal(g["keys"], o["keys"])


def test_entities_with_transforms(cuda):
    """Per-entity model matrices (TransformHost) move the mean only (project.slang:43-48)."""
    recs = configs.scene("cfg0", 6000).records
    ent = (np.arange(len(recs)) % 3).astype(np.uint32)
    c, s = np.cos(0.3), np.sin(0.3)
    tr = np.stack([np.eye(4, dtype=np.float32),
                   np.array([[c, 0, s, 0.2], [0, 1, 0, -0.1], [-s, 0, c, 0.4], [0, 0, 0, 1]], np.float32),
                   np.array([[1, 0, 0, 0], [0, 1, 0, -1.0], [0, 0, 1, -0.5], [0, 0, 0, 1]], np.float32)])
    cam = T.Camera.orbit((1.0, -0.5, -4.5), 320, 240)
    eng, stats = H.render(recs, [cam], entity_index=ent, n_entities=3, transforms=tr)
    g = H.gpu_state(eng, stats)
    eng.close()
    o = H.oracle_frame(recs, cam, ent_idx=ent, transforms=tr.reshape(3, 16), f64=False)
    np.testing.assert_array_equal(g["splats"], o["s32"])
    np.testing.assert_array_equal(g["keys"], o["keys"])
    np.testing.assert_array_equal(g["vals"], o["vals"])


def test_rgba8_pack(cuda):
    recs, cam = _scene("cfg0")
    eng, stats = H.render(recs, [cam])
    rgb = eng.read_image()[0]
    rgba = eng.read_image(rgba8=True)[0]
    eng.close()
    exp = np.clip(np.rint(np.clip(rgb, 0, 1) * 255.0), 0, 255).astype(np.uint8)
    assert np.abs(rgba[..., :3].astype(int) - exp.astype(int)).max() <= 1
    assert np.all(rgba[..., 3] == 255)


def test_graph_replay_matches_eager(cuda):
    recs, cam = _scene("cfg0")
    eng = T.GaussianEngine(use_graph=True)
    eng.compile(recs)
    eng.set_camera(cam)
    first = eng.raster_frame()
    img1 = eng.read_image()[0].copy()
    cam2 = T.Camera.orbit((0.5, 0.2, -4.0), cam.width, cam.height)
    for _ in range(3):  # graph replays, including a camera change between replays
        eng.set_camera(cam2)
        eng.raster_frame()
    eng.set_camera(cam)
    again = eng.raster_frame()
    img2 = eng.read_image()[0]
    eng.close()
    assert first["keys"] == again["keys"]
    np.testing.assert_array_equal(img1, img2)


def test_render_async_pipelined_matches_synchronous(cuda):
    """tpd_render_async / tpd_wait_render with two renders in flight and the
    camera changed between them give the synchronous frames bit for bit
    (RGBA8 into pinned host memory, RGB32F into device memory); a third
    outstanding render is refused."""
    torch = cuda
    recs, cam = _scene("cfg0")
    cam2 = T.Camera.orbit((0.7, -0.4, -4.2), cam.width, cam.height)
    ref = {}
    for name, c in (("a", cam), ("b", cam2)):
        e = T.GaussianEngine()
        e.compile(recs)
        e.set_camera(c)
        e.raster_frame()
        ref[name] = (e.read_image(rgba8=True)[0].copy(), e.read_image()[0].copy())
        e.close()
    eng = T.GaussianEngine()
    eng.compile(recs)
    eng.set_camera(cam)
    eng.raster_frame()
    px = cam.width * cam.height
    host = [torch.zeros(px * 4, dtype=torch.uint8, pin_memory=True) for _ in range(2)]
    dev = [torch.zeros(px * 3, dtype=torch.float32, device="cuda") for _ in range(2)]
    order = ["a", "b", "a", "b"]
    for rgba in (True, False):
        bufs = host if rgba else dev
        for i, name in enumerate(order):
            eng.set_camera(cam if name == "a" else cam2)
            eng.render_async(bufs[i % 2], rgba8=rgba)
            if i == 1:
                with pytest.raises(T.TpdError):  # a third render while two are outstanding
                    eng.render_async(bufs[0], rgba8=rgba)
            if i >= 1:
                st = eng.wait_render()
                assert st["status"] == 0
                prev = order[i - 1]
                got = bufs[(i - 1) % 2].cpu().numpy()
                if rgba:
                    np.testing.assert_array_equal(got.reshape(cam.height, cam.width, 4), ref[prev][0])
                else:
                    np.testing.assert_array_equal(got.reshape(cam.height, cam.width, 3), ref[prev][1])
        eng.wait_render()
        got = bufs[(len(order) - 1) % 2].cpu().numpy()
        last = ref[order[-1]][0 if rgba else 1]
        np.testing.assert_array_equal(got.reshape(last.shape), last)
    eng.close()


def test_render_async_views_and_transforms(cuda):
    """Pipelined renders of three views of mixed sizes with per-entity model
    matrices, the matrices changed between renders: each slot's captured
    graph uploads its own views and transforms and the blend writes the
    RGBA8 image itself, bit for bit the synchronous frames' packed images."""
    torch = cuda
    recs = configs.scene("cfg0", 6000).records
    ent = (np.arange(len(recs)) % 3).astype(np.uint32)
    c, s = np.cos(0.3), np.sin(0.3)
    tr_a = np.stack([np.eye(4, dtype=np.float32),
                     np.array([[c, 0, s, 0.2], [0, 1, 0, -0.1], [-s, 0, c, 0.4], [0, 0, 0, 1]], np.float32),
                     np.array([[1, 0, 0, 0], [0, 1, 0, -1.0], [0, 0, 1, -0.5], [0, 0, 0, 1]], np.float32)])
    tr_b = tr_a.copy()
    tr_b[1, 0, 3] = -0.3
    cams = [T.Camera.orbit((1.0, -0.5, -4.5), 320, 240), T.Camera.orbit((-0.8, 0.3, -4.0), 173, 91),
            T.Camera.orbit((0.2, 0.9, -4.8), 256, 256)]

    def make():
        e = T.GaussianEngine()
        e.compile(recs, ent, 3)
        e.set_views(cams)
        return e

    ref = {}
    for name, tr in (("a", tr_a), ("b", tr_b)):
        e = make()
        for k, m in enumerate(tr):
            e.transform_host.transform(k, m)
        e.raster_frame()
        ref[name] = [img.copy() for img in e.read_image(rgba8=True)]
        e.close()
    eng = make()
    for k, m in enumerate(tr_a):
        eng.transform_host.transform(k, m)
    eng.raster_frame()
    px = sum(cm.width * cm.height for cm in cams)
    host = [torch.zeros(px * 4, dtype=torch.uint8, pin_memory=True) for _ in range(2)]
    order = ["a", "b", "b", "a"]
    for i, name in enumerate(order):
        for k, m in enumerate(tr_a if name == "a" else tr_b):
            eng.transform_host.transform(k, m)
        eng.render_async(host[i % 2], rgba8=True)
        if i >= 1:
            assert eng.wait_render()["status"] == 0
            got, off = host[(i - 1) % 2].cpu().numpy(), 0
            for cm, want in zip(cams, ref[order[i - 1]]):
                n = cm.width * cm.height * 4
                np.testing.assert_array_equal(got[off:off + n].reshape(want.shape), want)
                off += n
    eng.wait_render()
    eng.close()
