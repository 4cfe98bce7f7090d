"""The oracle against hand-built known answers, its two arithmetic forms against
each other, and its sort / scan / range properties (CPU only)."""
import math

import numpy as np
import pytest

import torpedo_gb300 as T
from oracle import oracle as O
from torpedo_gb300 import configs
from tests import kat
from tests import tolerances as tol


def ocam(cam):
    return O.camera(cam.view, cam.projview(), cam.width, cam.height, focal=(cam.proj[0, 0], cam.proj[1, 1]))


def f32(splat_u32):
    return splat_u32.view(np.float32)


@pytest.mark.parametrize("compat", [False, True])
def test_single_isotropic_known_answer(compat):
    rec, cam, exp = kat.single_isotropic()
    s = O.preprocess_f32(rec, ocam(cam), band3_compat=compat)[0]
    f = f32(s)
    assert f[4] == pytest.approx(exp["px"], abs=1e-4) and f[5] == pytest.approx(exp["py"], abs=1e-4)
    assert f[6] == pytest.approx(exp["depth"], rel=1e-6)
    assert f[7] == exp["radius"]
    np.testing.assert_allclose(f[8:11], exp["conic"], rtol=1e-5, atol=1e-7)
    shift = exp["compat_shift"] if compat else 0.0
    np.testing.assert_allclose(f[0:3], np.array(exp["color"]) + shift, atol=1e-6)
    assert s[3] == exp["tiles"]
    assert f[11] == pytest.approx(0.8)


def test_single_isotropic_pixel_value():
    rec, cam, exp = kat.single_isotropic()
    sp = O.preprocess_f32(rec, ocam(cam), band3_compat=False)
    offs, k = O.scan_tiles(sp)
    keys, vals = O.keygen(sp, offs, k, 256, 256)
    keys, vals = O.stable_sort(keys, vals)
    rng = O.tile_ranges(keys, 256)
    img, T_, nc = O.blend_f32(sp, vals, rng, 256, 256)
    # pixel (127, 127): d = (0.5, 0.5)
    power = -0.5 * (0.25 / exp["var"] + 0.25 / exp["var"])
    alpha = min(0.99, 0.8 * math.exp(power))
    np.testing.assert_allclose(img[127, 127], np.array(exp["color"]) * alpha, atol=1e-5)
    assert T_[127, 127] == pytest.approx(1 - alpha, abs=1e-6)
    assert nc[127, 127] == 1
    assert np.all(img[0:100, 0:100] == 0)  # outside the splat's tiles


def test_two_depths_front_to_back():
    recs, cam = kat.two_depths()
    sp = O.preprocess_f32(recs, ocam(cam))
    offs, k = O.scan_tiles(sp)
    keys, vals = O.stable_sort(*O.keygen(sp, offs, k, 256, 256))
    tile = 7 * 16 + 7
    rng = O.tile_ranges(keys, 256)
    s, e = rng[tile]
    assert list(vals[s:e]) == [1, 0]  # depth 4 before depth 6
    img, _, _ = O.blend_f32(sp, vals, rng, 256, 256)
    c = img[127, 127]
    assert c[0] > c[2]  # red in front dominates


def test_culled_known_answer():
    recs, cam = kat.culled()
    s = O.preprocess_f32(recs, ocam(cam))
    assert np.all(s == 0)


@pytest.mark.parametrize("k", list(range(1, 16)))
def test_sh_degree_cutoff(k):
    rec, cam = kat.sh_probe(k)
    band = 1 if k <= 3 else 2 if k <= 8 else 3
    cols = []
    for deg in range(4):
        s = O.preprocess_f32(rec, ocam(cam), sh_degree=deg)
        cols.append(f32(s[0])[0])
    for deg in range(4):
        if deg < band:
            assert cols[deg] == pytest.approx(0.5, abs=1e-7)
    if k != 12:
        assert cols[3] != pytest.approx(0.5, abs=1e-6) or k in ()  # feature contributes at full degree


def test_band3_compat_quirk():
    """common.slang:69 adds feature 12 instead of multiplying it: with compat on, a
    feature-12 coefficient of 1 shifts channel 0 by exactly 1 (before clamping)."""
    rec, cam = kat.sh_probe(12)
    on = f32(O.preprocess_f32(rec, ocam(cam), sh_degree=3, band3_compat=True)[0])[0]
    rec0 = rec.copy()
    rec0[0, 12 + 3 + 11] = 0.0
    base_on = f32(O.preprocess_f32(rec0, ocam(cam), sh_degree=3, band3_compat=True)[0])[0]
    assert on - base_on == pytest.approx(1.0, abs=1e-6)
    # without the quirk a coefficient of 1 multiplies the basis value, which the quirk adds alone
    off = f32(O.preprocess_f32(rec, ocam(cam), sh_degree=3, band3_compat=False)[0])[0]
    assert off == base_on


def _cfg0(n=None):
    cfg = configs.CONFIGS["cfg0"]
    sc = configs.scene(cfg, n)
    cam = configs.cameras(cfg)[0]
    return sc, cam


def test_f32_vs_f64_preprocess():
    sc, cam = _cfg0()
    oc = ocam(cam)
    s32 = O.preprocess_f32(sc.records, oc)
    s64, rect, frag = O.preprocess_f64(sc.records, oc)
    vis = (s32[:, 7] != 0) & (s64[:, 7] != 0) & ~frag
    err = tol.splat_rel_error(f32(s32)[vis], s64[vis], cam.width, cam.height)
    assert err.max() <= tol.PREPROCESS_REL, err.max()
    assert np.all(f32(s32)[vis][:, 7] == s64[vis][:, 7])
    tiles_ok = (s32[:, 3] == s64[:, 3].astype(np.uint32)) | frag
    assert tiles_ok.all()
    assert frag.sum() < 0.01 * len(frag)


def test_radix4_equals_stable_sort_random():
    rng = np.random.default_rng(0)
    for k, bits in [(1, 41), (255, 41), (256, 41), (257, 41), (5000, 46), (70000, 46)]:
        keys = rng.integers(0, 1 << 32, size=k, dtype=np.uint64) | (
            rng.integers(0, 1 << (bits - 32), size=k, dtype=np.uint64) << np.uint64(32))
        keys[::7] = keys[0]  # ties
        vals = np.arange(k, dtype=np.uint32)
        a = O.radix4_sort(keys, vals, (bits + 1) // 2)
        b = O.stable_sort(keys, vals)
        np.testing.assert_array_equal(a[0], b[0])
        np.testing.assert_array_equal(a[1], b[1])


def test_pipeline_properties_cfg0():
    sc, cam = _cfg0()
    oc = ocam(cam)
    sp = O.preprocess_f32(sc.records, oc)
    offs, k = O.scan_tiles(sp)
    assert k == int(sp[:, 3].astype(np.uint64).sum())
    keys, vals = O.keygen(sp, offs, k, 256, 256)
    ka, va = O.radix4_sort(keys, vals, O.radix_pass_count(256, 256))
    kb, vb = O.stable_sort(keys, vals)
    np.testing.assert_array_equal(ka, kb)
    np.testing.assert_array_equal(va, vb)
    assert np.all(np.diff(ka.astype(np.uint64)) >= 0) if k > 1 else True
    rng = O.tile_ranges(ka, 256)
    nonempty = rng[:, 1] > rng[:, 0]
    assert int((rng[nonempty, 1] - rng[nonempty, 0]).sum()) == k
    tiles = (ka >> np.uint64(32)).astype(np.int64)
    for t in np.nonzero(nonempty)[0][:50]:
        assert np.all(tiles[rng[t, 0]:rng[t, 1]] == t)


def test_blend_f32_vs_f64():
    sc, cam = _cfg0()
    oc = ocam(cam)
    sp = O.preprocess_f32(sc.records, oc)
    s64, _, _ = O.preprocess_f64(sc.records, oc)
    offs, k = O.scan_tiles(sp)
    keys, vals = O.stable_sort(*O.keygen(sp, offs, k, 256, 256))
    rng = O.tile_ranges(keys, 256)
    img32, _, _ = O.blend_f32(sp, vals, rng, 256, 256)
    img64, _, _, frag = O.blend_f64(s64, vals, rng, 256, 256)
    err = np.abs(img32 - img64).max(axis=2)
    assert err[~frag].max() <= tol.IMAGE_ABS
    assert frag.mean() < 0.02


def test_backward_f64_matches_finite_differences():
    sc = configs.scene("cfg0", 300)
    cam = T.Camera.orbit((0.0, 0.0, -5.0), 64, 64)
    oc = ocam(cam)
    sp = O.preprocess_f32(sc.records, oc)
    offs, k = O.scan_tiles(sp)
    keys, vals = O.stable_sort(*O.keygen(sp, offs, k, 64, 64))
    rng = O.tile_ranges(keys, 16)
    params = [sc.means.astype(np.float64), sc.log_scales.astype(np.float64), sc.quats.astype(np.float64),
              sc.opacity_logits.astype(np.float64), sc.sh.astype(np.float64)]
    dimg = np.random.default_rng(5).normal(size=(64, 64, 3))
    grads, _ = O.backward_f64(params, oc, vals, rng, dimg)
    loss = lambda ps: float((O.render_params_f64(ps, oc, vals, rng) * dimg).sum())
    r = np.random.default_rng(6)
    vis = np.nonzero(sp[:, 7])[0]
    checked = 0
    bad = 0
    for gi, (pidx, shape) in enumerate([(0, 3), (1, 3), (2, 4), (3, 1), (4, 48)]):
        for _ in range(12):
            i = int(r.choice(vis))
            j = int(r.integers(0, shape))
            ps = [p.copy() for p in params]
            h = 1e-4
            flat = ps[pidx].reshape(len(ps[pidx]), -1)
            flat[i, j] += h
            lp = loss(ps)
            flat[i, j] -= 2 * h
            lm = loss(ps)
            fd = (lp - lm) / (2 * h)
            an = grads[pidx].reshape(len(grads[pidx]), -1)[i, j]
            checked += 1
            if abs(fd - an) > 1e-3 * max(1.0, abs(fd), abs(an)) + 1e-6:
                bad += 1
    # decisions (alpha threshold, early stop) make a few parameters non-smooth
    assert bad <= checked // 20, (bad, checked)
