"""The oracle's FP32 transcription against the reference's own compute
shaders. tests/golden/reference_shaders.npz holds frames of the scenes in
tests/golden/shader_scenes.py run through the reference's Slang source
(translated token by token to C++ and run on the CPU with the dispatch
sequence of GaussianEngine::rasterFrame: oracle/slang_to_cpp.py,
oracle/slang_cpu.h, oracle/ref_shaders.cpp). Splats, prefix offsets, sorted
keys and values, tile ranges and the stored image must equal the
transcription's bit for bit. Where the reference tree is present, the
shaders are built and run again on a few scenes to check the fixture."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.golden import shader_scenes as SS


@pytest.fixture(scope="module")
def fixture():
    return SS.load_fixture()


def _oracle_frame(d):
    oc = O.camera(d["view"], d["projview"], d["width"], d["height"], focal=tuple(float(x) for x in d["focal"]))
    s32 = O.preprocess_f32(d["records"], oc, d["sh_degree"], True, d.get("ent_idx"), d.get("transforms"))
    offs, k = O.scan_tiles(s32)
    keys, vals = O.stable_sort(*O.keygen(s32, offs, k, d["width"], d["height"]))
    tiles = ((d["width"] + 15) // 16) * ((d["height"] + 15) // 16)
    ranges = O.tile_ranges(keys, tiles)
    img, _, _ = O.blend_f32(s32, vals, ranges, d["width"], d["height"])
    rgba = np.concatenate([img, np.ones(img.shape[:2] + (1,), np.float32)], axis=2)
    return dict(splats=s32, offsets=offs, keys=keys, vals=vals, ranges=ranges, image=rgba, K=k)


def test_fixture_covers_the_scenes(fixture):
    assert set(fixture) == set(SS.build_scenes())
    assert fixture["cfg0"]["K"] == 23403 and fixture["cfg0"]["passes"] == 21
    assert fixture["cfg1_patch"]["passes"] == 23


@pytest.mark.parametrize("name", sorted(SS.build_scenes()))
def test_transcription_equals_reference_shaders(fixture, name):
    d = fixture[name]
    o = _oracle_frame(d)
    assert o["K"] == d["K"]
    for k in ("splats", "offsets", "keys", "vals", "ranges", "image"):
        if SS.digest(o[k]) != str(d[f"sha_{k}"]):
            detail = ""
            if k in d:
                bad = np.argwhere(np.asarray(o[k]) != d[k])
                detail = f": {len(bad)} elements differ, first at {bad[:3].tolist()}"
            pytest.fail(f"{name}: {k} differs from the reference shaders{detail}")


def test_rect_bound_rounds_like_the_shader(fixture):
    """The edge Gaussian's right (bottom) tile bound p + r + 16 - 1 rounds up
    to the next tile, so it covers 2 tiles, not the 1 that (p + r) + 15 gives."""
    for name in ("rect_edge_x", "rect_edge_y"):
        sp = fixture[name]["splats"]
        assert int(sp[0, 3]) == 2, name
        p = np.float32(sp[0, 4 if name.endswith("x") else 5].view(np.float32))
        r = np.float32(sp[0, 7].view(np.float32))
        assert np.float32(p + r) == np.float32(1009.0) - np.float32(2.0 ** -14)
        assert int((np.float32(np.float32(p + r) + np.float32(16)) - np.float32(1)) / np.float32(16)) == 64
        assert int(np.float32(np.float32(p + r) + np.float32(15)) / np.float32(16)) == 63


@pytest.mark.parametrize("name", ["two_depths", "rect_edge_x", "sh_degree_1", "tiny_view"])
def test_fixture_matches_reference_shaders_run_here(fixture, name):
    from oracle import reference

    if not reference.build_ref.available():
        pytest.skip("the reference tree is not present on this machine; the fixture stands in for it")
    d = fixture[name]
    r = reference.frame(d["records"], d["view"], d["projview"], d["focal"], d["width"], d["height"], d["sh_degree"],
                        d.get("ent_idx"), d.get("transforms"))
    assert r["oob"] == 0 and r["K"] == d["K"]
    for k in ("splats", "offsets", "keys", "vals", "ranges", "image"):
        assert SS.digest(r[k]) == str(d[f"sha_{k}"]), (name, k)
