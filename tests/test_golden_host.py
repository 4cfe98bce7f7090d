"""Host-side inputs of the path against golden vectors produced by the reference's
own C++ (tests/golden/make_golden.py compiles PerspectiveCamera, Camera::lookAt,
math::mul, GaussianPoint::fromModel and getHigherMSB from the reference tree).
Bit-exact: these feed the kernels, so they must match the reference exactly."""
from pathlib import Path

import numpy as np
import pytest

import torpedo_gb300 as T
from oracle import oracle as O

GOLD = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD / "reference_host.npz")


def test_camera_matrices_bit_exact(gold):
    meta = gold["cam_meta"]
    for i in range(meta.shape[0]):
        eye, ctr, up = meta[i, 0:3], meta[i, 3:6], meta[i, 6:9]
        w, h, fov, near, far = int(meta[i, 9]), int(meta[i, 10]), float(meta[i, 11]), float(meta[i, 12]), float(meta[i, 13])
        view = T.look_at(eye, ctr, up).reshape(16)
        proj = T.perspective(w, h, fov, near, far).reshape(16)
        pv = T.mat4_mul(proj, view).reshape(16)
        np.testing.assert_array_equal(view.view(np.uint32), gold["cam_view"][i].view(np.uint32), err_msg=f"view {i}")
        np.testing.assert_array_equal(proj.view(np.uint32), gold["cam_proj"][i].view(np.uint32), err_msg=f"proj {i}")
        np.testing.assert_array_equal(pv.view(np.uint32), gold["cam_projview"][i].view(np.uint32), err_msg=f"pv {i}")
        assert proj[0] == gold["cam_focal"][i][0] and proj[5] == gold["cam_focal"][i][1]


def test_oracle_camera_matrices_bit_exact(gold):
    """The oracle's own camera maths (it builds the reference arm's inputs
    without the product library) against the same golden vectors."""
    meta = gold["cam_meta"]
    for i in range(meta.shape[0]):
        eye, ctr, up = meta[i, 0:3], meta[i, 3:6], meta[i, 6:9]
        w, h, fov, near, far = int(meta[i, 9]), int(meta[i, 10]), float(meta[i, 11]), float(meta[i, 12]), float(meta[i, 13])
        view = O.look_at(eye, ctr, up).reshape(16)
        proj = O.perspective(w, h, fov, near, far).reshape(16)
        pv = O.mat4_mul(proj.reshape(4, 4), view.reshape(4, 4)).reshape(16)
        np.testing.assert_array_equal(view.view(np.uint32), gold["cam_view"][i].view(np.uint32), err_msg=f"view {i}")
        np.testing.assert_array_equal(proj.view(np.uint32), gold["cam_proj"][i].view(np.uint32), err_msg=f"proj {i}")
        np.testing.assert_array_equal(pv.view(np.uint32), gold["cam_projview"][i].view(np.uint32), err_msg=f"pv {i}")
    for a, b, ab in zip(gold["mul_a"], gold["mul_b"], gold["mul_ab"]):
        np.testing.assert_array_equal(O.mat4_mul(a.reshape(4, 4), b.reshape(4, 4)).reshape(16).view(np.uint32),
                                      ab.view(np.uint32))


@pytest.mark.parametrize("seed,box", [(0, 0.0), (1, 3.0), (3, 0.0), (4, 10.0)])
def test_oracle_scene_generator_equals_the_product_generator(seed, box):
    """The seeded scene the oracle generates is the product's, byte for byte."""
    a = O.synthetic_records(seed, 3000, box)
    b = T.synthetic_scene(seed, 3000, box).records
    np.testing.assert_array_equal(a.view(np.uint32), b.view(np.uint32))


def test_mat4_mul_bit_exact(gold):
    for a, b, ab in zip(gold["mul_a"], gold["mul_b"], gold["mul_ab"]):
        np.testing.assert_array_equal(T.mat4_mul(a, b).reshape(16).view(np.uint32), ab.view(np.uint32))


def test_key_bits_match_get_higher_msb(gold):
    for n, msb in zip(gold["msb_n"], gold["msb_ref"]):
        assert T.key_bits_for_tiles(int(n)) == int(msb) + 32
        assert O.higher_msb(int(n)) == int(msb)


def test_pass_counts_of_configs():
    # 2-bit passes of the reference for the workload image sizes
    assert O.radix_pass_count(256, 256) == 21
    assert O.radix_pass_count(800, 800) == 22
    assert O.radix_pass_count(640, 480) == 22
    assert O.radix_pass_count(1280, 720) == 22
    assert O.radix_pass_count(1920, 1080) == 23
    assert O.radix_pass_count(3840, 2160) == 24


@pytest.mark.parametrize("name", ["ply_deg3_binary", "ply_deg1_ascii"])
def test_ply_loader_matches_from_model(gold, name):
    rec = T.load_ply(GOLD / f"{name}.ply")
    ref = gold[f"{name}_records"]
    assert rec.shape == ref.shape
    np.testing.assert_array_equal(rec.view(np.uint32), ref.view(np.uint32))


def test_ply_loader_errors(tmp_path):
    bad = tmp_path / "bad.ply"
    bad.write_text("not a ply\n")
    with pytest.raises(T.TpdError):
        T.load_ply(bad)
    with pytest.raises(T.TpdError):
        T.load_ply(tmp_path / "missing.ply")


@pytest.mark.parametrize("key,row", [("random_records", 0), ("random_records_b", 1)])
def test_random_points_match_the_reference_generator(gold, key, row):
    """GaussianPoint::random (GaussianGeometry.cpp:8-32) with its mt19937
    seeded: positions, opacities, quaternions, scales and SH bit for bit. The
    reference fills the DC colour with rgb2sh(dist_sh(rng), dist_sh(rng),
    dist_sh(rng)), whose argument order C++ leaves to the compiler: clang, the
    reference's own (README.md:116), evaluates left to right, as tpd_random_points
    does; the g++ build that recorded the fixture evaluates right to left
    (random_args_right_to_left), which swaps the red and blue draws."""
    a = gold["random_args"][row]
    ref = gold[key].copy()
    got = T.random_points(int(a[0]), int(a[1]), float(a[2]), tuple(float(x) for x in a[3:6]), float(a[6]), float(a[7]),
                          float(a[8]), float(a[9]))
    if int(gold["random_args_right_to_left"]):
        ref[:, [12, 14]] = ref[:, [14, 12]]
    np.testing.assert_array_equal(got.view(np.uint32), ref.view(np.uint32))
