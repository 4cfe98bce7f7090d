"""Generates the golden fixtures of tests/golden/ from the reference's own C++.

Run where the reference tree is present (oracle/build_ref.py locates it; set
TPD_REFERENCE_ROOT to point elsewhere): it builds oracle/_ref/libtpdref.so
with oracle/build_ref.py and records
  reference_host.npz   camera matrices (view, projection, proj*view, focal) from
                       PerspectiveCamera + Camera::lookAt + math::mul, the
                       getHigherMSB table, and GaussianPoint::fromModel records
                       of the PLY files below
  ply_*.ply            small seeded 3DGS PLY files (binary and ASCII)
  reference_shaders.npz  (`make_golden.py shaders`) frames of the scenes in
                       shader_scenes.py run through the reference's own
                       compute shaders (their Slang source, translated and run
                       on the CPU by oracle/ref_shaders.cpp): K, pass count and
                       SHA-256 digests of splats, offsets, sorted keys and
                       values, ranges and image; the arrays of small scenes
The tests compare libtpdsplat's host code, the oracle and the CUDA pipeline
against these.
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from oracle import build_ref  # noqa: E402
from torpedo_gb300.configs import FAR, FOV, NEAR, UP, fibonacci_sphere  # noqa: E402


def ref_lib():
    lib = C.CDLL(str(build_ref.build(force=True)))
    F = C.POINTER(C.c_float)
    lib.ref_camera.argtypes = [F, F, F, C.c_uint32, C.c_uint32, C.c_float, C.c_float, C.c_float, F, F, F, F]
    lib.ref_mat4_mul.argtypes = [F, F, F]
    lib.ref_higher_msb.argtypes = [C.c_uint32]
    lib.ref_higher_msb.restype = C.c_uint32
    lib.ref_gaussian_point_size.restype = C.c_uint32
    lib.ref_from_model.argtypes = [C.c_char_p, F, C.c_uint32]
    lib.ref_from_model.restype = C.c_uint32
    lib.ref_random_points.argtypes = [C.c_uint32, C.c_uint32, C.c_float, F, C.c_float, C.c_float, C.c_float,
                                      C.c_float, F]
    lib.ref_args_right_to_left.restype = C.c_int
    return lib


def fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def camera_cases():
    cases = []
    sizes = [(256, 256), (1920, 1080), (800, 800), (640, 480), (1280, 720), (3840, 2160), (64, 64), (17, 33)]
    for w, h in sizes:
        cases.append(((0.0, 0.0, -5.0), (0.0, 0.0, 0.0), UP, w, h, FOV, NEAR, FAR))
    for i, eye in enumerate(fibonacci_sphere(16)):
        w, h = sizes[i % len(sizes)]
        cases.append((tuple(float(x) for x in eye), (0.0, 0.0, 0.0), UP, w, h, FOV, NEAR, FAR))
    # VolumeSplatting demo camera (demo/VolumeSplatting/main.cpp:108), constructor projection
    cases.append(((-2.0, -1.0, 0.0), (0.0, 0.0, 0.0), (0.0, -1.0, 0.0), 1280, 720, 0.0, 0.01, 100.0))
    cases.append(((0.3, -0.7, 2.5), (0.1, 0.2, -0.3), (0.0, 0.0, 1.0), 1920, 1080, 45.0, 0.5, 50.0))
    return cases


def write_ply(path: Path, rng, n: int, n_rest: int, binary: bool):
    names = ["x", "y", "z", "nx", "ny", "nz", "f_dc_0", "f_dc_1", "f_dc_2"] + [f"f_rest_{i}" for i in range(n_rest)]
    names += ["opacity", "scale_0", "scale_1", "scale_2", "rot_0", "rot_1", "rot_2", "rot_3"]
    data = rng.normal(0.0, 1.0, size=(n, len(names))).astype(np.float32)
    data[:, names.index("scale_0"):names.index("scale_2") + 1] -= 4.0
    hdr = "ply\nformat {} 1.0\nelement vertex {}\n".format("binary_little_endian" if binary else "ascii", n)
    hdr += "".join(f"property float {nm}\n" for nm in names) + "end_header\n"
    with open(path, "wb") as f:
        f.write(hdr.encode())
        if binary:
            f.write(data.astype("<f4").tobytes())
        else:
            for row in data:
                f.write((" ".join(repr(float(v)) for v in row) + "\n").encode())


def main():
    lib = ref_lib()
    assert lib.ref_gaussian_point_size() == 240
    cams = camera_cases()
    out = {}
    meta = np.zeros((len(cams), 14), np.float32)  # eye3 center3 up3 w h fov near far
    views, projs, pvs, focals = [], [], [], []
    for i, (eye, ctr, up, w, h, fov, near, far) in enumerate(cams):
        e, c, u = (np.asarray(v, np.float32) for v in (eye, ctr, up))
        v = np.zeros(16, np.float32); p = np.zeros(16, np.float32); pv = np.zeros(16, np.float32)
        fo = np.zeros(2, np.float32)
        lib.ref_camera(fp(e), fp(c), fp(u), w, h, fov, near, far, fp(v), fp(p), fp(pv), fp(fo))
        meta[i] = [*eye, *ctr, *up, w, h, fov, near, far]
        views.append(v); projs.append(p); pvs.append(pv); focals.append(fo)
    out["cam_meta"] = meta
    out["cam_view"] = np.stack(views)
    out["cam_proj"] = np.stack(projs)
    out["cam_projview"] = np.stack(pvs)
    out["cam_focal"] = np.stack(focals)

    rng = np.random.default_rng(1234)
    a = rng.normal(0, 3, size=(32, 16)).astype(np.float32)
    b = rng.normal(0, 3, size=(32, 16)).astype(np.float32)
    prod = np.zeros((32, 16), np.float32)
    for i in range(32):
        r = np.zeros(16, np.float32)
        lib.ref_mat4_mul(fp(np.ascontiguousarray(a[i])), fp(np.ascontiguousarray(b[i])), fp(r))
        prod[i] = r
    out["mul_a"], out["mul_b"], out["mul_ab"] = a, b, prod

    tiles = sorted(set([0, 1, 2, 3, 255, 256, 257, 1200, 2500, 3600, 8160, 8192, 32400, 65535, 65536, 65537,
                        1 << 20, (1 << 31) + 5] + [int(x) for x in rng.integers(1, 1 << 24, size=64)]))
    out["msb_n"] = np.asarray(tiles, np.uint32)
    out["msb_ref"] = np.asarray([lib.ref_higher_msb(t) for t in tiles], np.uint32)

    for name, n, n_rest, binary in [("ply_deg3_binary", 96, 45, True), ("ply_deg1_ascii", 24, 9, False)]:
        path = HERE / f"{name}.ply"
        write_ply(path, rng, n, n_rest, binary)
        cnt = lib.ref_from_model(str(path).encode(), None, 0)
        rec = np.zeros((cnt, 60), np.float32)
        lib.ref_from_model(str(path).encode(), fp(rec), cnt)
        out[f"{name}_records"] = rec

    # GaussianPoint::random with its generator seeded: (seed, n, radius, center xyz, scale and opacity bounds)
    rp_args = np.array([[1, 64, 2.5, 0.1, -0.2, 0.3, 0.01, 0.1, 0.2, 0.9],
                        [7, 40, 10.0, 0.0, 0.0, 0.0, 0.005, 0.2, 0.1, 1.0]], np.float32)
    rp = []
    for a in rp_args:
        rec = np.zeros((int(a[1]), 60), np.float32)
        ctr = np.ascontiguousarray(a[3:6])
        lib.ref_random_points(int(a[0]), int(a[1]), float(a[2]), fp(ctr), float(a[6]), float(a[7]), float(a[8]),
                              float(a[9]), fp(rec))
        rp.append(rec)
    out["random_args"] = rp_args
    out["random_records"] = np.stack(rp[:1])[0]
    out["random_records_b"] = rp[1]
    out["random_args_right_to_left"] = np.array(lib.ref_args_right_to_left(), np.int32)

    np.savez_compressed(HERE / "reference_host.npz", **out)
    print("wrote", HERE / "reference_host.npz", {k: v.shape for k, v in out.items()})


def shaders():
    import time

    from oracle import reference
    from tests.golden import shader_scenes as SS

    out = {}
    names = []
    for name, sc in SS.build_scenes().items():
        t0 = time.perf_counter()
        r = reference.frame(sc["records"], sc["view"], sc["projview"], sc["focal"], sc["width"], sc["height"],
                            sc["sh_degree"], sc["ent_idx"], sc["transforms"])
        assert r["oob"] == 0, f"{name}: {r['oob']} out-of-range buffer accesses"
        n = sc["records"].shape[0]
        out[f"{name}/meta"] = np.array([sc["width"], sc["height"], sc["sh_degree"], r["K"], r["passes"], n], np.int64)
        for k in ("view", "proj", "projview", "focal"):
            out[f"{name}/{k}"] = sc[k]
        if sc["gen"] is not None:
            out[f"{name}/gen"] = np.array(sc["gen"], np.float64)
        else:
            out[f"{name}/records"] = sc["records"]
        if sc["ent_idx"] is not None:
            out[f"{name}/ent_idx"] = sc["ent_idx"]
            out[f"{name}/transforms"] = sc["transforms"]
        for k in ("splats", "offsets", "keys", "vals", "ranges", "image"):
            out[f"{name}/sha_{k}"] = np.array(SS.digest(r[k]))
        if r["K"] <= SS.SMALL_KEYS:
            for k in ("splats", "keys", "vals", "ranges"):
                out[f"{name}/{k}"] = r[k]
        if sc["width"] * sc["height"] <= SS.SMALL_PIXELS:
            out[f"{name}/image"] = r["image"][..., :3]
        names.append(name)
        print(f"{name}: K={r['K']} passes={r['passes']} ({time.perf_counter() - t0:.1f} s)", flush=True)
    out["scenes"] = np.array(names)
    np.savez_compressed(SS.FIXTURE, **out)
    print("wrote", SS.FIXTURE, SS.FIXTURE.stat().st_size, "bytes")


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "shaders":
        shaders()
    else:
        main()
