"""The scenes whose reference-shader outputs are recorded as golden vectors
(tests/golden/reference_shaders.npz, written by make_golden.py), and the
helpers that read them back.

Each scene is a frame of the reference pipeline: records, one camera, the SH
degree and optional per-entity model matrices. The fixture keeps every input
it needs (records of the hand-built scenes, or the seed of a generated one;
camera constants as arrays), and for the outputs K, the radix pass count and a
SHA-256 of each array (splats after project, prefix offsets, sorted keys and
values, tile ranges, the stored float image), plus the arrays themselves for
the small scenes (the image as RGB: the shader stores (C, 1)).
"""
from __future__ import annotations

import hashlib
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
FIXTURE = HERE / "reference_shaders.npz"
SMALL_KEYS = 512  # scenes with at most this many keys keep their arrays too
SMALL_PIXELS = 4096  # and scenes with at most this many pixels their image (RGB)


def digest(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _camera(eye, w, h):
    """view, proj, proj * view and (P00, P11) of a view at `eye` looking at
    the origin (60 degrees, near 0.2, far 100, up (0, -1, 0))."""
    from oracle import oracle as O

    view = O.look_at(eye, (0.0, 0.0, 0.0), (0.0, -1.0, 0.0))
    proj = O.perspective(w, h, 60.0, 0.2, 100.0)
    return view, proj, O.mat4_mul(proj, view), np.array([proj[0, 0], proj[1, 1]], np.float32)


def build_scenes() -> dict:
    """name -> scene dict (records, view, proj, projview, focal, width,
    height, sh_degree, ent_idx, transforms, gen)."""
    from oracle import oracle as O
    from tests import kat

    scenes = {}

    def add(name, recs, eye, w, h, sh=3, ent_idx=None, transforms=None, gen=None):
        view, proj, pv, focal = _camera(eye, w, h)
        scenes[name] = dict(records=np.ascontiguousarray(recs, np.float32), view=view, proj=proj, projview=pv,
                            focal=focal, width=w, height=h, sh_degree=sh, ent_idx=ent_idx, transforms=transforms,
                            gen=gen)

    add("cfg0", O.synthetic_records(0, 10_000, 0.0), (0.0, 0.0, -5.0), 256, 256, gen=(0, 10_000, 0.0))
    add("cfg1_patch", O.synthetic_records(1, 20_000, 3.0), (0.0, 0.0, -5.0), 1920, 1080, gen=(1, 20_000, 3.0))
    sub = O.synthetic_records(0, 2_000, 0.0)
    for deg in (0, 1, 2):
        add(f"sh_degree_{deg}", sub, (0.0, 0.0, -5.0), 128, 96, sh=deg, gen=(0, 2_000, 0.0))
    ent = (np.arange(6_000) % 3).astype(np.uint32)
    c, s = np.cos(0.3), np.sin(0.3)
    tr = np.stack([np.eye(4, dtype=np.float32),
                   np.array([[c, 0, s, 0.2], [0, 1, 0, -0.1], [-s, 0, c, 0.4], [0, 0, 0, 1]], np.float32),
                   np.array([[1, 0, 0, 0], [0, 1, 0, -1.0], [0, 0, 1, -0.5], [0, 0, 0, 1]], np.float32)])
    add("entities", O.synthetic_records(0, 6_000, 0.0), (1.0, -0.5, -4.5), 320, 240, ent_idx=ent,
        transforms=tr.reshape(3, 16), gen=(0, 6_000, 0.0))
    for name in ("single_isotropic", "two_depths", "culled", "tile_edge", "screen_filling", "tiny_view",
                 "thin_rotated", "wide_row", "rect_edge_x", "rect_edge_y"):
        out = getattr(kat, name)()
        recs, cam = out[0], out[1]
        eye = _eye_of(cam)
        add(name, recs, eye, cam.width, cam.height)
    for k in range(1, 16):
        recs, cam = kat.sh_probe(k)
        add(f"sh_probe_{k}", recs, _eye_of(cam), cam.width, cam.height)
    return scenes


def _eye_of(cam) -> tuple:
    """The eye of a camera looking at the origin: -R^T t of its view matrix."""
    v = np.asarray(cam.view, np.float64)
    return tuple(float(x) for x in -v[:3, :3].T @ v[:3, 3])


def load_fixture() -> dict:
    """name -> dict of the recorded inputs and outputs."""
    z = np.load(FIXTURE, allow_pickle=False)
    out = {}
    for name in z["scenes"]:
        name = str(name)
        d = {k.split("/", 1)[1]: z[k] for k in z.files if k.startswith(name + "/")}
        meta = d.pop("meta")
        d.update(width=int(meta[0]), height=int(meta[1]), sh_degree=int(meta[2]), K=int(meta[3]),
                 passes=int(meta[4]), n=int(meta[5]))
        if "gen" in d:
            from oracle import oracle as O

            seed, n, box = d["gen"]
            d["records"] = O.synthetic_records(int(seed), int(n), float(box))
        out[name] = d
    return out
