"""Hand-built known-answer scenes shared by the oracle and GPU tests.

Each builder returns (records, camera) with expected values worked out by hand
from the shaders' formulas (project.slang, splat/*.slang, blend.slang)."""
from __future__ import annotations

import math

import numpy as np

import torpedo_gb300 as T

C0 = 0.28209479177387814


def rgb2sh(r, g, b):
    sh = np.zeros(48, np.float32)
    sh[0], sh[1], sh[2] = (r - 0.5) / C0, (g - 0.5) / C0, (b - 0.5) / C0
    return sh


def record(pos, opacity, scale, quat=(0, 0, 0, 1), sh=None, modifier=1.0):
    r = np.zeros(60, np.float32)
    r[0:3] = pos
    r[3] = opacity
    r[4:8] = quat
    r[8:11] = scale
    r[11] = modifier
    r[12:60] = rgb2sh(0.5, 0.5, 0.5) if sh is None else sh
    return r


def camera(w=256, h=256):
    return T.Camera.orbit((0.0, 0.0, -5.0), w, h)


def single_isotropic():
    """One isotropic Gaussian at the origin, seen from (0,0,-5): centred at pixel (127.5, 127.5)."""
    cam = camera()
    rec = record((0, 0, 0), 0.8, (0.05, 0.05, 0.05), sh=rgb2sh(0.2, 0.4, 0.6))[None]
    fy = float(cam.proj[1, 1])
    focal = 0.5 * 256 * fy
    var = (focal / 5.0) ** 2 * 0.05 ** 2 + 0.3
    # isotropic: mid^2 - det = 0, so the shader's max(0.1, .) adds sqrt(0.1) to the eigenvalue
    lam = var + math.sqrt(0.1)
    exp = dict(px=127.5, py=127.5, depth=5.0, conic=(1 / var, 0.0, 1 / var), radius=math.ceil(3 * math.sqrt(lam)),
               color=(0.2, 0.4, 0.6), var=var,
               # with the band-3 quirk (common.slang:69) the scalar C3[3]*z*(2zz-3xx-3yy) is added to
               # every channel; on the optical axis dir = (0, 0, 1) it is 2*C3[3]
               compat_shift=2 * 0.3731763325901154)
    x0 = int((127.5 - exp["radius"]) / 16)
    x1 = int((127.5 + exp["radius"] + 15) / 16)
    exp["tiles"] = (x1 - x0) * (x1 - x0)
    return rec, cam, exp


def two_depths():
    """Red in front (depth 4), blue behind (depth 6), both centred."""
    cam = camera()
    recs = np.stack([record((0, 0, 1.0), 0.5, (0.08,) * 3, sh=rgb2sh(0.0, 1.0, 1.0)),   # depth 6, index 0
                     record((0, 0, -1.0), 0.6, (0.08,) * 3, sh=rgb2sh(1.0, 0.0, 0.0))])  # depth 4, index 1
    return recs, cam


def culled():
    """Behind the camera, outside the left/right planes, beyond far: all culled."""
    cam = camera()
    recs = np.stack([record((0, 0, -6.0), 0.9, (0.1,) * 3), record((10.0, 0, 0), 0.9, (0.1,) * 3),
                     record((0, 0, 200.0), 0.9, (0.1,) * 3)])
    return recs, cam


def tile_edge():
    """Gaussians whose centre lies on tile boundaries and at image corners."""
    cam = camera()
    fy = float(cam.proj[1, 1])
    recs = []
    for px in (15.5, 16.0, 127.5, 0.0, 255.0):
        # pixel -> ndc -> world x at depth 5
        ndc = (2 * px + 1) / 256 - 1
        x = ndc * 5.0 / fy
        recs.append(record((x, x * 0.5, 0.0), 0.7, (0.03, 0.02, 0.04)))
    return np.stack(recs), cam


def sh_probe(k: int):
    """One Gaussian on the axis with a single SH feature k (1..15) set to 1 in channel 0."""
    cam = camera()
    sh = np.zeros(48, np.float32)
    sh[3 + 0 * 15 + (k - 1)] = 1.0
    rec = record((0.3, -0.2, 0.5), 0.9, (0.05,) * 3, sh=sh)[None]
    return rec, cam


def screen_filling():
    """One large opaque Gaussian just in front of the camera that covers every
    tile of a 160x96 image, with a few small ones behind and in front of it:
    one Gaussian contributes a key to all 60 tiles."""
    cam = camera(160, 96)
    recs = [record((0.0, 0.0, -3.0), 0.9, (0.6, 0.5, 0.4), quat=(0.2, 0.1, 0.0, 0.97), sh=rgb2sh(0.3, 0.6, 0.2))]
    rng = np.random.default_rng(11)
    for _ in range(40):
        z = float(rng.uniform(-3.8, 1.0))
        recs.append(record((float(rng.uniform(-1, 1)), float(rng.uniform(-0.6, 0.6)), z), float(rng.uniform(0.2, 0.9)),
                           tuple(float(v) for v in rng.uniform(0.01, 0.08, 3)),
                           sh=rgb2sh(*(float(c) for c in rng.uniform(0, 1, 3)))))
    return np.stack(recs), cam


def tiny_view():
    """The cfg0-style random scene seen through a 5x3 image: one partial tile."""
    recs = np.stack([record((float(x), float(y), float(z)), 0.7, (0.04, 0.05, 0.03), sh=rgb2sh(0.9, 0.5, 0.1))
                     for x, y, z in np.random.default_rng(12).normal(0, 0.2, (300, 3))])
    return recs, camera(5, 3)


def thin_rotated():
    """400 needle-like Gaussians (one long axis of 0.3-2 world units, the other
    two 0.002-0.01), randomly rotated, half of them with opacity just above
    1/255, over a 256x256 view: alpha >= 1/255 regions that are long, thin
    and diagonal, where a conservative per-block cull is easiest to get wrong."""
    rng = np.random.default_rng(13)
    recs = []
    for _ in range(400):
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        scale = rng.uniform(0.002, 0.01, 3)
        scale[int(rng.integers(0, 3))] = rng.uniform(0.3, 2.0)
        op = float(rng.uniform(1.0 / 255, 1.3 / 255)) if rng.random() < 0.5 else float(rng.uniform(0.3, 0.99))
        pos = (float(rng.uniform(-2.5, 2.5)), float(rng.uniform(-2.5, 2.5)), float(rng.uniform(-1.0, 1.0)))
        recs.append(record(pos, op, tuple(float(s) for s in scale), quat=tuple(float(v) for v in q),
                           sh=rgb2sh(*(float(c) for c in rng.uniform(0, 1, 3)))))
    return np.stack(recs), camera()


def wide_row():
    """A 4200x48 view (263 x 3 tiles) with one large Gaussian just in front of
    the camera whose tile rectangle spans every column, plus small ones along
    the row: rows of more than 256 consecutive tile ids, where the low tile-id
    digit wraps round all 256 values."""
    cam = camera(4200, 48)
    recs = [record((0.0, 0.0, -4.7), 0.6, (8.0, 0.4, 0.2), sh=rgb2sh(0.8, 0.3, 0.1))]
    rng = np.random.default_rng(14)
    for _ in range(60):
        recs.append(record((float(rng.uniform(-40, 40)), float(rng.uniform(-0.1, 0.1)), float(rng.uniform(-1, 1))),
                           float(rng.uniform(0.3, 0.9)), tuple(float(v) for v in rng.uniform(0.02, 0.1, 3)),
                           sh=rgb2sh(*(float(c) for c in rng.uniform(0, 1, 3)))))
    return np.stack(recs), cam


def _f32_bits(bits: int) -> float:
    return float(np.array([bits], np.uint32).view(np.float32)[0])


def _edge_scene(cam, axis: int, coord_bits: int):
    """One Gaussian placed (by a search over float positions) so that its
    centre plus radius is exactly 1009 - 2^-14 pixels along `axis`, plus 20
    ordinary ones. The shader's rect bound p + r + BLOCK - 1 adds 16 first:
    1024.99994 rounds (ties to even) to 1025, so after the - 1 the bound is
    1024 / 16 = 64, one tile more than (p + r) + 15 = 1023.99994 would give."""
    pos = [0.0, 0.0, 0.0]
    pos[axis] = _f32_bits(coord_bits)
    recs = [record(tuple(pos), 0.8, (0.004, 0.004, 0.004), sh=rgb2sh(0.9, 0.2, 0.4))]
    rng = np.random.default_rng(15 + axis)
    for _ in range(20):
        p = [0.0, 0.0, float(rng.uniform(-1, 1))]
        p[axis] = float(rng.uniform(-3, 3))
        recs.append(record(tuple(p), float(rng.uniform(0.3, 0.9)), tuple(float(v) for v in rng.uniform(0.005, 0.05, 3)),
                           sh=rgb2sh(*(float(c) for c in rng.uniform(0, 1, 3)))))
    return np.stack(recs), cam


def rect_edge_x():
    """A 2048x48 view with a Gaussian whose right tile bound comes from the
    rounding of p + r + 16 - 1 (see _edge_scene): 2 tiles, not 1."""
    return _edge_scene(camera(2048, 48), 0, 0xC006B72F)


def rect_edge_y():
    """The same along y, on a 48x2048 view: 2 tiles, not 1."""
    return _edge_scene(camera(48, 2048), 1, 0xBD612AD6)
