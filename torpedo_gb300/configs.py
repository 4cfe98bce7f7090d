"""The five synthetic workloads of the splatting pipeline (seeded; no dataset).

  cfg0  10,000 Gaussians, means ~ N(0,1)^3, one 256x256 view
  cfg1  1,000,000 Gaussians, means ~ U[-3,3]^3, one 1920x1080 view (the bench workload)
  cfg2  200,000 Gaussians as cfg0, one 800x800 view, forward + backward
  cfg3  500,000 Gaussians as cfg0, 64 views on a sphere of radius 5, sizes drawn
        from {640x480, 1280x720, 1920x1080} (seed 3), forward + backward batched
  cfg4  6,000,000 Gaussians, means ~ U[-10,10]^3, 8 views at 3840x2160

Shared by all: log-scales ~ N(-4, 0.5), unit quaternions from normalised
N(0,1)^4, opacity = sigmoid(N(0,1)), 48 SH coefficients ~ N(0, 0.2), SH
degree 3; cameras look at the origin with up (0, -1, 0), vertical FOV 60
degrees, near 0.2, far 100, 16x16 tiles. The scene seed is the config index.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .engine import Camera, Scene, synthetic_scene

FOV = 60.0
NEAR = 0.2
FAR = 100.0
UP = (0.0, -1.0, 0.0)


@dataclass(frozen=True)
class Config:
    name: str
    n: int
    mean_box: float
    views: int
    sizes: tuple
    backward: bool


CONFIGS = {
    "cfg0": Config("cfg0", 10_000, 0.0, 1, ((256, 256),), False),
    "cfg1": Config("cfg1", 1_000_000, 3.0, 1, ((1920, 1080),), False),
    "cfg2": Config("cfg2", 200_000, 0.0, 1, ((800, 800),), True),
    "cfg3": Config("cfg3", 500_000, 0.0, 64, ((640, 480), (1280, 720), (1920, 1080)), True),
    "cfg4": Config("cfg4", 6_000_000, 10.0, 8, ((3840, 2160),), True),
}


def fibonacci_sphere(count: int, radius: float = 5.0) -> np.ndarray:
    """count points on a sphere (golden-angle spiral), used as camera eyes."""
    golden = math.pi * (3.0 - math.sqrt(5.0))
    pts = []
    for i in range(count):
        y = 1.0 - 2.0 * (i + 0.5) / count
        r = math.sqrt(max(0.0, 1.0 - y * y))
        phi = i * golden
        pts.append((radius * r * math.cos(phi), radius * y, radius * r * math.sin(phi)))
    return np.asarray(pts, np.float32)


def cameras(cfg: Config | str) -> list[Camera]:
    cfg = CONFIGS[cfg] if isinstance(cfg, str) else cfg
    if cfg.views == 1:
        w, h = cfg.sizes[0]
        return [Camera.orbit((0.0, 0.0, -5.0), w, h, up=UP, fov_y_degrees=FOV, near=NEAR, far=FAR)]
    eyes = fibonacci_sphere(cfg.views)
    rng = np.random.default_rng(3)
    picks = rng.integers(0, len(cfg.sizes), size=cfg.views)
    return [Camera.orbit(tuple(float(x) for x in eyes[i]), *cfg.sizes[int(picks[i])], up=UP, fov_y_degrees=FOV,
                         near=NEAR, far=FAR) for i in range(cfg.views)]


def scene(cfg: Config | str, n: int | None = None) -> Scene:
    cfg = CONFIGS[cfg] if isinstance(cfg, str) else cfg
    seed = int(cfg.name[3:])
    return synthetic_scene(seed, n if n is not None else cfg.n, cfg.mean_box)
