"""GB300-native Gaussian-splatting compute pipeline (the hot path of ndming/torpedo's
GaussianEngine): preprocess -> tile-count scan -> key duplication -> onesweep
radix sort -> tile ranges -> alpha blend, plus a backward pass and a batched
multi-view form, as hand-written sm_103a kernels behind a C ABI (libtpdsplat).
"""
from ._lib import TpdError, load  # noqa: F401
from .engine import (  # noqa: F401
    Camera,
    GaussianEngine,
    Scene,
    TransformHost,
    key_bits_for_tiles,
    load_ply,
    look_at,
    mat4_mul,
    perspective,
    random_points,
    scan_tiles,
    sort_pairs,
    synthetic_scene,
)

__all__ = [
    "Camera", "GaussianEngine", "Scene", "TransformHost", "TpdError", "key_bits_for_tiles", "load", "load_ply",
    "look_at", "mat4_mul", "perspective", "random_points", "scan_tiles", "sort_pairs", "synthetic_scene",
]
