"""Tolerances of the parity tests, stated once.

Preprocess (Splat fields) must agree to relative error 1e-5, where "relative"
divides by a per-field scale so that values near zero are compared against the
quantity they belong to:
  colour r, g, b      max(|ref|, 1)
  px, py              max(|ref|, image width / height)
  viewZ               |ref|
  conic x, y, z       max(|conic.x|, |conic.z|) of the same Gaussian
  opacity             |ref| (copied, expected exact)
Tile counts and radii are exact except for Gaussians the FP64 oracle flags as
lying within a small window of a tile edge / ceil / culling threshold.
Images: max-abs error <= 1e-3 per channel against the FP64 oracle, outside the
pixels the oracle flags as deciding alpha / skip / early stop near a threshold.
Gradients: relative error <= 1e-3 against the FP64 oracle's analytic gradient.
Sort order, key arrays and tile ranges: bit-exact.
"""
import numpy as np

PREPROCESS_REL = 1e-5
IMAGE_ABS = 1e-3
GRAD_REL = 1e-3


def splat_rel_error(a32: np.ndarray, b64: np.ndarray, width: int, height: int) -> np.ndarray:
    """Per-Gaussian, per-field scaled error between float32 splats a32 (n, 12 as float32 view)
    and float64 reference splats b64 (n, 12); columns 3 (tiles) and 7 (radius) are returned as 0."""
    a = a32.astype(np.float64)
    b = b64
    scale = np.ones_like(b)
    scale[:, 0:3] = np.maximum(np.abs(b[:, 0:3]), 1.0)
    scale[:, 4] = np.maximum(np.abs(b[:, 4]), width)
    scale[:, 5] = np.maximum(np.abs(b[:, 5]), height)
    scale[:, 6] = np.maximum(np.abs(b[:, 6]), 1e-30)
    cs = np.maximum(np.abs(b[:, 8]), np.abs(b[:, 10]))
    scale[:, 8:11] = np.maximum(cs, 1e-30)[:, None]
    scale[:, 11] = np.maximum(np.abs(b[:, 11]), 1e-30)
    err = np.abs(a - b) / scale
    err[:, 3] = 0
    err[:, 7] = 0
    return err
