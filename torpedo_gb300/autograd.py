"""torch.autograd.Function over the engine's forward and hand-written backward.

The reference has no differentiable path (its differential/ module is an
empty placeholder). Forward: raw parameters -> records on the device ->
preprocess / scan / keygen / sort / ranges / blend. Backward: the blend
adjoint (reverse per-tile traversal recomputing transmittance from the final
T) and the preprocess adjoint down to means, log-scales, quaternions,
opacity logits and SH coefficients, all in libtpdsplat.

The engine keeps the forward's lists and per-pixel state until the next
frame, so one engine serves one forward/backward pair at a time.
"""
from __future__ import annotations

import torch

from .engine import Camera, GaussianEngine


class RasterizeGaussians(torch.autograd.Function):
    @staticmethod
    def forward(ctx, means, log_scales, quats, opacity_logits, sh, engine: GaussianEngine, cams: list):
        tensors = [t.detach().contiguous().float() for t in (means, log_scales, quats, opacity_logits, sh)]
        torch.cuda.current_stream(means.device).synchronize()
        engine.compile_params(*tensors)
        if len(cams) == 1:
            engine.set_camera(cams[0])
        else:
            engine.set_views(cams)
        engine.raster_frame()
        out = torch.empty(engine.pixels * 3, dtype=torch.float32, device=means.device)
        engine.read_image_device(out)
        ctx.engine = engine
        ctx.n = means.shape[0]
        return out

    @staticmethod
    def backward(ctx, grad_out):
        g = ctx.engine.backward(grad_out.contiguous().float())
        return g[0], g[1], g[2], g[3], g[4], None, None


def rasterize(means, log_scales, quats, opacity_logits, sh, engine: GaussianEngine, cams: list[Camera]):
    """Packed HWC RGB images of all views (pixels * 3 floats), differentiable w.r.t. the raw parameters."""
    return RasterizeGaussians.apply(means, log_scales, quats, opacity_logits, sh, engine, cams)
