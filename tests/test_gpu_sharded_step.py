"""The engine's batched training step sharded by view over two ranks (gloo;
both ranks share the one GPU, and they exchange nothing but host buffers):
the parameters are broadcast from rank 0 once, each rank runs its views
through GaussianEngine.step_async, one all-reduce of the flattened gradients
sums them, and every rank ends with the gradient of the whole batch computed
by one engine in one process (within float-atomic reordering)."""
import os
import socket

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 30_000


def _cams():
    import torpedo_gb300 as T
    from torpedo_gb300 import configs

    eyes = configs.fibonacci_sphere(6)
    sizes = [(320, 240), (256, 144), (384, 216), (320, 240), (200, 128), (256, 256)]
    return [T.Camera.orbit(tuple(float(x) for x in eyes[i]), *sizes[i]) for i in range(6)]


def _inputs(torch, dev):
    from torpedo_gb300 import configs

    sc = configs.scene("cfg3", N)
    params = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in
              (sc.means, sc.log_scales, sc.quats, sc.opacity_logits, sc.sh)]
    pixels = sum(c.width * c.height for c in _cams())
    dimg = torch.from_numpy(np.random.default_rng(6).normal(size=pixels * 3).astype(np.float32))
    return params, dimg


def _rank_main(rank, world, port, out_dir):
    import torch
    import torch.distributed as dist

    from torpedo_gb300.sharding import ShardedStep

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    dev = torch.device("cuda", 0)
    params, dimg = _inputs(torch, dev)
    if rank != 0:  # rank 0's parameters are broadcast at construction
        params = [torch.zeros_like(p) for p in params]
    step = ShardedStep(_cams(), params, blend_persistent=True)
    grads = step.step(dimg)
    np.savez(os.path.join(out_dir, f"rank{rank}.npz"), *[g.cpu().numpy() for g in grads],
             views=np.array([len(step.mine)]))
    step.close()
    dist.barrier()
    dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_sharded_step_equals_unsharded(cuda, tmp_path):
    torch = cuda
    import torch.multiprocessing as mp

    import torpedo_gb300 as T

    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    dev = torch.device("cuda", 0)
    params, dimg = _inputs(torch, dev)
    eng = T.GaussianEngine(blend_persistent=True)
    eng.compile_params(*params)
    eng.set_views(_cams())
    eng.raster_frame()
    grads = [torch.empty_like(p) for p in params]
    eng.step_async(dimg.to(dev), grads, 1)
    eng.sync()
    eng.close()
    ref = [g.cpu().numpy().astype(np.float64) for g in grads]
    outs = [np.load(tmp_path / f"rank{r}.npz") for r in range(world)]
    assert sum(int(o["views"][0]) for o in outs) == 6 and all(int(o["views"][0]) > 0 for o in outs)
    for o in outs:
        for k, b in enumerate(ref):
            a = o[f"arr_{k}"].astype(np.float64)
            scale = np.abs(b).max() + 1e-12
            assert np.abs(a - b).max() <= 1e-4 * scale, k
