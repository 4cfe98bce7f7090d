"""View sharding of the batched backward across two and three ranks (gloo,
CPU): each rank differentiates its share of the views with the FP64 oracle, one
all-reduce sums the per-Gaussian gradients, and the result equals the
gradient of the whole batch computed in one process."""
import os
import socket

import numpy as np
import pytest

import torpedo_gb300 as T
from torpedo_gb300 import configs
from torpedo_gb300.sharding import shard_cameras, view_shard


def test_view_shard_covers_every_view_once():
    for px in ([640 * 480, 1280 * 720, 1920 * 1080] * 7, [100] * 3, [5, 1, 1, 1, 9], [1]):
        for world in (1, 2, 3, 4, 8):
            parts = [view_shard(px, r, world) for r in range(world)]
            flat = [i for p in parts for i in p]
            assert flat == list(range(len(px)))
            if len(px) >= world * 3 and len(set(px)) == 1:
                sizes = [len(p) for p in parts]
                assert max(sizes) - min(sizes) <= 1


def _setup():
    sc = configs.scene("cfg0", 400)
    eyes = configs.fibonacci_sphere(5)
    sizes = [(48, 40), (32, 32), (64, 48), (40, 24), (32, 48)]
    cams = [T.Camera.orbit(tuple(float(x) for x in eyes[i]), *sizes[i]) for i in range(5)]
    params = [sc.means.astype(np.float64), sc.log_scales.astype(np.float64), sc.quats.astype(np.float64),
              sc.opacity_logits.astype(np.float64), sc.sh.astype(np.float64)]
    return sc, cams, params


def _view_grads(sc, cam, params, seed):
    from oracle import oracle as O

    oc = O.camera(cam.view, cam.projview(), cam.width, cam.height, focal=(cam.proj[0, 0], cam.proj[1, 1]))
    sp = O.preprocess_f32(sc.records, oc)
    offs, k = O.scan_tiles(sp)
    keys, vals = O.stable_sort(*O.keygen(sp, offs, k, cam.width, cam.height))
    rng = O.tile_ranges(keys, ((cam.width + 15) // 16) * ((cam.height + 15) // 16))
    dimg = np.random.default_rng(seed).normal(size=(cam.height, cam.width, 3))
    g, _ = O.backward_f64(params, oc, vals, rng, dimg)
    return g


def _rank_main(rank, world, port, out_dir):
    import torch
    import torch.distributed as dist

    from torpedo_gb300.sharding import allreduce_gradients

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sc, cams, params = _setup()
    mine = view_shard([c.width * c.height for c in cams], rank, world)
    assert [c.width for c in shard_cameras(cams, rank, world)] == [cams[v].width for v in mine]
    acc = [np.zeros_like(p) for p in params]
    for v in mine:
        for a, g in zip(acc, _view_grads(sc, cams[v], params, seed=v)):
            a += g.reshape(a.shape)
    tensors = [torch.from_numpy(a) for a in acc]
    allreduce_gradients(tensors)
    np.savez(os.path.join(out_dir, f"rank{rank}.npz"), *[t.numpy() for t in tensors])
    dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("world", [2, 3])
def test_sharded_backward_allreduce_equals_whole_batch(tmp_path, world):
    """World size 3 splits the five views of uneven sizes unevenly (a rank
    with one view beside ranks with two)."""
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    mp.spawn(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    sc, cams, params = _setup()
    whole = [np.zeros_like(p) for p in params]
    for v, cam in enumerate(cams):
        for a, g in zip(whole, _view_grads(sc, cam, params, seed=v)):
            a += g.reshape(a.shape)
    for r in range(world):
        got = np.load(tmp_path / f"rank{r}.npz")
        for i, w in enumerate(whole):
            np.testing.assert_allclose(got[f"arr_{i}"], w, rtol=1e-12, atol=1e-12)
