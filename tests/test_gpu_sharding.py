"""Ray sharding through the library: two gloo ranks, each with its own handle and CUDA context on the
same GPU, answer their contiguous shares of one ray batch with the neural query; the shares
concatenate to the unsharded answer of a third handle, word for word. The ranks' kernels never
wait on one another (the only collective is the host-side timing reduction over gloo), so sharing
one GPU between them is safe; on a multi-GPU node each rank would take its own device.
"""

import os
import socket

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _scene():
    import nbvh_gb300 as nb
    from nbvh_gb300 import scenes
    v, f = scenes.fbm_sphere(5, seed=21)
    h = nb.NBVH(nb.default_config())
    h.set_mesh(v, f)
    h.build_classic()
    h.build_neural_cut(6)
    _, bbox = h.neural_bvh()
    rays = scenes.uniform_rays(20011, bbox[:3], bbox[3:], seed=22)  # odd count: ragged shares
    return h, rays


def _rank_main(rank, world, port, out_dir):
    import torch
    import torch.distributed as dist

    from nbvh_gb300.shard import max_over_ranks, shard

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        torch.cuda.set_device(0)
        h, rays = _scene()
        mine = shard(rays, rank, world)
        hits = h.query_closest_neural(torch.from_numpy(np.ascontiguousarray(mine)).cuda())
        torch.cuda.synchronize()
        np.save(os.path.join(out_dir, "hits_%d.npy" % rank), hits.cpu().numpy())
        worst = max_over_ranks([float(len(mine))])
        np.save(os.path.join(out_dir, "max_%d.npy" % rank), np.array(worst))
        dist.barrier()
        h.close()
    finally:
        dist.destroy_process_group()


def test_two_rank_neural_shards_concatenate(built, tmp_path):
    import torch
    import torch.multiprocessing as mp

    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    h, rays = _scene()
    try:
        full = h.query_closest_neural(torch.from_numpy(rays).cuda()).cpu().numpy()
    finally:
        h.close()
    parts = [np.load(os.path.join(tmp_path, "hits_%d.npy" % r)) for r in range(world)]
    assert [len(p) for p in parts] == [10006, 10005]
    assert np.array_equal(np.concatenate(parts).view(np.uint32), full.view(np.uint32))
    assert ((full.view(np.uint32)[:, 8] & 1) != 0).sum() > 100  # some rays hit
    for r in range(world):
        np.testing.assert_array_equal(np.load(os.path.join(tmp_path, "max_%d.npy" % r)), [10006.0])
