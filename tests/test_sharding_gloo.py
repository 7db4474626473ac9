"""Ray sharding over two gloo ranks on the CPU.

Each rank answers its contiguous share of one ray batch with the CPU restatement of the classic
closest-hit query (the checker; the GPU kernel is compared with it in the gpu tests) and the shares
are checked to concatenate to the unsharded answer. The only collective is the timing reduction.
"""

import os
import socket

import numpy as np
import pytest

from nbvh_gb300.shard import max_over_ranks, shard, shard_bounds


def test_shard_bounds_cover_once():
    for n in (0, 1, 7, 1000, (1 << 22) + 3):
        for world in (1, 2, 3, 8):
            spans = [shard_bounds(n, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            for (s0, e0), (s1, _) in zip(spans, spans[1:]):
                assert e0 == s1
            sizes = [e - s for s, e in spans]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_bounds(10, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist

    import nbvh_gb300 as nb
    from nbvh_gb300 import scenes
    from oracle.bindings import Oracle

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        v, f = scenes.fbm_sphere(4, seed=3)
        nodes, prims = nb.build_bvh2_host(v, f)
        mn, mx = nb.nodes_to_float(nodes[:1])
        rays = scenes.uniform_rays(4099, mn[0], mx[0], seed=11)  # odd count: ragged shares
        orc = Oracle()
        scene = orc.classic_scene(nodes, prims, v, f)
        mine = orc.classic_query(scene, shard(rays, rank, world))
        np.save(os.path.join(out_dir, "hits_%d.npy" % rank), mine)
        worst = max_over_ranks([float(rank + 1), -float(rank)])
        np.save(os.path.join(out_dir, "max_%d.npy" % rank), np.array(worst))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_rank_shards_concatenate_to_full_query(tmp_path, oracle):
    import torch.multiprocessing as mp

    import nbvh_gb300 as nb
    from nbvh_gb300 import scenes

    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    v, f = scenes.fbm_sphere(4, seed=3)
    nodes, prims = nb.build_bvh2_host(v, f)
    mn, mx = nb.nodes_to_float(nodes[:1])
    rays = scenes.uniform_rays(4099, mn[0], mx[0], seed=11)
    full = oracle.classic_query(oracle.classic_scene(nodes, prims, v, f), rays)
    parts = [np.load(os.path.join(tmp_path, "hits_%d.npy" % r)) for r in range(world)]
    assert [len(p) for p in parts] == [2050, 2049]
    np.testing.assert_array_equal(np.concatenate(parts), full)
    for r in range(world):
        np.testing.assert_array_equal(np.load(os.path.join(tmp_path, "max_%d.npy" % r)), [2.0, 0.0])
