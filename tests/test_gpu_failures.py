"""Failure paths on the GPU, in forms that fault, trap or hang no GPU.

* A bounded wait that runs out: with nbvh_debug_inject_stall the tensor-core kernels wait on an
  mbarrier that nothing arrives at, under a short limit (nbvh_debug_set_wait_limit). The kernel
  gives up, lets its copies finish, frees its tensor memory and returns; the MLP, the neural query
  and the training pass report NBVH_ETIMEOUT, and afterwards the handle answers exactly as before.
* The traversal-step cap (max_traversal_steps, src/cuda/neural/path/path_module.cu:68): the rays the
  query caps carry NBVH_HIT_STEP_CAP as in the oracle, and the statistics count them.
* Neural stack overflow (include/cuda/neural/accel/neural_bvh2.cuh:282-285): a cut deeper than the
  24-entry traversal stack, imported through the .nbvh reader; the overflowing rays are flagged as
  in the oracle and counted.
* Device allocation failure (nbvh_debug_fail_allocations): NBVH_ENOMEM, then the same calls work.
"""

import ctypes as C
import os

import numpy as np
import pytest
import torch

import nbvh_gb300 as nb
from helpers import as_u32, handle
from nbvh_gb300 import abi, scenes
from test_gpu_neural import _borderline, _compare_queries, _cuda, _spread_params

pytestmark = pytest.mark.gpu


def test_bounded_wait_runs_out_and_the_handle_recovers(built):
    h, s = handle(kind="sphere4k", seed=3)
    lib = h.lib
    try:
        params = _spread_params(h, seed=2)
        g = torch.Generator(device="cuda").manual_seed(4)
        feats = (torch.rand((4096, h.layout.n_inputs), device="cuda", generator=g) * 0.2 - 0.1).half().contiguous()
        rays = _cuda(scenes.uniform_rays(1 << 14, s["bbox"][:3], s["bbox"][3:], seed=5))
        ref_mlp = h.mlp_inference(feats).cpu().numpy()
        ref_q = as_u32(h.query_closest_neural(rays))
        pos, tgt, _ = h.generate_training_batch(1, 4096)
        ref_g, ref_loss = h.compute_gradients(pos, tgt)
        ref_g = ref_g.cpu().numpy()
        assert lib.nbvh_debug_set_wait_limit(h.h, 200_000) == abi.NBVH_OK  # 0.2 ms
        assert lib.nbvh_debug_inject_stall(h.h, 1) == abi.NBVH_OK
        try:
            for call in (lambda: h.mlp_inference(feats), lambda: h.query_closest_neural(rays),
                         lambda: h.compute_gradients(pos, tgt)):
                with pytest.raises(nb.NBVHError) as e:
                    call()
                assert e.value.status == abi.NBVH_ETIMEOUT, e.value
        finally:
            lib.nbvh_debug_inject_stall(h.h, 0)
            lib.nbvh_debug_set_wait_limit(h.h, 0)
        torch.cuda.synchronize()
        assert np.array_equal(h.mlp_inference(feats).cpu().numpy(), ref_mlp)
        assert np.array_equal(as_u32(h.query_closest_neural(rays)), ref_q)
        g2, loss2 = h.compute_gradients(pos, tgt)
        assert np.allclose(g2.cpu().numpy(), ref_g, rtol=1e-4, atol=1e-9) and abs(loss2 - ref_loss) < 1e-5
        assert np.array_equal(h.params(), params)
    finally:
        h.close()


def test_step_cap_flags_and_counts(built, oracle):
    cfg = nb.default_config(max_traversal_steps=1)
    h, s = handle(cfg, kind="sphere65k", seed=1)
    try:
        s["params"] = _spread_params(h, seed=6)
        rays = scenes.uniform_rays(1 << 15, s["bbox"][:3], s["bbox"][3:], seed=8)
        got = as_u32(h.query_closest_neural(_cuda(rays)))
        net = oracle.network(h.cfg, h.layout, s["params"])
        ref = oracle.neural_query(oracle.neural_scene(s["neural"], s["bbox"]), net, oracle.neural_consts(h.cfg),
                                  rays, threads=8)
        border = _borderline(h, oracle, s, rays)
        cap_g, cap_r = (got[:, 8] & 0x4) != 0, (ref[:, 8] & 0x4) != 0  # NBVH_HIT_STEP_CAP
        assert cap_r.sum() > 1000
        assert np.all(cap_g[~border] == cap_r[~border])
        assert np.all(got[cap_g, 9] == 2)  # segments evaluated before the cap: max_traversal_steps + 1
        _compare_queries(got, ref, border)
        assert h.query_stats().step_capped == int(cap_g.sum())
    finally:
        h.close()


def _chain_cut(depth, delta=1.0 / 40):
    """A cut of `depth` interior nodes in a chain along x: interior k spans x in [0, 1 - k delta],
    its first child is a leaf on the far slab [1 - (k + 1) delta, 1 - k delta], its second the
    next interior node. A ray travelling along +x enters the near interior child first at every
    level and keeps the far leaf on the stack, so the stack grows by one per level."""
    f = lambda x: int(np.float32(x).view(np.uint32))
    nodes, idx = [], 0
    for k in range(depth):
        nodes.append([f(0), f(0), f(0), 0, f(1 - k * delta), f(1), f(1), idx + 1])
        nodes.append([f(1 - (k + 1) * delta), f(0), f(0), 8, f(1 - k * delta), f(1), f(1), 0xFFFFFFFF])
        idx += 2
    nodes.append([f(0), f(0), f(0), 8, f(1 - depth * delta), f(1), f(1), 0xFFFFFFFF])
    return np.array(nodes, np.uint32)


@pytest.mark.parametrize("depth", [23, 30])
def test_neural_stack_overflow_flags_and_counts(built, oracle, tmp_path, depth):
    h, s = handle(kind="sphere4k", seed=1)
    try:
        path = str(tmp_path / "chain.nbvh")
        nb.write_nbvh(path, _chain_cut(depth))
        h.import_neural_cut(path)
        nn, bbox = h.neural_bvh()
        params = _spread_params(h, seed=3)
        rng = np.random.default_rng(9)
        n = 4096
        rays = np.zeros((n, 8), np.float32)
        d = np.stack([np.ones(n), rng.uniform(-0.02, 0.02, n), rng.uniform(-0.02, 0.02, n)], 1)
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        rays[:, 0] = -0.5
        rays[:, 1:3] = rng.uniform(0.2, 0.8, (n, 2))
        rays[:, 3] = 1e-4
        rays[:, 4:7] = d
        rays[:, 7] = np.float32(3.4e38)
        got = as_u32(h.query_closest_neural(_cuda(rays)))
        net = oracle.network(h.cfg, h.layout, params)
        ref = oracle.neural_query(oracle.neural_scene(nn, bbox), net, oracle.neural_consts(h.cfg), rays, threads=8)
        ov_g, ov_r = (got[:, 8] & 0x8) != 0, (ref[:, 8] & 0x8) != 0
        assert np.array_equal(ov_g, ov_r)
        assert ov_r.all() if depth > 23 else not ov_r.any()
        assert h.query_stats().stack_overflow == int(ov_g.sum())
    finally:
        h.close()


def test_allocation_failure_reports_enomem(built):
    lib = nb.load_library()
    v, f = scenes.fbm_sphere(4, seed=1)
    # a handle built while every device allocation fails: the first call that allocates says so
    assert lib.nbvh_debug_fail_allocations(0) == abi.NBVH_OK
    statuses, made = [], []
    try:
        try:
            made.append(nb.NBVH(nb.default_config()))
            for step in (lambda: made[0].set_mesh(v, f), made[0].build_classic, made[0].build_neural_cut):
                step()
        except nb.NBVHError as e:
            statuses.append(e.status)
    finally:
        lib.nbvh_debug_fail_allocations(-1)
        for m in made:
            m.close()
    assert statuses == [abi.NBVH_ENOMEM]
    # a working handle whose query buffers cannot grow: NBVH_ENOMEM, then the same query works
    h, s = handle(kind="sphere4k", seed=1)
    try:
        rays = _cuda(scenes.uniform_rays(1 << 15, s["bbox"][:3], s["bbox"][3:], seed=4))
        lib.nbvh_debug_fail_allocations(0)
        try:
            with pytest.raises(nb.NBVHError) as e:
                h.query_closest_neural(rays)
            assert e.value.status == abi.NBVH_ENOMEM
        finally:
            lib.nbvh_debug_fail_allocations(-1)
        a = as_u32(h.query_closest_neural(rays))
        b = as_u32(h.query_closest_neural(rays))
        assert np.array_equal(a, b) and (a[:, 8] & 1).any()
    finally:
        h.close()
