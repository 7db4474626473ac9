"""The allocation-free neural query (nbvh_query_closest_neural_noalloc) against the ordinary one.

Both entry points run the same kernels on each ray, so the tolerance is zero: every word of every
hit record must match. The comparison is made on two calls in a row, so the second call runs on
scratch that the first one left behind. The file is named to be collected last, and each test also
passes alone in a fresh process (the first call on the device does the scratch setup).
"""

import ctypes as C

import numpy as np
import pytest
import torch

from helpers import handle
from nbvh_gb300 import scenes

pytestmark = pytest.mark.gpu

MAX_RAYS = 16384  # NBVH_NOALLOC_MAX_RAYS in include/nbvh.h
NBVH_OK, NBVH_EINVAL = 0, 1


def _noalloc(h, rays, out, n=None):
    n = rays.shape[0] if n is None else n
    return h.lib.nbvh_query_closest_neural_noalloc(h.h, C.c_void_p(rays.data_ptr()), n, 1,
                                                   C.c_void_p(out.data_ptr()), None)


def _err(h):
    return h.lib.nbvh_last_error(h.h).decode()


@pytest.fixture(scope="module")
def scene(built):
    h, s = handle(kind="sphere65k", seed=1, albedo=True)
    rng = np.random.default_rng(5)
    p = h.params()
    nn = h.layout.n_network_params
    p[:nn] *= 2.5  # spread the outputs over (0, 1) so that rays both hit and miss
    p[nn:] = rng.uniform(-1.0, 1.0, p.size - nn).astype(np.float32)
    h.set_params(p)
    yield h, s
    h.close()


@pytest.mark.parametrize("n", [MAX_RAYS, 5003])
def test_noalloc_matches_ordinary_query_twice(scene, n):
    h, s = scene
    rays = torch.from_numpy(scenes.uniform_rays(n, s["bbox"][:3], s["bbox"][3:], seed=77 + n)).cuda()
    ref = h.query_closest_neural(rays, 1).cpu().numpy()
    assert (ref[:, 8] & 1).any() and not (ref[:, 8] & 1).all()
    for _ in range(2):
        out = torch.full((n, 12), -1, dtype=torch.int32, device="cuda")
        assert _noalloc(h, rays, out) == NBVH_OK, _err(h)
        np.testing.assert_array_equal(out.cpu().numpy(), ref)


def _alloc_count(h):
    c = C.c_uint64(0)
    assert h.lib.nbvh_debug_alloc_count(C.byref(c)) == NBVH_OK
    return c.value


def test_noalloc_uses_no_device_memory(built):
    """A fresh handle that has only ever answered allocation-free queries: the library's count of
    its own device allocations does not move across the calls, and no device memory goes."""
    h, s = handle(kind="sphere4k", seed=2)
    try:
        rays = torch.from_numpy(scenes.uniform_rays(MAX_RAYS, s["bbox"][:3], s["bbox"][3:], seed=9)).cuda()
        outs = [torch.empty((MAX_RAYS, 12), dtype=torch.int32, device="cuda") for _ in range(2)]
        assert _noalloc(h, rays, outs[0], n=0) == NBVH_OK  # setup call
        torch.cuda.synchronize()
        count0 = _alloc_count(h)
        free0, _ = torch.cuda.mem_get_info()
        for o in outs:
            assert _noalloc(h, rays, o) == NBVH_OK, _err(h)
        torch.cuda.synchronize()
        free1, _ = torch.cuda.mem_get_info()
        assert _alloc_count(h) == count0
        assert free0 - free1 < (1 << 20)
        np.testing.assert_array_equal(outs[0].cpu().numpy(), outs[1].cpu().numpy())
        # the ordinary query on the same handle does allocate (its buffers grow to the batch)
        h.query_closest_neural(rays, 1)
        assert _alloc_count(h) > count0
    finally:
        h.close()


def test_noalloc_rejects_batches_above_the_limit(scene):
    h, s = scene
    n = MAX_RAYS + 1
    rays = torch.from_numpy(scenes.uniform_rays(n, s["bbox"][:3], s["bbox"][3:], seed=3)).cuda()
    out = torch.full((n, 12), -7, dtype=torch.int32, device="cuda")
    assert _noalloc(h, rays, out) == NBVH_EINVAL
    assert "NBVH_NOALLOC_MAX_RAYS" in _err(h)
    assert bool((out == -7).all())


def test_noalloc_follows_the_classic_switch(scene):
    h, s = scene
    rays = torch.from_numpy(scenes.uniform_rays(4096, s["bbox"][:3], s["bbox"][3:], seed=21)).cuda()
    h.set_ignore_neural_blas(True)
    try:
        ref = h.query_closest_neural(rays, 1).cpu().numpy()
        out = torch.empty((4096, 12), dtype=torch.int32, device="cuda")
        assert _noalloc(h, rays, out) == NBVH_OK, _err(h)
    finally:
        h.set_ignore_neural_blas(False)
    np.testing.assert_array_equal(out.cpu().numpy(), ref)


def test_noalloc_deep_cut_fallback_and_non_neural_leaves(built):
    """A cut deeper than the node-sorted range (16,383 nodes: the tail takes over after step 3), a
    confidence fallback margin and non-neural leaves (both answered from the fallback list by the
    classic BLAS, on the fixed scratch): every word equals the ordinary query's."""
    import nbvh_gb300 as nb
    h, s = handle(nb.default_config(fallback_margin=0.05), kind="sphere65k", seed=1, depth=13, albedo=True)
    try:
        assert h.neural_bvh()[0].shape[0] > 8192
        rng = np.random.default_rng(6)
        p = h.params()
        nn = h.layout.n_network_params
        p[:nn] *= 2.5
        p[nn:] = rng.uniform(-1.0, 1.0, p.size - nn).astype(np.float32)
        h.set_params(p)
        nodes = h.neural_bvh()[0]
        leaves = np.where(nodes.view(np.uint32)[:, 3] != 0)[0].astype(np.uint32)
        h.set_non_neural_leaves(leaves[::7], True)
        rays = torch.from_numpy(scenes.uniform_rays(MAX_RAYS, s["bbox"][:3], s["bbox"][3:], seed=91)).cuda()
        ref = h.query_closest_neural(rays, 1).cpu().numpy()
        assert ((ref[:, 8] & 2) != 0).sum() > 100  # answered by the classic BLAS
        for _ in range(2):
            out = torch.full((MAX_RAYS, 12), -1, dtype=torch.int32, device="cuda")
            assert _noalloc(h, rays, out) == NBVH_OK, _err(h)
            np.testing.assert_array_equal(out.cpu().numpy(), ref)
    finally:
        h.close()

