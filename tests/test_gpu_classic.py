"""K1 classic closest-hit / any-hit on the GPU against the CPU restatement of
CudaBVH2::intersect + BaseCudaBLAS::intersect_triangle (include/cuda/accel/bvh2.cuh:12-88,
include/cuda/accel/bvh.cuh:98-136): prim, t, u and v must be bit-identical on the same BVH, and the
FP32 answer agrees with the FP64 Moller-Trumbore adjudicator except on grazing/tie rays."""

import numpy as np
import pytest
import torch

from helpers import as_u32, handle
from nbvh_gb300 import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scene(built):
    h, s = handle(kind="sphere65k", seed=1)
    yield h, s
    h.close()


def _cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_uniform_rays_bit_exact(scene, oracle):
    h, s = scene
    rays = scenes.uniform_rays(1 << 16, s["bbox"][:3], s["bbox"][3:], seed=11)
    got = as_u32(h.query_closest_classic(_cuda(rays)))
    cs = oracle.classic_scene(s["nodes"], s["prims"], s["v"], s["f"])
    ref = oracle.classic_query(cs, rays, threads=8)
    assert np.array_equal(got, ref)
    assert (ref[:, 3] != 0xFFFFFFFF).mean() > 0.1


def test_camera_and_bounce_rays_bit_exact(scene, oracle):
    """512 x 512 pinhole primary rays from a seeded orbit camera plus one cosine-sampled bounce
    per hit (the classic closest-hit workload)."""
    h, s = scene
    org, tgt, up = scenes.orbit_camera(s["bbox"][:3], s["bbox"][3:], seed=4)
    prim_rays = scenes.camera_rays(512, 512, org, tgt, up, seed=4)
    cs = oracle.classic_scene(s["nodes"], s["prims"], s["v"], s["f"])
    got = as_u32(h.query_closest_classic(_cuda(prim_rays)))
    ref = oracle.classic_query(cs, prim_rays, threads=8)
    assert np.array_equal(got, ref)
    bounce = scenes.bounce_rays(prim_rays, got, s["v"], s["f"], seed=4)
    assert len(bounce) > 10000
    got_b = as_u32(h.query_closest_classic(_cuda(bounce)))
    ref_b = oracle.classic_query(cs, bounce, threads=8)
    assert np.array_equal(got_b, ref_b)


def test_any_hit_bit_exact(scene, oracle):
    h, s = scene
    rays = scenes.uniform_rays(1 << 14, s["bbox"][:3], s["bbox"][3:], seed=12)
    got = as_u32(h.query_any_classic(_cuda(rays)))
    cs = oracle.classic_scene(s["nodes"], s["prims"], s["v"], s["f"])
    ref = oracle.classic_query(cs, rays, any_hit=True)
    assert np.array_equal(got, ref)
    closest = oracle.classic_query(cs, rays)
    assert np.array_equal(got[:, 3] != 0xFFFFFFFF, closest[:, 3] != 0xFFFFFFFF)


def test_fp64_adjudication(scene, oracle):
    """FP32 prim ids equal the FP64 brute force except on grazing or tied rays (<= 1e-5 of rays
    allowed without adjudication; every mismatch must be a t tie within 1e-5 relative)."""
    h, s = scene
    rays = scenes.uniform_rays(3000, s["bbox"][:3], s["bbox"][3:], seed=13)
    got = as_u32(h.query_closest_classic(_cuda(rays)))
    cs = oracle.classic_scene(s["nodes"], s["prims"], s["v"], s["f"])
    t64, p64 = oracle.fp64_closest(cs, rays)
    mism = np.where(got[:, 3] != p64)[0]
    t32 = got[:, 0].view(np.float32)
    for i in mism:
        # grazing edge or tie: both hit at the same distance, or the FP64 hit is an edge graze
        assert p64[i] == 0xFFFFFFFF or got[i, 3] == 0xFFFFFFFF or abs(t32[i] - t64[i]) <= 1e-5 * max(1.0, t64[i])
    hit = p64 != 0xFFFFFFFF
    both = hit & (got[:, 3] != 0xFFFFFFFF)
    assert np.max(np.abs(t32[both] - t64[both]) / t64[both]) < 1e-5


def test_edge_cases(scene, oracle):
    h, s = scene
    cs = oracle.classic_scene(s["nodes"], s["prims"], s["v"], s["f"])
    c = 0.5 * (s["bbox"][:3] + s["bbox"][3:])
    o = np.tile(c, (12, 1)).astype(np.float32)
    d = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1],
                  [1, 1, 0], [0, 1, 1], [1, 0, 1], [-1, -1, -1], [0.3, -0.2, 0.9], [1e-8, 1, 0]], np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = scenes.make_rays(o, d)
    rays[3, 7] = 1e-3        # short tmax
    rays[4, 3] = -1.0        # negative tmin
    rays = np.concatenate([rays, scenes.make_rays(np.array([[5, 5, 5]], np.float32),
                                                  np.array([[1, 0, 0]], np.float32))])  # misses the box
    got = as_u32(h.query_closest_classic(_cuda(rays)))
    ref = oracle.classic_query(cs, rays)
    assert np.array_equal(got, ref)
    assert ref[-1, 3] == 0xFFFFFFFF
    # empty batch
    empty = torch.empty((0, 8), dtype=torch.float32, device="cuda")
    out = h.query_closest_classic(empty)
    assert out.shape[0] == 0


def test_other_meshes_bit_exact(oracle, built):
    for kind in ("soup64k", "terrain32k"):
        h, s = handle(kind=kind, seed=2, depth=8)
        try:
            rays = scenes.uniform_rays(1 << 14, s["bbox"][:3], s["bbox"][3:], seed=21)
            got = as_u32(h.query_closest_classic(_cuda(rays)))
            cs = oracle.classic_scene(s["nodes"], s["prims"], s["v"], s["f"])
            ref = oracle.classic_query(cs, rays, threads=8)
            assert np.array_equal(got, ref), kind
        finally:
            h.close()


def test_host_pipeline_matches_device(scene):
    h, s = scene
    rays = scenes.uniform_rays(3 * (1 << 20) // 2, s["bbox"][:3], s["bbox"][3:], seed=14)
    dev = as_u32(h.query_closest_classic(_cuda(rays)))
    host = h.query_closest_classic_host(rays)
    assert np.array_equal(host.view(np.uint32).reshape(-1, 4), dev)
