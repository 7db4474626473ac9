"""Host BVH2 builder and fixed neural cut (no GPU): node format and invariants of the reference
layout (include/base/accel/bvh.h:66-72, src/base/accel/bvh.cpp:133-151), leaves of 1..2
triangles, flat-box regularisation (src/cuda/cuda_backend.cpp:212-223), and the cut of
traverse_and_build_neural_bvh (src/cuda/neural/neural_bvh_renderer_accel.cpp:25-88)."""

import numpy as np
import pytest

import nbvh_gb300 as nb
from helpers import mesh
from nbvh_gb300 import scenes


def _check_bvh(nodes, prims, v, f):
    mn, mx = nb.nodes_to_float(nodes)
    cnt, off = nodes[:, 3], nodes[:, 7]
    leaf = cnt > 0
    assert np.all(cnt <= 2)
    # every primitive appears once across the leaves
    covered = np.concatenate([prims[o:o + c] for o, c in zip(off[leaf], cnt[leaf])])
    assert np.array_equal(np.sort(covered), np.arange(len(f)))
    # children adjacent and inside the parent box; depth bounded by the 32-entry stack
    depth = np.zeros(len(nodes), np.int64)
    for i in np.where(~leaf)[0]:
        for c in (off[i], off[i] + 1):
            # a flat child padded by the regularisation may stick out of its parent by 0.5e-4
            assert np.all(mn[c] >= mn[i] - 0.5e-4) and np.all(mx[c] <= mx[i] + 0.5e-4)
            depth[c] = depth[i] + 1
    assert depth.max() <= 31
    # triangle boxes inside their leaf boxes
    tri = v[f]
    for i in np.where(leaf)[0][:2000]:
        for p in prims[off[i]:off[i] + cnt[i]]:
            assert np.all(tri[p].min(0) >= mn[i]) and np.all(tri[p].max(0) <= mx[i])
    # no axis thinner than the regularisation
    assert np.all(mx - mn > 0)
    return depth


@pytest.mark.parametrize("kind", ["sphere4k", "soup64k", "terrain32k"])
def test_bvh_invariants(built, kind):
    v, f = mesh(kind, 3)
    nodes, prims = nb.build_bvh2_host(v, f)
    _check_bvh(nodes, prims, v, f)


def test_flat_boxes_are_padded(built):
    # an axis-aligned quad in the z = 0.5 plane: every node is flat in z
    v = np.array([[0, 0, 0.5], [1, 0, 0.5], [1, 1, 0.5], [0, 1, 0.5], [2, 0, 0.5], [2, 1, 0.5]], np.float32)
    f = np.array([[0, 1, 2], [0, 2, 3], [1, 4, 5], [1, 5, 2]], np.uint32)
    nodes, prims = nb.build_bvh2_host(v, f)
    mn, mx = nb.nodes_to_float(nodes)
    ext = mx[:, 2] - mn[:, 2]
    assert np.allclose(ext, 1e-4, rtol=1e-2)


def test_neural_cut(built):
    v, f = mesh("sphere65k", 1)
    nodes, prims = nb.build_bvh2_host(v, f)
    for depth in (0, 3, 10):
        nn = nb.build_neural_cut_host(nodes, depth)
        cnt, off = nn[:, 3], nn[:, 7]
        leaves = cnt > 0
        assert np.all(off[leaves] == 0xFFFFFFFF)
        assert np.all(np.isin(cnt[leaves], [1, 8]))
        assert np.all(cnt[~leaves] == 0)
        assert leaves.sum() == (len(nn) + 1) // 2
        if depth == 10:
            assert leaves.sum() == 1024 and len(nn) == 2047
        # boxes copied from the classic BVH in the reference's allocation order
        mn, mx = nb.nodes_to_float(nn)
        cmn, cmx = nb.nodes_to_float(nodes)
        assert np.array_equal(mn[0], cmn[0]) and np.array_equal(mx[0], cmx[0])
        stack = [(0, 0)]
        while stack:
            ni, ci = stack.pop()
            assert np.array_equal(mn[ni], cmn[ci]) and np.array_equal(mx[ni], cmx[ci])
            if cnt[ni] == 0:
                stack.append((off[ni], nodes[ci, 7]))
                stack.append((off[ni] + 1, nodes[ci, 7] + 1))


def test_neural_cut_final_leaves(built):
    v, f = mesh("sphere1k", 2)
    nodes, prims = nb.build_bvh2_host(v, f)
    nn = nb.build_neural_cut_host(nodes, 40)  # deeper than the tree: every leaf is a classic leaf
    leaves = nn[:, 3] > 0
    assert np.all(nn[leaves, 3] == 1) and len(nn) == len(nodes)


def test_mesh_generators_deterministic():
    a = scenes.fbm_sphere(5, seed=4)
    b = scenes.fbm_sphere(5, seed=4)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert len(scenes.fbm_sphere(7, seed=1)[1]) == 65536
    assert len(scenes.terrain(64, 32)[1]) == 64 * 32 * 2
    v, f = scenes.soup(1000, seed=1)
    assert len(f) == 1000 and v.min() >= 0 and v.max() <= 1


@pytest.mark.parametrize("kind", ["sphere262k", "soup200k", "terrain131k"])
def test_parallel_build_is_identical_to_single_thread(monkeypatch, kind):
    """Meshes of 65,536 triangles or more build on several threads (NBVH_BUILD_THREADS or the
    host's hardware threads): the top of the tree depth-first with large ranges binned in chunks,
    the subtrees concurrently, every node placed where the single-threaded build puts it. The
    nodes and the primitive order are identical for any thread count."""
    if kind == "sphere262k":
        v, f = scenes.fbm_sphere(8, seed=3)
    elif kind == "soup200k":  # overlapping random triangles: many equal-centroid and median splits
        v, f = scenes.soup(200000, seed=4)
    else:  # a height field: flat boxes, regular centroids
        v, f = scenes.terrain(256, 256, seed=5)
    monkeypatch.setenv("NBVH_BUILD_THREADS", "1")
    ref_nodes, ref_prims = nb.build_bvh2_host(v, f)
    for threads in ("2", "5", "16"):
        monkeypatch.setenv("NBVH_BUILD_THREADS", threads)
        nodes, prims = nb.build_bvh2_host(v, f)
        assert np.array_equal(nodes, ref_nodes) and np.array_equal(prims, ref_prims), threads
    _check_bvh(ref_nodes, ref_prims, v, f)
