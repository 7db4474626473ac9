"""The serving loop (nbvh_server_*) on the GPU.

* Every query request's hits are bit-identical alone (the handle's own nbvh_query_closest_neural_host)
  and in the mix: several client threads submitting uneven requests against two resident models,
  merged into shared batches, padded to graph buckets and replayed from captured CUDA graphs,
  including a request larger than a slot (split across batches).
* A render request equals nbvh_render_path alone; when its samples are split across batches the
  image equals the unsplit one up to float summation order (relative 1e-5).
* The server reports request latency percentiles and merged batches.
* A query-lane slot (queries only, highest stream priority) answers queries submitted beside
  renders with the same hits.
"""

import threading

import numpy as np
import pytest

import nbvh_gb300 as nb
from helpers import handle
from nbvh_gb300 import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def models(built):
    h1, s1 = handle(kind="sphere4k", seed=1, depth=6)
    h1.run_optimisation(200)
    h2, s2 = handle(kind="terrain32k", seed=2, depth=8)
    h2.run_optimisation(200)
    yield [(h1, s1), (h2, s2)]
    h1.close()
    h2.close()


def _requests(models, seed=0):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(24):
        m = k % 2
        n = int(rng.choice([1, 100, 3000, 20000, 70000]))
        bbox = models[m][1]["bbox"]
        out.append((m, scenes.uniform_rays(n, bbox[:3], bbox[3:], seed=1000 + k), 1 + (k % 3 == 0)))
    # one request larger than a slot (capacity 2^16 below)
    bbox = models[0][1]["bbox"]
    out.append((0, scenes.uniform_rays(150000, bbox[:3], bbox[3:], seed=99), 1))
    return out


def test_queries_same_alone_and_in_mix(models):
    reqs = _requests(models)
    alone = [models[m][0].query_closest_neural_host(r, depth=d) for m, r, d in reqs]
    srv = nb.Server(n_slots=3, hbm_budget_gb=0.2, max_batch_rays=1 << 16)
    try:
        ids = [srv.add_model(h) for h, _ in models]
        assert srv.stats().slot_capacity_rays == 1 << 16
        results = [None] * len(reqs)

        def client(idx):
            tickets = [(i, srv.submit_query(ids[reqs[i][0]], reqs[i][1], reqs[i][2])) for i in idx]
            for i, t in tickets:
                results[i] = srv.wait(t)

        threads = [threading.Thread(target=client, args=(list(range(c, len(reqs), 4)),)) for c in range(4)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        for i, (hits, res) in enumerate(results):
            assert res.status == 0 and res.rays_traced == len(reqs[i][1])
            assert np.array_equal(hits.view(np.uint32), alone[i].view(np.uint32)), i
        # a second round replays the captured graphs
        again = [srv.wait(srv.submit_query(ids[m], r, d))[0] for m, r, d in reqs[:6]]
        for i, hits in enumerate(again):
            assert np.array_equal(hits.view(np.uint32), alone[i].view(np.uint32)), i
        st = srv.stats()
        assert st.requests_done == len(reqs) + 6
        assert 0 < st.p50_ms <= st.p99_ms <= st.max_ms
        assert st.batches >= 1
        assert st.graphs_captured >= 1 and st.graph_replays >= 1
    finally:
        srv.close()


def test_render_same_alone_and_split(models):
    h, s = models[0]
    org, tgt, up = scenes.orbit_camera(s["bbox"][:3], s["bbox"][3:], seed=9)
    cam = nb.render_request(64, 48, org, tgt, up, 45.0, sample_idx=1, sample_offset=2)
    req = nb.path_request(cam, spp=6, max_bounces=3, seed=4, ground_height=float(s["bbox"][1]) - 0.01)
    alone, traced = h.render_path(req)
    alone = alone.cpu().numpy()
    srv = nb.Server(n_slots=2, hbm_budget_gb=0.2, max_batch_rays=1 << 16)
    try:
        mid = srv.add_model(h)
        img, res = srv.wait(srv.submit_render(mid, req))
        assert res.status == 0 and res.rays_traced == traced
        np.testing.assert_array_equal(img, alone)
    finally:
        srv.close()
    # a slot of 2^12 paths holds 1 sample of 64 x 48: six chunks, averaged on the host
    srv = nb.Server(n_slots=2, hbm_budget_gb=0.02, max_batch_rays=1 << 12, autotune=False)
    try:
        mid = srv.add_model(h)
        img, res = srv.wait(srv.submit_render(mid, req))
        assert res.status == 0 and res.rays_traced == traced
        np.testing.assert_allclose(img, alone, rtol=1e-5, atol=1e-6)
    finally:
        srv.close()


def test_query_lane_same_results_beside_renders(models):
    """A server with one query-lane slot (highest stream priority, queries only) and two render
    slots: query hits submitted while renders run equal the handle's own, page-locked caller-owned
    hit buffers included, and every render equals nbvh_render_path alone."""
    import torch
    h, s = models[0]
    reqs = _requests(models, seed=5)[:8]
    alone = [models[m][0].query_closest_neural_host(r, depth=d) for m, r, d in reqs]
    org, tgt, up = scenes.orbit_camera(s["bbox"][:3], s["bbox"][3:], seed=11)
    cam = nb.render_request(96, 64, org, tgt, up, 45.0, sample_idx=3)
    preq = nb.path_request(cam, spp=2, max_bounces=2, seed=8, ground_height=float(s["bbox"][1]) - 0.01)
    ref_img, ref_traced = h.render_path(preq)
    ref_img = ref_img.cpu().numpy()
    srv = nb.Server(n_slots=3, query_slots=1, hbm_budget_gb=0.3, max_batch_rays=1 << 16)
    try:
        ids = [srv.add_model(hh) for hh, _ in models]
        renders = [srv.submit_render(ids[0], preq) for _ in range(6)]
        tickets = []
        for i, (m, r, d) in enumerate(reqs):
            out = None
            if i % 2 == 0:  # caller-owned page-locked output
                out = torch.empty(len(r) * 12, dtype=torch.int32).pin_memory().numpy().view(nb.NEURAL_HIT_DTYPE)
            tickets.append(srv.submit_query(ids[m], r, d, hits=out))
        for i, t in enumerate(tickets):
            hits, res = srv.wait(t)
            assert res.status == 0
            assert np.array_equal(hits.view(np.uint32), alone[i].view(np.uint32)), i
        for t in renders:
            img, res = srv.wait(t)
            assert res.status == 0 and res.rays_traced == ref_traced
            np.testing.assert_array_equal(img, ref_img)
    finally:
        srv.close()


def test_budget_too_small_is_refused(built):
    with pytest.raises(nb.NBVHError):
        nb.Server(n_slots=4, hbm_budget_gb=1e-4)


def test_model_changed_between_requests(built):
    h, s = handle(kind="sphere4k", seed=3, depth=5)
    h.run_optimisation(50)
    rays = scenes.uniform_rays(5000, s["bbox"][:3], s["bbox"][3:], seed=7)
    srv = nb.Server(n_slots=2, hbm_budget_gb=0.1, max_batch_rays=1 << 14)
    try:
        mid = srv.add_model(h)
        first = srv.wait(srv.submit_query(mid, rays))[0]
        assert np.array_equal(first.view(np.uint32), h.query_closest_neural_host(rays).view(np.uint32))
        # a deeper cut (new node arrays) and a learned cut grown by training: the slots drop the
        # graphs that hold the old arrays and answer like the handle itself
        h.build_neural_cut(9)
        after = srv.wait(srv.submit_query(mid, rays))[0]
        assert np.array_equal(after.view(np.uint32), h.query_closest_neural_host(rays).view(np.uint32))
        h.begin_tree_cut(nb.tree_cut_options(splitting_interval=5, last_split_iteration=40), 2)
        h.run_optimisation(45)
        learned = srv.wait(srv.submit_query(mid, rays))[0]
        assert np.array_equal(learned.view(np.uint32), h.query_closest_neural_host(rays).view(np.uint32))
        assert not np.array_equal(learned.view(np.uint32), after.view(np.uint32))
    finally:
        srv.close()
        h.close()
