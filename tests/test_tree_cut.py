"""Learned tree cut (tree_cut_learning of NeuralBVHRenderer::render,
src/cuda/neural/neural_bvh_renderer.cu:196-282).

* The split schedule (BvhSplitScheduler, include/cuda/neural/utils/bvh_split_scheduler.h:13-145)
  equals the oracle's restatement and reproduces the cut the reference ships: 25,249 nodes for
  that cut's configuration, with its nodes allocated in the schedule's order (every split event
  splits pre-existing leaves in ascending index order and appends their children).
* On the GPU, each part of a training step is checked against the oracle from the device state
  before the step: node survival in the sampler (bit-exact batch, including the slots a rejected
  sample leaves unchanged), per-node loss accounting (samples and iter_alive exact, loss within
  1e-5 relative: float atomics), the heuristic maximum (bit-exact), the selection and split
  (node arrays, statistics and node map exact) and the LoD assignment.
"""

import os

import numpy as np
import pytest

import nbvh_gb300 as nb
from helpers import mesh
from oracle.bindings import SplitScheduler

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# the reference's chess configurations (bvh_split_scheduler blocks): interval, scaling
CHESS = {7: (3000, 2.0), 155: (300, 2.0), 1243: (100, 2.0), 10903: (50, 2.3), 32940: (40, 2.5),
         72814: (50, 3.2), 141511: (90, 5.0)}


def _opts(**kw):
    return nb.tree_cut_options(**kw)


@pytest.mark.parametrize("name", sorted(CHESS))
def test_schedule_matches_restatement(built, name):
    interval, scaling = CHESS[name]
    o = _opts(splitting_interval=interval, split_scaling=scaling, last_split_iteration=3000)
    splits, nodes = nb.split_schedule(o, 1, 10000)
    ref = SplitScheduler(interval, 3000, 1, scaling, 2.0)
    sched, n, total = [], 1, 0
    for it in range(10000):
        k = ref.get_bvh_splits(it)
        k = min(k, (n + 1) // 2) if k > 0 else 0
        n += 2 * k
        sched.append(k)
    assert np.array_equal(splits, np.array(sched, np.uint32))
    assert nodes == n


def test_schedule_reproduces_shipped_cut(built):
    topo = np.load(os.path.join(GOLDEN, "nbvh_chess_topology.npz"))
    count, first = topo["prim_count"], topo["first"]
    assert len(count) == 25249
    o = _opts(splitting_interval=40, split_scaling=2.5, last_split_iteration=3000)
    splits, nodes = nb.split_schedule(o, 1, 10000)
    assert nodes == len(count)
    # children are appended two by two; ordered by child index, the parents of each split event
    # ascend and already existed when the event started
    interior = np.where(count == 0)[0]
    order = np.argsort(first[interior])
    parents, children = interior[order], first[interior][order]
    assert np.array_equal(children, 1 + 2 * np.arange(len(children)))
    pos, n = 0, 1
    for k in splits[splits > 0]:
        seg = parents[pos:pos + k]
        assert np.all(np.diff(seg) > 0) and seg.max() < n
        pos += k
        n += 2 * k
    assert pos == len(parents)
    # leaves: final (1) or the coarsest LoD (8) -- one learned LoD
    assert set(np.unique(count[count > 0]).tolist()) == {1, 8}


def _node_map(classic, neural):
    """Classic node of every node of a fixed cut (walked in parallel from the roots)."""
    nmap = np.zeros(len(neural), np.uint32)
    stack = [(0, 0)]
    while stack:
        ni, ci = stack.pop()
        nmap[ni] = ci
        if neural[ni, 3] == 0:
            stack.append((neural[ni, 7], classic[ci, 7]))
            stack.append((neural[ni, 7] + 1, classic[ci, 7] + 1))
    return nmap


def _planted_stats(neural, rng, depth):
    n = len(neural)
    st = np.zeros((n, 4), np.uint32)
    leaf = neural[:, 7] == 0xFFFFFFFF
    loss = rng.permutation(np.arange(1, n + 1)).astype(np.float32) * np.float32(0.125) + np.float32(1.0)
    st[:, 0] = np.where(leaf, loss, 0).astype(np.float32).view(np.uint32)
    st[:, 1] = rng.integers(1, 5, n)
    st[:, 2] = depth
    st[:, 3] = np.where(leaf, rng.integers(8, 800, n), 0)
    return st


def _depths(neural):
    d = np.zeros(len(neural), np.uint32)
    for i in range(len(neural)):
        if neural[i, 7] != 0xFFFFFFFF and neural[i, 3] == 0:
            d[neural[i, 7]] = d[i] + 1
            d[neural[i, 7] + 1] = d[i] + 1
    return d


def test_oracle_split_keeps_a_valid_cut(built, oracle, tmp_path):
    v, f = mesh("sphere4k", 2)
    classic, _ = nb.build_bvh2_host(v, f)
    neural = nb.build_neural_cut_host(classic, 3)
    nmap = _node_map(classic, neural)
    st = _planted_stats(neural, np.random.default_rng(3), _depths(neural))
    k = 3
    mx, idx, st2 = oracle.tree_cut_decisions(neural, st, k)
    h = oracle.loss_heuristic(st2)
    cand = (neural[:, 7] == 0xFFFFFFFF) & (neural[:, 3] != 1)
    top = np.argsort(-np.where(cand, h, -np.inf))[:k]
    assert set(idx.tolist()) == set(top.tolist())
    assert np.array_equal(mx, np.sort(h[top])[::-1])
    assert np.array_equal(st2[:, 1] - st[:, 1], (neural[:, 7] == 0xFFFFFFFF).astype(np.uint32))
    nodes, st3, nm3, m = oracle.tree_cut_split(neural, st2, nmap, classic, idx, k, 6, len(classic))
    assert m == k and len(nodes) == len(neural) + 2 * k
    nb.write_nbvh(tmp_path / "c.nbvh", nodes)  # validates the tree
    mn, mxb = nb.nodes_to_float(nodes)
    cmn, cmx = nb.nodes_to_float(classic)
    assert np.array_equal(mn, cmn[nm3]) and np.array_equal(mxb, cmx[nm3])
    new = np.arange(len(neural), len(nodes))
    assert np.all(nodes[new, 3] == np.where(classic[nm3[new], 3] > 0, 1, 8))
    assert np.all(st3[new, 1] == 1) and np.all(st3[new, 3] == 0)


# ----------------------------------------------------------------------------------------------
# GPU: each part of a step against the oracle, from the device state before the step
# ----------------------------------------------------------------------------------------------

def _session(oracle, depth, batch=1 << 14, **kw):
    from helpers import handle
    cfg = nb.default_config()
    cfg.batch_size = batch
    h, s = handle(cfg)
    h.begin_tree_cut(_opts(**kw), depth)
    nscene = lambda nodes: oracle.neural_scene(nodes, s["bbox"])
    cscene = oracle.classic_scene(s["nodes"], s["prims"], s["v"], s["f"])
    consts = oracle.neural_consts(h.cfg)
    return h, s, nscene, cscene, consts


def _replay_batch(oracle, h, nscene, cscene, consts, nodes, stats, max_loss, prev, opts):
    pos, tgt, nd = oracle.training_batch_rr(nscene(nodes), cscene, None, consts, h.training_step, h.cfg.batch_size,
                                            h.cfg.batch_size, stats, max_loss, prev[0], prev[1],
                                            opts.survival_probability_scale, opts.min_rr_survival_prob, 6, True)
    return pos, tgt, nd


@pytest.mark.gpu
def test_node_survival_sampler_matches_oracle(built, oracle):
    h, s, nscene, cscene, consts = _session(oracle, 4, tree_cut_learning=0)
    o = _opts()
    n, P = h.cfg.batch_size, h.cfg.module.input_segment_points
    prev = (np.zeros((n, P, 3), np.float32), np.zeros((n, 8), np.float32))
    for step in range(3):
        nodes, stats, _ = h.tree_cut()
        info = h.tree_cut_info()
        ref = _replay_batch(oracle, h, nscene, cscene, consts, nodes, stats, info.max_node_loss, prev, o)
        h.run_optimisation(1)
        got = h.training_batch()
        assert np.array_equal(got[2], ref[2]), step
        assert np.array_equal(got[0].view(np.uint32), ref[0].view(np.uint32)), step
        assert np.array_equal(got[1].view(np.uint32), ref[1].view(np.uint32)), step
        prev = (got[0], got[1])
        if step == 0:  # max 0 and no samples yet: survival 0.005
            kept = np.mean(np.any(got[1] != 0, axis=1) | np.any(got[0] != 0, axis=(1, 2)))
            assert kept < 0.02
    h.close()


@pytest.mark.gpu
def test_loss_accounting_and_maximum(built, oracle):
    h, s, nscene, cscene, consts = _session(oracle, 5, tree_cut_learning=0)
    h.run_optimisation(2)
    nodes, before, _ = h.tree_cut()
    st = h.run_optimisation(1)
    pos, tgt, snodes, sloss = h.training_batch()
    nodes2, after, _ = h.tree_cut()
    assert np.array_equal(nodes, nodes2)
    dims = 8
    vals = np.zeros((len(sloss), dims), np.float32)
    vals[:, 0] = sloss
    ref = oracle.tree_cut_accumulate(before, vals, snodes, dims)
    leaf = nodes[:, 7] == 0xFFFFFFFF
    ref[:, 1] += leaf.astype(np.uint32)
    assert np.array_equal(after[:, 1:], ref[:, 1:])
    la, lr = after[:, 0].view(np.float32), ref[:, 0].view(np.float32)
    np.testing.assert_allclose(la, lr, rtol=1e-5, atol=1e-12)
    # the per-sample losses add up to the step's mean loss
    np.testing.assert_allclose(sloss.astype(np.float64).sum(), st.last_loss, rtol=1e-4)
    # the maximum the next step uses: the largest positive heuristic of the non-final leaves
    hv = oracle.loss_heuristic(after)
    cand = leaf & (nodes[:, 3] != 1) & (hv > 0)
    assert h.tree_cut_info().max_node_loss == hv[cand].max()
    h.close()


def _check_split_step(oracle, h, s, k, lod_before, assign_lod=None):
    nodes, stats, nmap = h.tree_cut()
    h.run_optimisation(1)
    _, _, snodes, sloss = h.training_batch()
    nodes2, stats2, nmap2 = h.tree_cut()
    n0 = len(nodes)
    # oracle from the device's accumulated losses (float atomics), the rest replayed exactly
    acc = stats.copy()
    acc[:, 0] = stats2[:n0, 0]
    acc[:, 3] = stats2[:n0, 3]
    mx, idx, st_dec = oracle.tree_cut_decisions(nodes, acc, k)
    hv = oracle.loss_heuristic(st_dec)
    pos_h = np.sort(hv[(nodes[:, 7] == 0xFFFFFFFF) & (nodes[:, 3] != 1) & (hv > 0)])[::-1]
    assert len(np.unique(pos_h[:k + 1])) == min(k + 1, len(pos_h))  # no ties at the cut-off
    ref_nodes, ref_stats, ref_map, m = oracle.tree_cut_split(nodes, st_dec, nmap, s["nodes"], idx, k, lod_before,
                                                             len(s["nodes"]))
    if assign_lod is not None:
        ref_nodes = oracle.tree_cut_assign_lod(ref_nodes, assign_lod)
    assert m > 0
    assert np.array_equal(nodes2, ref_nodes)
    assert np.array_equal(nmap2, ref_map)
    assert np.array_equal(stats2[:, 1:], ref_stats[:, 1:])
    assert np.array_equal(stats2[:, 0], ref_stats[:, 0])
    return m


@pytest.mark.gpu
def test_selection_and_split_match_oracle(built, oracle):
    h, s, *_ = _session(oracle, 3, splitting_interval=1, start_split_num=5, split_scaling=1.0,
                        split_interval_scaling=1.0, last_split_iteration=1000)
    nodes, stats, nmap = h.tree_cut()
    rng = np.random.default_rng(11)
    h.set_tree_cut_stats(_planted_stats(nodes, rng, stats[:, 2]))
    for _ in range(4):
        assert _check_split_step(oracle, h, s, 5, 6) == 5
    info = h.tree_cut_info()
    assert info.total_splits == 20 and info.n_nodes == 15 + 40
    h.close()


@pytest.mark.gpu
def test_lod_assignment_matches_oracle(built, oracle):
    h, s, *_ = _session(oracle, 2, splitting_interval=1, start_split_num=3, split_scaling=1.0,
                        split_interval_scaling=1.0, last_split_iteration=30, num_lods_learned=3)
    h.run_optimisation(20)  # LoD 6 assigned at iteration 10: the current LoD is 5 from then on
    assert h.tree_cut_info().current_learned_lod == 5
    _check_split_step(oracle, h, s, 3, 5, assign_lod=5)  # iteration 20 assigns LoD 5
    assert h.tree_cut_info().current_learned_lod == 4
    h.run_optimisation(20)
    info = h.tree_cut_info()
    assert info.learning == 0 and info.current_learned_lod == 0
    lod_nodes = np.array(info.n_lod_nodes, np.int64)
    assert np.all(np.diff(lod_nodes) <= 0) and lod_nodes[0] == info.n_nodes
    nodes, _, nmap = h.tree_cut()
    # at every LoD the leaves form a complete cut: the cut of the moment that LoD was assigned
    for lod in range(7):
        leaves, inner, stack = 0, 0, [0]
        while stack:
            i = stack.pop()
            pc, left = nodes[i, 3], nodes[i, 7]
            if (0 < pc <= 2 + lod) or left == 0xFFFFFFFF:
                leaves += 1
                continue
            inner += 1
            stack += [left, left + 1]
        assert leaves == inner + 1 and leaves == (lod_nodes[lod] + 1) // 2, lod
    assert np.all((nodes[:, 3] == 1) <= (s["nodes"][nmap, 3] > 0))
    h.close()


@pytest.mark.gpu
def test_learning_from_the_root(built, oracle, tmp_path):
    o = dict(splitting_interval=10, last_split_iteration=100, start_split_num=1, split_scaling=2.0,
             split_interval_scaling=2.0)
    h, s, *_ = _session(oracle, 0, **o)
    h.run_optimisation(120)
    info = h.tree_cut_info()
    _, expected = nb.split_schedule(_opts(**o), 1, 120)
    assert info.expected_nodes == expected
    assert info.n_nodes == expected and info.total_splits == (expected - 1) // 2
    nodes, stats, nmap = h.tree_cut()
    nb.write_nbvh(tmp_path / "learned.nbvh", nodes)  # a valid cut
    mn, mx = nb.nodes_to_float(nodes)
    cmn, cmx = nb.nodes_to_float(s["nodes"])
    assert np.array_equal(mn, cmn[nmap]) and np.array_equal(mx, cmx[nmap])
    leaf = nodes[:, 7] == 0xFFFFFFFF
    assert np.all(nodes[leaf, 3] == np.where(s["nodes"][nmap[leaf], 3] > 0, 1, 8))
    assert info.max_depth == stats[:, 2].max()
    # the host copy follows the device cut, and queries run on it
    nn, _ = h.neural_bvh()
    assert np.array_equal(nn, nodes)
    from nbvh_gb300 import scenes
    import torch
    rays = scenes.uniform_rays(1 << 12, s["bbox"][:3], s["bbox"][3:], seed=4)
    segs, counts = h.query_segments(torch.from_numpy(rays).cuda(), 16)
    ref_segs, ref_counts = oracle.neural_segments(nodes, oracle.neural_consts(h.cfg), rays, 16)
    counts = counts.cpu().numpy()
    assert np.array_equal(counts, ref_counts) and counts.sum() > 1000
    segs = segs.cpu().numpy().view(np.uint32)
    for k in range(16):
        live = counts > k
        assert np.array_equal(segs[live, k], ref_segs[live, k])
    h.close()
