"""The GPU kernels against the golden vectors of the independent Python restatement
(tests/golden/pyref.py, the vectors that also pin the C oracle bit for bit), on the same mesh and
depth-4 cut:

* the neural query with a 4-level hash grid (2 features, 256-entry tables), 2 points per segment, a
  2-hidden-layer FP16 network and the default constants, on the same 120 rays. The network runs on
  the tensor cores, which sum in another order than the restatement's double sums, so the bar is
  the query bar: hit decisions equal except on threshold-borderline rays, and t, normal and albedo
  close on rays that hit in both;
* 96 training rows of step 3 of 4,096-row batches with their classic labels, leaf-boundary sampling
  off and on: bit-identical;
* hash-grid features of the 4-level grid with 2, 4 and 8 features per entry: bit-identical."""

import os

import numpy as np
import pytest
import torch

import nbvh_gb300 as nb

pytestmark = pytest.mark.gpu

G = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden.npz"))


def test_neural_query_against_the_restatement(built):
    cfg = nb.default_config(**{"hashgrid.n_levels": 4, "hashgrid.n_features_per_level": 2,
                               "hashgrid.log2_hashmap_size": 8, "hashgrid.base_resolution": 4,
                               "hashgrid.per_level_scale": 2.0, "network.n_hidden_layers": 2,
                               "module.input_segment_points": 2, "module.segment_distribution": 0})
    with nb.NBVH(cfg) as h:
        h.set_mesh(G["mesh_v"], G["mesh_f"])
        h.build_classic()
        h.build_neural_cut(4)
        nodes, bbox = h.neural_bvh()
        # the handle holds the restatement's cut, scene box and grid geometry
        assert np.array_equal(nodes, G["neural_nodes"])
        assert np.array_equal(bbox.view(np.uint32), G["query_scene_box"].view(np.uint32))
        L = h.layout
        nl = L.n_levels
        assert list(L.level_offset[:nl]) == list(G["grid_offsets"]) and list(L.level_size[:nl]) == list(G["grid_sizes"])
        assert list(L.level_resolution[:nl]) == list(G["grid_res"])
        assert np.array_equal(np.array(L.level_scale[:nl], np.float32), G["grid_scale"])
        w = G["query_weights"].view(np.float16).astype(np.float32)
        assert L.n_network_params == len(w) and L.n_params == len(w) + G["grid_values"].size
        h.set_params(np.concatenate([w, G["grid_values"].reshape(-1)]).astype(np.float32))
        rays = torch.from_numpy(np.ascontiguousarray(G["neural_rays"])).cuda()
        got = h.query_closest_neural(rays).cpu().numpy().view(np.uint32)
    want = G["query_hits"]
    hit_got, hit_want = (got[:, 8] & 1) != 0, (want[:, 8] & 1) != 0
    assert 10 < hit_want.sum() < len(want)
    # a visibility output within the network's rounding of the threshold may go either way
    assert (hit_got != hit_want).sum() <= 2
    both = hit_got & hit_want
    tg, tw = got[both, 0].view(np.float32), want[both, 0].view(np.float32)
    close = np.abs(tg - tw) <= 1e-3 * np.maximum(np.abs(tw), 1e-2)
    assert close.mean() >= 0.97, (tg[~close], tw[~close])
    fg, fw = got[both, 1:7].view(np.float32), want[both, 1:7].view(np.float32)
    assert np.abs(fg - fw)[close].max() <= 1e-2  # normal and albedo


@pytest.mark.parametrize("name,ratio", [("train0", 0.0), ("train1", 1.0)])
def test_training_rows_against_the_restatement(built, name, ratio):
    cfg = nb.default_config(batch_size=4096, **{"bvh.leaf_boundary_sampling_ratio": ratio})
    with nb.NBVH(cfg) as h:
        h.set_mesh(G["mesh_v"], G["mesh_f"], G["train_albedo"])
        h.build_classic()
        h.build_neural_cut(4)
        assert np.array_equal(h.neural_bvh()[0], G["neural_nodes"])
        pos, tgt, nodes = h.generate_training_batch(3, 96)
        pos, tgt = pos.cpu().numpy(), tgt.cpu().numpy()
        nodes = nodes.cpu().numpy().view(np.uint32)
    assert np.array_equal(nodes, G[name + "_nodes"])
    assert np.array_equal(pos.view(np.uint32), G[name + "_points"].view(np.uint32))
    assert np.array_equal(tgt.view(np.uint32), G[name + "_targets"].view(np.uint32))


@pytest.mark.parametrize("nf", [2, 4, 8])
def test_encoding_against_the_restatement(built, nf):
    key = "" if nf == 2 else "_f%d" % nf
    pts, want = G["grid_points" + key], G["grid_features" + key]
    P = 2 if nf == 2 else 1  # 2 x 4 x 2 inputs: network inputs come in multiples of 16
    cfg = nb.default_config(**{"hashgrid.n_levels": 4, "hashgrid.n_features_per_level": nf,
                               "hashgrid.log2_hashmap_size": 8, "hashgrid.base_resolution": 4,
                               "hashgrid.per_level_scale": 2.0, "module.input_segment_points": P})
    with nb.NBVH(cfg) as h:
        grid = G["grid_values" + key]
        L = h.layout
        assert L.n_grid_entries == grid.shape[0]
        h.set_params(np.concatenate([np.zeros(L.n_network_params, np.float32), grid.reshape(-1)]))
        n = len(pts) // P * P
        got = h.encode(torch.from_numpy(np.ascontiguousarray(pts[:n].reshape(-1, P, 3))).cuda()).cpu().numpy()
    assert np.array_equal(got.reshape(n, -1).view(np.uint32), want[:n].view(np.uint32))
