"""Pins the C oracle to the golden vectors of the independent Python restatement
(tests/golden/pyref.py -> golden.npz): RNG, sin/cos, classic closest/any hit, neural segments,
hash-grid features (2, 4 and 8 per entry), the network forward, Adam, the whole neural query,
training rays with their labels, a path-traced frame, LocalT decode and the composite-loss
terms."""

import ctypes as C
import os

import numpy as np
import pytest

from oracle.bindings import Network

G = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden.npz"))


def test_rng_streams(oracle):
    for seed, stream in zip(G["rng_seeds"], G["rng_streams"]):
        got = oracle.lcg_stream(int(seed[0]), int(seed[1]), int(seed[2]), 6)
        assert np.array_equal(got.view(np.uint32), stream.view(np.uint32))


def test_sincos(oracle):
    for u, (s, c) in zip(G["sincos_u"], G["sincos"]):
        gs, gc = oracle.sincos_turns(float(u))
        assert abs(gs - s) <= 1e-7 and abs(gc - c) <= 1e-7
        assert abs(gs - np.sin(2 * np.pi * float(u))) < 2e-7
        assert abs(gc - np.cos(2 * np.pi * float(u))) < 2e-7


def test_classic(oracle):
    cs = oracle.classic_scene(G["bvh_nodes"], G["bvh_prims"], G["mesh_v"], G["mesh_f"])
    assert np.array_equal(oracle.classic_query(cs, G["classic_rays"]), G["classic_hits"])
    assert np.array_equal(oracle.classic_query(cs, G["classic_rays"], any_hit=True), G["any_hits"])
    assert (G["classic_hits"][:, 3] != 0xFFFFFFFF).sum() > 30


def test_neural_segments(oracle):
    import nbvh_gb300 as nb
    consts = oracle.neural_consts(nb.default_config())
    segs, counts = oracle.neural_segments(G["neural_nodes"], consts, G["neural_rays"], 32)
    assert np.array_equal(counts, G["neural_counts"])
    for i, c in enumerate(counts):
        assert np.array_equal(segs[i, :c, :3], G["neural_segments"][i, :c, :3])
    assert counts.max() >= 2


def test_grid_features(oracle):
    off, size, res, scl = G["grid_offsets"], G["grid_sizes"], G["grid_res"], G["grid_scale"]
    g16 = np.ascontiguousarray(G["grid_values"].astype(np.float16).view(np.uint16))
    w16 = np.zeros(16, np.uint16)
    net = Network()
    net.n_levels, net.n_points, net.n_inputs, net.n_neurons, net.n_hidden_layers = 4, 1, 8, 64, 1
    keep = [off, size, res, scl, g16, w16]
    net.level_offset, net.level_size = off.ctypes.data, size.ctypes.data
    net.level_resolution, net.level_scale = res.ctypes.data, scl.ctypes.data
    net.grid_f16, net.weights_f16 = g16.ctypes.data, w16.ctypes.data
    feats = oracle.encode(net, G["grid_points"].reshape(-1, 1, 3))
    assert np.array_equal(feats.view(np.uint32), G["grid_features"].view(np.uint32))
    del keep


@pytest.mark.parametrize("nf", [4, 8])
def test_grid_features_wide(oracle, nf):
    """4 and 8 FP16 features per table entry: feature k of every corner accumulated in corner order."""
    off, size, res, scl = G["grid_offsets"], G["grid_sizes"], G["grid_res"], G["grid_scale"]
    g16 = np.ascontiguousarray(G["grid_values_f%d" % nf].astype(np.float16).view(np.uint16))
    w16 = np.zeros(16, np.uint16)
    net = Network()
    net.n_levels, net.n_points, net.n_inputs, net.n_neurons, net.n_hidden_layers = 4, 1, 4 * nf, 64, 1
    net.n_features = nf
    keep = [off, size, res, scl, g16, w16]
    net.level_offset, net.level_size = off.ctypes.data, size.ctypes.data
    net.level_resolution, net.level_scale = res.ctypes.data, scl.ctypes.data
    net.grid_f16, net.weights_f16 = g16.ctypes.data, w16.ctypes.data
    feats = oracle.encode(net, G["grid_points_f%d" % nf].reshape(-1, 1, 3))
    assert np.array_equal(feats.view(np.uint32), G["grid_features_f%d" % nf].view(np.uint32))
    del keep


def test_network_forward(oracle):
    """The network on encoded points: matrix layout and order, no biases, ReLU, the FP16 rounding of
    the features and of every hidden activation, the sigmoid output."""
    off, size, res, scl = G["grid_offsets"], G["grid_sizes"], G["grid_res"], G["grid_scale"]
    g16 = np.ascontiguousarray(G["grid_values"].astype(np.float16).view(np.uint16))
    w16 = np.ascontiguousarray(G["mlp_weights"])
    net = Network()
    net.n_levels, net.n_points, net.n_inputs, net.n_neurons, net.n_hidden_layers = 4, 1, 8, 64, 2
    keep = [off, size, res, scl, g16, w16]
    net.level_offset, net.level_size = off.ctypes.data, size.ctypes.data
    net.level_resolution, net.level_scale = res.ctypes.data, scl.ctypes.data
    net.grid_f16, net.weights_f16 = g16.ctypes.data, w16.ctypes.data
    out = oracle.network_inference(net, G["mlp_points"].reshape(-1, 1, 3))
    want = G["mlp_outputs"]
    # both sum the products in double in the same order; the outputs agree to the last bit
    # unless a double lands within an ulp of an FP32 / FP16 rounding boundary
    assert np.abs(out - want).max() <= 1e-6
    assert (out.view(np.uint32) == want.view(np.uint32)).mean() >= 0.99
    assert want.std() > 0.01  # the outputs are not all saturated
    del keep


def test_adam(oracle):
    """Three Adam steps across the start of the learning-rate decay, L2 term on: parameters and both
    moments bit-identical."""
    from types import SimpleNamespace
    opt = SimpleNamespace(learning_rate=1e-2, beta1=0.9, beta2=0.999, epsilon=1e-8, l2_reg=1e-3, decay_start=10,
                          decay_interval=1, decay_base=0.5)
    cfg = SimpleNamespace(optimizer=opt)
    p = G["adam_params0"].copy()
    m = np.zeros_like(p)
    v = np.zeros_like(p)
    for k in range(3):
        oracle.adam_step(p, m, v, G["adam_grads"][k], 9 + k, cfg)
    for got, key in ((p, "adam_params3"), (m, "adam_m3"), (v, "adam_v3")):
        assert np.array_equal(got.view(np.uint32), G[key].view(np.uint32)), key


def test_neural_query(oracle):
    """The whole neural closest-hit query of every ray (traversal resumed with the current depth,
    segment points, features, network, visibility threshold, LocalT, nearest hit, normal and albedo):
    all 12 record words bit-identical."""
    from oracle.bindings import NeuralConsts
    off, size, res, scl = G["grid_offsets"], G["grid_sizes"], G["grid_res"], G["grid_scale"]
    g16 = np.ascontiguousarray(G["grid_values"].astype(np.float16).view(np.uint16))
    w16 = np.ascontiguousarray(G["query_weights"])
    net = Network()
    net.n_levels, net.n_points, net.n_inputs, net.n_neurons, net.n_hidden_layers = 4, 2, 16, 64, 2
    keep = [off, size, res, scl, g16, w16]
    net.level_offset, net.level_size = off.ctypes.data, size.ctypes.data
    net.level_resolution, net.level_scale = res.ctypes.data, scl.ctypes.data
    net.grid_f16, net.weights_f16 = g16.ctypes.data, w16.ctypes.data
    c = NeuralConsts()
    c.inference_mint_epsilon, c.inference_maxt_epsilon = 1e-4, 1e-3
    c.fixed_node_dilation, c.node_extent_dilation = 1e-5, 1e-4
    c.primary_visibility_threshold = c.secondary_visibility_threshold = 0.5
    c.depth_epsilon, c.fixed_depth_epsilon = 0.2, 1e-5
    c.input_segment_points, c.segment_distribution, c.bvh_lod, c.max_traversal_steps = 2, 0, 0, 1000
    scene = oracle.neural_scene(G["neural_nodes"], G["query_scene_box"])
    hits = oracle.neural_query(scene, net, c, G["neural_rays"], depth=1)
    want = G["query_hits"]
    assert np.array_equal(hits, want), np.argwhere(hits != want)[:5]
    assert 10 < ((want[:, 8] & 1) != 0).sum() < len(want)  # hits and misses
    assert want[:, 9].max() >= 2  # rays that go on past a first segment
    del keep


@pytest.mark.parametrize("name,ratio", [("train0", 0.0), ("train1", 1.0)])
def test_training_rays(oracle, name, ratio):
    """Training rays (direction, LoD and dilation draws, origins in the scaled scene box until a leaf
    is entered, leaf-boundary resampling, segment points) and their classic labels (visibility,
    LocalT depth, geometric normal, albedo): bit-identical, with leaf-boundary sampling off and on."""
    from oracle.bindings import NeuralConsts
    c = NeuralConsts()
    c.learning_mint_epsilon, c.learning_maxt_epsilon = 1e-3, 1e-3
    c.fixed_node_dilation, c.node_extent_dilation = 1e-5, 1e-4
    c.sampling_bbox_scaling, c.leaf_boundary_sampling_ratio = 1.5, ratio
    c.input_segment_points, c.segment_distribution, c.bvh_lod, c.max_traversal_steps = 4, 0, 0, 1000
    nscene = oracle.neural_scene(G["neural_nodes"], G["query_scene_box"])
    cscene = oracle.classic_scene(G["bvh_nodes"], G["bvh_prims"], G["mesh_v"], G["mesh_f"])
    pos, tgt, nodes = oracle.training_batch(nscene, cscene, G["train_albedo"], c, 3, 4096, 96)
    assert np.array_equal(pos.view(np.uint32), G[name + "_points"].view(np.uint32))
    assert np.array_equal(tgt.view(np.uint32), G[name + "_targets"].view(np.uint32))
    assert np.array_equal(nodes, G[name + "_nodes"])
    assert 10 < (tgt[:, 0] == 1).sum() < len(tgt)  # labelled hits and misses


def test_path_trace(oracle):
    """A path-traced frame (camera jitter, neural hits, ground plane, sky, cosine bounces,
    throughput, per-pixel average) on the query's network and cut: every pixel bit-identical, and
    the same number of rays traced."""
    from oracle.bindings import NeuralConsts, PathParams
    off, size, res, scl = G["grid_offsets"], G["grid_sizes"], G["grid_res"], G["grid_scale"]
    g16 = np.ascontiguousarray(G["grid_values"].astype(np.float16).view(np.uint16))
    w16 = np.ascontiguousarray(G["query_weights"])
    net = Network()
    net.n_levels, net.n_points, net.n_inputs, net.n_neurons, net.n_hidden_layers = 4, 2, 16, 64, 2
    keep = [off, size, res, scl, g16, w16]
    net.level_offset, net.level_size = off.ctypes.data, size.ctypes.data
    net.level_resolution, net.level_scale = res.ctypes.data, scl.ctypes.data
    net.grid_f16, net.weights_f16 = g16.ctypes.data, w16.ctypes.data
    c = NeuralConsts()
    c.inference_mint_epsilon, c.inference_maxt_epsilon = 1e-4, 1e-3
    c.fixed_node_dilation, c.node_extent_dilation = 1e-5, 1e-4
    c.primary_visibility_threshold = c.secondary_visibility_threshold = 0.5
    c.depth_epsilon, c.fixed_depth_epsilon = 0.2, 1e-5
    c.input_segment_points, c.segment_distribution, c.bvh_lod, c.max_traversal_steps = 2, 0, 0, 1000
    scene = oracle.neural_scene(G["neural_nodes"], G["query_scene_box"])
    v = G["path_params"]
    pp = PathParams()
    for k in range(3):
        pp.origin[k], pp.du[k], pp.dv[k], pp.tl[k] = v[k], v[3 + k], v[6 + k], v[9 + k]
        pp.ground_albedo[k], pp.sky_zenith[k], pp.sky_horizon[k] = v[13 + k], v[16 + k], v[19 + k]
    pp.width, pp.height, pp.spp, pp.sample_base, pp.sample_offset, pp.seed = 8, 6, 2, 4, 1, 7
    pp.max_bounces, pp.has_ground, pp.ground_y = 2, 1, v[12]
    img = np.empty((48, 4), np.float32)
    traced = oracle.lib.orc_path_trace(C.byref(scene), C.byref(net), C.byref(c), C.byref(pp),
                                       C.c_void_p(img.ctypes.data), C.c_int(1))
    assert traced == int(G["path_traced"][0])
    assert np.array_equal(img[:, :3].view(np.uint32), G["path_image"].view(np.uint32))
    assert (G["path_image"].sum(1) > 0).sum() > 10  # lit pixels
    del keep


def test_decode_local_t(oracle):
    lib = oracle.lib
    # the oracle's decode is internal; exercise it through a one-segment neural query is heavy, so
    # the decode golden values are checked against the C restatement compiled into a helper
    fn = getattr(lib, "orc_decode_local_t", None)
    if fn is None:
        pytest.skip("decode helper not exported")
    fn.restype = C.c_float
    fn.argtypes = [C.c_float, C.c_float, C.c_float, C.c_int, C.c_float, C.c_float]
    for u, a, b, ref in G["decode"]:
        got = fn(float(u), float(a), float(b), int(a < 0), 0.2, 1e-5)
        assert np.float32(got).view(np.uint32) == np.float32(ref).view(np.uint32)


def test_losses(oracle):
    import nbvh_gb300 as nb
    kinds = {0: 3, 1: 1, 2: 0, 3: 5}  # golden kind index -> nbvh loss enum (L1, L2, RelativeL2, BCE)
    cfg = nb.default_config()
    for ki, t, p, loss, grad in G["losses"]:
        lc = oracle.loss_consts(cfg)
        lc.visibility_loss = kinds[int(ki)]
        pred = np.zeros((1, 16), np.float32)
        tgt = np.zeros((1, 8), np.float32)
        pred[0, 0], tgt[0, 0] = p, t
        vals, grads = oracle.composite_loss(lc, pred, tgt)
        dims = 8.0
        assert abs(vals[0, 0] * dims - loss) <= 2e-6 * max(1.0, abs(loss))
        assert abs(grads[0, 0] * dims - grad) <= 2e-6 * max(1.0, abs(grad))
