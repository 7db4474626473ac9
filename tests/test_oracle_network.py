"""The oracle's network restatement on its own (no GPU): forward against a numpy implementation,
backward against central finite differences of its own forward (FP32 exact mode, smooth losses),
and the composite-loss masking / linear-activation rules of
include/cuda/neural/utils/pt_composite_loss.cuh:18-123."""

import numpy as np
import pytest

import nbvh_gb300 as nb


def small_cfg(**kw):
    base = {"hashgrid.n_levels": 4, "hashgrid.log2_hashmap_size": 8, "hashgrid.base_resolution": 4,
            "hashgrid.per_level_scale": 2.0, "network.n_hidden_layers": 2, "module.input_segment_points": 2}
    base.update(kw)
    return nb.default_config(**base)


def random_params(cfg, seed=0):
    L = nb.param_layout(cfg)
    rng = np.random.default_rng(seed)
    p = nb.init_params(cfg) * 2.0
    p[L.n_network_params:] = rng.uniform(-1, 1, p.size - L.n_network_params).astype(np.float32)
    return L, p


def numpy_forward(cfg, L, p, feats):
    H = cfg.network.n_hidden_layers
    off = 0
    x = feats.astype(np.float64)
    for m in range(H + 1):
        rows = 16 if m == H else 64
        cols = L.n_inputs if m == 0 else 64
        W = p[off:off + rows * cols].reshape(rows, cols).astype(np.float64)
        off += rows * cols
        x = x @ W.T
        if m < H:
            x = np.maximum(x, 0)
    return 1.0 / (1.0 + np.exp(-x))


@pytest.mark.parametrize("features", [2, 4, 8])
def test_forward_matches_numpy(oracle, built, features):
    cfg = small_cfg(**{"hashgrid.n_features_per_level": features})
    L, p = random_params(cfg)
    net = oracle.network(cfg, L, p, exact=True)
    pos = np.random.default_rng(1).uniform(0, 1, (64, 2, 3)).astype(np.float32)
    feats = oracle.encode(net, pos)
    out = oracle.network_inference(net, pos)
    ref = numpy_forward(cfg, L, p, feats)
    assert np.max(np.abs(out - ref)) < 1e-6
    # FP16 mode rounds features / activations / parameters: close but not equal
    out16 = oracle.network_inference(oracle.network(cfg, L, p), pos)
    assert 0 < np.max(np.abs(out16 - ref)) < 2e-2


@pytest.mark.parametrize("features", [4, 8])
def test_wide_entries_equal_two_feature_grids(oracle, built, features):
    """A level of F features per entry computes exactly what F / 2 grids of 2-feature entries
    compute when grid k holds features 2k and 2k + 1 of every entry: the corners, weights and
    per-feature accumulation order do not depend on F."""
    cfg = small_cfg(**{"hashgrid.n_features_per_level": features})
    L, p = random_params(cfg, seed=11)
    pos = np.random.default_rng(12).uniform(-0.2, 1.2, (257, 2, 3)).astype(np.float32)
    wide = oracle.encode(oracle.network(cfg, L, p), pos).reshape(257, 2, 4, features)
    cfg2 = small_cfg()
    L2 = nb.param_layout(cfg2)
    assert L2.n_grid_entries == L.n_grid_entries
    grid = p[L.n_network_params:].reshape(L.n_grid_entries, features)
    for k in range(features // 2):
        p2 = np.zeros(L2.n_params, np.float32)
        p2[L2.n_network_params:] = grid[:, 2 * k:2 * k + 2].reshape(-1)
        narrow = oracle.encode(oracle.network(cfg2, L2, p2), pos).reshape(257, 2, 4, 2)
        assert np.array_equal(narrow.view(np.uint32), wide[..., 2 * k:2 * k + 2].copy().view(np.uint32))


def _bf16_round(x):
    from oracle.bindings import bf16_bits
    return (bf16_bits(x).astype(np.uint32) << 16).view(np.float32)


def test_bf16_forward_matches_rounded_numpy(oracle, built):
    """BF16 mode: the network matrices, the encoded inputs and every hidden activation are rounded
    to bfloat16 (the grid table stays FP16); accumulation stays in higher precision."""
    cfg = small_cfg(**{"network.precision": 1})
    L, p = random_params(cfg, seed=3)
    net = oracle.network(cfg, L, p)
    pos = np.random.default_rng(2).uniform(0, 1, (64, 2, 3)).astype(np.float32)
    feats = oracle.encode(net, pos)
    H = cfg.network.n_hidden_layers
    x = _bf16_round(feats).astype(np.float64)
    off = 0
    for m in range(H + 1):
        rows = 16 if m == H else 64
        cols = L.n_inputs if m == 0 else 64
        W = _bf16_round(p[off:off + rows * cols]).reshape(rows, cols).astype(np.float64)
        off += rows * cols
        x = x @ W.T
        if m < H:
            x = _bf16_round(np.maximum(x, 0).astype(np.float32)).astype(np.float64)
    ref = 1.0 / (1.0 + np.exp(-x))
    out = oracle.network_inference(net, pos)
    assert np.max(np.abs(out - ref)) < 1e-5
    # and it differs from the FP16 network on the same parameters
    out16 = oracle.network_inference(oracle.network(small_cfg(), L, p), pos)
    assert np.max(np.abs(out16 - out)) > 1e-4


@pytest.mark.parametrize("features", [2, 4, 8])
def test_backward_matches_finite_differences(oracle, built, features):
    cfg = small_cfg(**{"hashgrid.n_features_per_level": features,
                       "output.visibility_loss": nb.abi.LOSS["L2"], "output.depth_loss": nb.abi.LOSS["L2"],
                       "output.normal_loss": nb.abi.LOSS["L2"], "output.albedo_loss": nb.abi.LOSS["L2"],
                       "output.visibility_masking_loss": 0, "output.output_normal_linear_activation": 0})
    L, p = random_params(cfg, seed=3)
    rng = np.random.default_rng(4)
    n = 32
    pos = rng.uniform(0.05, 0.95, (n, 2, 3)).astype(np.float32)
    tgt = rng.uniform(0, 1, (n, 8)).astype(np.float32)
    lc = oracle.loss_consts(cfg)

    def loss_at(params):
        net = oracle.network(cfg, L, params, exact=True)
        return oracle.compute_gradients(net, lc, pos, tgt, L.n_params, loss_scale=1.0, fp16_backward=False)

    g, _ = loss_at(p)
    # network weights (first, hidden, output rows 0..7) and grid entries with non-zero gradient
    cand = list(rng.choice(64 * L.n_inputs, 12, replace=False))
    cand += list(64 * L.n_inputs + rng.choice(64 * 64, 8, replace=False))
    cand += list(L.n_network_params - 16 * 64 + rng.choice(8 * 64, 8, replace=False))
    grid_nz = np.where(np.abs(g[L.n_network_params:]) > 1e-6)[0]
    cand += list(L.n_network_params + rng.choice(grid_nz, 12, replace=False))
    for i in cand:
        h = 1e-3 * max(1.0, abs(float(p[i])))
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (loss_at(pp)[1] - loss_at(pm)[1]) / (float(pp[i]) - float(pm[i]))
        assert abs(fd - g[i]) <= 2e-3 * max(abs(g[i]), 1e-3) + 1e-6, (i, fd, g[i])


def test_composite_loss_rules(oracle, built):
    cfg = nb.default_config()
    lc = oracle.loss_consts(cfg)
    pred = np.full((2, 16), 0.6, np.float32)
    tgt = np.array([[0.0, 0.3, 0.5, 0.5, 1.0, 0.2, 0.2, 0.2], [1.0, 0.3, 0.5, 0.5, 1.0, 0.2, 0.2, 0.2]], np.float32)
    vals, grads = oracle.composite_loss(lc, pred, tgt, loss_scale=1.0)
    # masked row: only visibility contributes; padding channels never do
    assert np.all(vals[0, 1:] == 0) and np.all(grads[0, 1:] == 0) and vals[0, 0] > 0
    assert np.all(vals[1, :8] != 0) and np.all(vals[:, 8:] == 0)
    # linearised-sigmoid normal: L1 on ((p*2-1)/0.1)*0.5+0.5, gradient scaled by 1/0.1
    lin = ((0.6 * 2 - 1) / 0.1) * 0.5 + 0.5
    n_total = 2 * 8
    assert abs(vals[1, 2] - abs(lin - 0.5) / n_total) < 1e-6
    assert abs(grads[1, 2] - 10.0 / n_total) < 1e-5
    # loss scale multiplies the gradient only
    v2, g2 = oracle.composite_loss(lc, pred, tgt, loss_scale=128.0)
    assert np.array_equal(v2, vals) and np.allclose(g2, grads * 128.0)


def _e4m3_table():
    """All finite FP8-E4M3 values, from their bit patterns (independent of the rounding code)."""
    vals = []
    for code in range(256):
        s, e, m = code >> 7, (code >> 3) & 0xF, code & 7
        if e == 15 and m == 7:
            continue  # NaN
        v = (m / 8.0) * 2.0 ** -6 if e == 0 else (1 + m / 8.0) * 2.0 ** (e - 7)
        vals.append((-v if s else v, m & 1))
    return vals


def _e4m3_reference(x):
    """Nearest E4M3 value, ties to the even mantissa, saturating at +-448."""
    table = _e4m3_table()
    out = np.empty_like(x)
    for i, v in enumerate(x.astype(np.float64)):
        if abs(v) >= 448.0:
            out[i] = np.copysign(448.0, v)
            continue
        d = [(abs(v - t), odd, t) for t, odd in table]
        best = min(d)[0]
        cands = [(odd, t) for dist, odd, t in d if dist == best]
        cands.sort()
        out[i] = cands[0][1] if cands[0][1] != 0 or len(cands) == 1 else np.copysign(0.0, v)
    return out


def test_e4m3_rounding_matches_the_format(oracle, built):
    rng = np.random.default_rng(8)
    x = np.concatenate([
        np.array([0.0, 1.0, 1.0625, 1.1875, 448.0, 464.0, 500.0, 1e9, 2.0 ** -6, 2.0 ** -10, 3 * 2.0 ** -10,
                  2.0 ** -9, 0.0147, -3.3, -2.0 ** -8, 240.0, 255.9], np.float32),
        (rng.standard_normal(400) * np.exp(rng.uniform(-9, 6, 400))).astype(np.float32)])
    got = oracle.e4m3_round(x)
    ref = _e4m3_reference(x).astype(np.float32)
    assert np.array_equal(np.abs(got), np.abs(ref)), x[np.abs(got) != np.abs(ref)][:5]
    assert np.all(np.sign(got[got != 0]) == np.sign(x[got != 0]))


def test_fp8_forward_matches_rounded_numpy(oracle, built):
    """FP8 mode: the hidden 64x64 matrices are FP8-E4M3 values at scale 2^6 and the activations
    entering them are E4M3 values at scale 2^7; the first and last matrices stay FP16."""
    cfg = small_cfg(**{"network.precision": 2})
    L, p = random_params(cfg, seed=5)
    net = oracle.network(cfg, L, p)
    pos = np.random.default_rng(6).uniform(0, 1, (64, 2, 3)).astype(np.float32)
    feats = oracle.encode(net, pos)
    H = cfg.network.n_hidden_layers
    x = feats.astype(np.float16).astype(np.float64)
    off = 0
    for m in range(H + 1):
        rows = 16 if m == H else 64
        cols = L.n_inputs if m == 0 else 64
        w = p[off:off + rows * cols]
        if 1 <= m <= H - 1:
            w = oracle.e4m3_round(w * 64.0) / np.float32(64.0)
        else:
            w = w.astype(np.float16).astype(np.float32)
        W = w.reshape(rows, cols).astype(np.float64)
        off += rows * cols
        x = x @ W.T
        if m < H:
            a = np.maximum(x, 0).astype(np.float32)
            q = (oracle.e4m3_round(a * np.float32(128.0)) / np.float32(128.0)).reshape(a.shape)
            x = (q if m + 1 <= H - 1 else a.astype(np.float16)).astype(np.float64)
    ref = 1.0 / (1.0 + np.exp(-x))
    out = oracle.network_inference(net, pos)
    assert np.max(np.abs(out - ref)) < 1e-5
    out16 = oracle.network_inference(oracle.network(small_cfg(), L, p), pos)
    assert np.max(np.abs(out16 - out)) > 1e-3


@pytest.mark.parametrize("levels,log2t,base,scale", [(16, 19, 16, (2048 / 16) ** (1 / 15)), (8, 18, 8, 2.0),
                                                     (12, 17, 4, 1.5), (32, 22, 2, 1.26)])
def test_grid_layout_follows_tcnn_and_matches_library(oracle, built, levels, log2t, base, scale):
    """Level scale exp2f(l * log2f(s)) * base - 1 (tcnn's grid_scale), resolution ceil(scale) + 1,
    entries min(roundup8(res^3), 2^log2T): the library's layout equals the oracle's bit for bit."""
    cfg = nb.default_config(**{"hashgrid.n_levels": levels, "hashgrid.log2_hashmap_size": log2t,
                               "hashgrid.base_resolution": base, "hashgrid.per_level_scale": scale,
                               "module.input_segment_points": 1 if levels == 32 else 4})
    if levels == 12:
        cfg.module.input_segment_points = 2
    L = nb.param_layout(cfg)
    off, size, res, scl, total = oracle.grid_layout(levels, log2t, base, cfg.hashgrid.per_level_scale)
    assert np.array_equal(np.array(L.level_scale[:levels], np.float32).view(np.uint32), scl.view(np.uint32))
    assert list(L.level_resolution[:levels]) == list(res) and list(L.level_size[:levels]) == list(size)
    assert list(L.level_offset[:levels]) == list(off) and L.n_grid_entries == total
    lg = np.log2(np.float32(cfg.hashgrid.per_level_scale))
    expect = (np.exp2(np.arange(levels, dtype=np.float64) * lg) * base - 1).astype(np.float32)
    np.testing.assert_allclose(scl, expect, rtol=1e-6)
    assert np.all(res == np.ceil(scl).astype(np.uint32) + 1)
