"""Reference-style JSON configuration (no GPU).

The reference renderer reads its settings from a JSON file whose missing keys keep the reference's
defaults (src/cuda/neural/neural_bvh_renderer_init.cu:690-712, include/cuda/neural/utils/
tcnn_config.h:94-101, include/cuda/neural/neural_bvh_renderer_constants.cuh:78-108,
include/cuda/neural/utils/bvh_split_scheduler.h:131-140). `config_from_reference_json` and
`tree_cut_options_from_reference_json` do the same: every key maps to its field, absent keys take
the reference defaults, and the configurations the reference ships load as the reference reads
them (when its tree is on this machine).
"""

import glob
import json
import os

import pytest

import nbvh_gb300 as nb
from helpers import reference_root
from nbvh_gb300 import abi


def test_reference_defaults_and_features_per_level(built):
    cfg = nb.reference_default_config()
    hg = cfg.hashgrid
    assert (hg.n_levels, hg.n_features_per_level, hg.log2_hashmap_size, hg.base_resolution) == (8, 4, 18, 8)
    assert hg.per_level_scale == 2.0 and cfg.module.input_segment_points == 3 and cfg.neural_bvh_max_depth == 0
    # the reference default (3 points x 8 levels x 4 features = 96 network inputs) lays out
    L = nb.param_layout(cfg)
    assert L.n_inputs == 3 * 8 * 4 and L.n_features_per_level == 4
    assert L.n_params == L.n_network_params + 4 * L.n_grid_entries
    for f in (2, 8):
        cfg.hashgrid.n_features_per_level = f
        if 3 * 8 * f <= 128:
            L = nb.param_layout(cfg)
            assert L.n_inputs == 3 * 8 * f and L.n_params == L.n_network_params + f * L.n_grid_entries
        else:  # 3 x 8 x 8 = 192 inputs: more than the fused MLP takes
            with pytest.raises(nb.NBVHError):
                nb.param_layout(cfg)
    cfg.module.input_segment_points = 2
    assert nb.param_layout(cfg).n_inputs == 2 * 8 * 8
    for f in (1, 3, 16):  # feature counts the table layout does not support
        cfg.hashgrid.n_features_per_level = f
        with pytest.raises(nb.NBVHError):
            nb.param_layout(cfg)


def test_every_key_maps_to_its_field(built):
    js = {"neural_bvh_renderer": {
        "batch_size": 1 << 16, "neural_bvh_min_depth": 7,
        "bvh_constants": {"inference_mint_epsilon": 2e-4, "inference_maxt_epsilon": 2e-3,
                          "learning_mint_epsilon": 3e-3, "learning_maxt_epsilon": 4e-3,
                          "sampling_bbox_scaling": 1.25, "fixed_node_dilation": 2e-5, "node_extent_dilation": 3e-4,
                          "leaf_boundary_sampling_ratio": 0.5, "ignore_neural_blas": True, "max_training_bounces": 1,
                          "sample_cosine_weighted": False, "backface_bounce_training": True,
                          "log2_bvh_max_traversals": 0, "num_lods_learned": 3, "training_node_survival": True,
                          "survival_probability_scale": 0.75, "min_rr_survival_prob": 0.01},
        "tree_cut_learning": True,
        "bvh_split_scheduler": {"splitting_interval": 40, "last_split_iteration": 2500, "start_split_num": 2,
                                "split_scaling": 2.5, "split_interval_scaling": 1.5},
        "neural_module": {
            "pt_output_constants": {"visibility_loss": "BinaryCrossEntropy", "depth_loss": "L2",
                                    "normal_loss": "L1", "albedo_loss": "RelativeL2",
                                    "visibility_loss_scale": 2.0, "depth_loss_scale": 3.0, "normal_loss_scale": 0.5,
                                    "albedo_loss_scale": 0.25, "primary_visibility_threshold": 0.4,
                                    "secondary_visibility_threshold": 0.6, "depth_epsilon": 0.1,
                                    "fixed_depth_epsilon": 2e-5, "output_normal_linear_activation": False,
                                    "output_albedo_linear_activation": True, "visibility_masking_loss": False,
                                    "output_normal_dim": 0, "output_albedo_dim": 3},
            "bvh_module_constants": {"input_segment_points": 2, "segment_distribution": "EquidistantExterior"},
            "network": {"n_neurons": 64, "n_hidden_layers": 3},
            "optimizer": {"learning_rate": 5e-3, "beta1": 0.85, "beta2": 0.99, "epsilon": 1e-7, "l2_reg": 1e-6,
                          "decay_base": 0.5, "decay_start": 5000, "decay_interval": 1000},
            "segment_encoding": {"hashgrid_options": {"n_levels": 12, "n_features_per_level": 2,
                                                      "log2_hashmap_size": 17, "base_resolution": 4,
                                                      "per_level_scale": 1.5}}}}}
    cfg = nb.config_from_reference_json(js)
    assert cfg.batch_size == 1 << 16 and cfg.neural_bvh_max_depth == 7
    b = cfg.bvh
    assert (b.inference_mint_epsilon, b.sampling_bbox_scaling, b.leaf_boundary_sampling_ratio) == pytest.approx(
        (2e-4, 1.25, 0.5))
    assert (b.ignore_neural_blas, b.sample_cosine_weighted, b.backface_bounce_training) == (1, 0, 1)
    o = cfg.output
    assert o.depth_loss == abi.LOSS["L2"] and o.visibility_loss == abi.LOSS["BinaryCrossEntropy"]
    assert (o.visibility_loss_scale, o.depth_loss_scale, o.primary_visibility_threshold) == pytest.approx((2, 3, 0.4))
    assert (o.output_normal_linear_activation, o.output_albedo_linear_activation, o.visibility_masking_loss) == (0, 1, 0)
    assert (o.learn_normal, o.learn_albedo) == (0, 1)
    assert cfg.module.input_segment_points == 2
    assert cfg.module.segment_distribution == abi.SEGMENT["EquidistantExterior"]
    assert cfg.network.n_hidden_layers == 3
    op = cfg.optimizer
    assert (op.learning_rate, op.beta1, op.decay_base) == pytest.approx((5e-3, 0.85, 0.5))
    assert (op.decay_start, op.decay_interval) == (5000, 1000)
    hg = cfg.hashgrid
    assert (hg.n_levels, hg.n_features_per_level, hg.log2_hashmap_size, hg.base_resolution) == (12, 2, 17, 4)
    assert hg.per_level_scale == pytest.approx(1.5)
    assert nb.param_layout(cfg).n_inputs == 2 * 12 * 2
    t = nb.tree_cut_options_from_reference_json(js)
    assert t.tree_cut_learning == 1
    assert (t.splitting_interval, t.last_split_iteration, t.start_split_num) == (40, 2500, 2)
    assert (t.split_scaling, t.split_interval_scaling) == pytest.approx((2.5, 1.5))
    assert (t.num_lods_learned, t.training_node_survival) == (3, 1)
    assert (t.survival_probability_scale, t.min_rr_survival_prob) == pytest.approx((0.75, 0.01))
    # absent keys keep the defaults
    d = nb.tree_cut_options_from_reference_json({})
    ref = nb.tree_cut_options()
    assert all(getattr(d, f) == getattr(ref, f) for f, _ in abi.TreeCutOptions._fields_ if f != "reserved")


def test_shipped_configurations_load_as_the_reference_reads_them(built):
    paths = sorted(glob.glob(os.path.join(reference_root(), "scene_data", "*", "*", "configs", "*.json")))
    if not paths:
        pytest.skip("the reference tree is not on this machine")
    for p in paths:
        with open(p) as f:
            js = json.load(f)
        r = js["neural_bvh_renderer"]
        cfg = nb.config_from_reference_json(js)
        hg = r.get("neural_module", {}).get("segment_encoding", {}).get("hashgrid_options", {})
        assert cfg.hashgrid.n_levels == hg.get("n_levels", 8)
        assert cfg.hashgrid.n_features_per_level == hg.get("n_features_per_level", 4)
        assert cfg.hashgrid.log2_hashmap_size == hg.get("log2_hashmap_size", 18)
        assert cfg.hashgrid.base_resolution == hg.get("base_resolution", 8)
        mc = r.get("neural_module", {}).get("bvh_module_constants", {})
        assert cfg.module.input_segment_points == mc.get("input_segment_points", 3)
        t = nb.tree_cut_options_from_reference_json(js)
        sch = r.get("bvh_split_scheduler", {})
        assert t.tree_cut_learning == int(r.get("tree_cut_learning", False))
        for k in ("splitting_interval", "last_split_iteration", "start_split_num"):
            if k in sch:
                assert getattr(t, k) == sch[k], (p, k)
        # the shipped grids use the reference's 4 features per level: they lay out as they are
        L = nb.param_layout(cfg)
        assert L.n_inputs == (cfg.module.input_segment_points * cfg.hashgrid.n_levels *
                              cfg.hashgrid.n_features_per_level)
        assert L.n_params == L.n_network_params + cfg.hashgrid.n_features_per_level * L.n_grid_entries
