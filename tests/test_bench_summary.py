"""The bench line's closing summary (the figures a reader of the line's tail needs): every key is
present, numbers are rounded, and sections the run skipped come out as None instead of raising."""

import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402

KEYS = {"neural_mrays", "classic_mrays", "neural_over_classic", "mesh4m_neural_over_classic", "mesh4m_neural_mrays",
        "mesh4m_classic_mrays", "vis_agree", "depth_rel_mean_raw", "depth_rel_mean_floor1pct", "depth_within_1pct",
        "depth_rel_mean_raw_origin_outside_leaves", "cpu_classic_mrays_all", "cpu_classic_mrays_1thr", "cpu_cores",
        "serving_render_p99_ms_requests_0p5_to_2m_rays", "serving_1m_batch_p99_ms", "serving_1m_batch_p50_ms",
        "train_ms_per_step", "train_mlp_tc_frac", "mlp_tc_frac", "e2e_mrays", "refdefault_f4_mrays",
        "refdefault_f4_vis_agree"}


def test_summary_of_a_full_line():
    line = {"value": 1318.01322, "classic_mrays": 3960.93, "neural_over_classic": 0.33276,
            "visibility_agreement": 0.997712, "depth_error": {"mean_rel_raw": 2.35029, "mean_rel_floor1pct": 0.40432,
                                                              "within_1pct": 0.92247},
            "depth_error_by_origin": {"origin_outside_leaves": {"mean_rel_raw": 0.010006}},
            "mesh_4m": {"neural_over_classic": 0.58219, "neural_mrays": 1468.94, "classic_mrays": 2523.01},
            "cpu_baseline": {"classic": {"value": 31.5612, "single_thread": 2.25713, "cores": 16}},
            "serving": {"neural": {"p99_ms_requests_0p5_to_2m_rays": 106.1688,
                                   "batch_1m": {"p99_ms": 11.5511, "p50_ms": 4.0451}}},
            "train_roofline": {"ms_per_step": 1.76512, "mlp_tc": {"frac": 0.08643}},
            "roofline_kernels": {"mlp_tc": {"frac": 0.40838}}, "e2e": {"value": 1112.909},
            "config_reference_default": {"query_mrays": 1818.21, "visibility_agreement": 0.99701}}
    s = bench.summary_of(line)
    assert set(s) == KEYS
    assert s["neural_mrays"] == 1318.0 and s["serving_1m_batch_p99_ms"] == 11.55 and s["vis_agree"] == 0.9977
    json.dumps(s)


def test_summary_of_a_line_with_sections_skipped():
    s = bench.summary_of({"value": 1000.0})
    assert set(s) == KEYS
    assert s["neural_mrays"] == 1000.0
    assert all(v is None for k, v in s.items() if k != "neural_mrays")
