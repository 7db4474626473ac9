"""The C ABI without a GPU: the library loads, exports every entry point include/nbvh.h declares,
its ctypes mirror has the C struct sizes, the host-only utilities work, and the device calls fail
with a status code (never an exception across the boundary)."""

import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

import nbvh_gb300 as nb
from nbvh_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "nbvh.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(nbvh_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported(built):
    lib = C.CDLL(nb.LIB_PATH)
    names = declared_functions()
    assert len(names) >= 40
    for name in names:
        assert hasattr(lib, name), name
    assert set(names) == set(abi.PROTOTYPES), set(names) ^ set(abi.PROTOTYPES)


def test_struct_sizes_match_c(built, tmp_path):
    src = tmp_path / "sz.c"
    structs = {"nbvh_config": abi.Config, "nbvh_param_layout": abi.ParamLayout, "nbvh_train_stats": abi.TrainStats,
               "nbvh_render_request": abi.RenderRequest, "nbvh_query_stats": abi.QueryStats,
               "nbvh_ray": None, "nbvh_hit": None, "nbvh_neural_hit": None, "nbvh_segment": None}
    body = "".join('printf("%%zu\\n", sizeof(%s));' % k for k in structs)
    src.write_text('#include <stdio.h>\n#include "nbvh.h"\nint main(void){%s return 0;}\n' % body)
    exe = tmp_path / "sz"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    sizes = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()]
    expect = {"nbvh_ray": 32, "nbvh_hit": 16, "nbvh_neural_hit": 48, "nbvh_segment": 16}
    for (name, cls), sz in zip(structs.items(), sizes):
        if cls is None:
            assert sz == expect[name], name
            assert sz == {"nbvh_ray": nb.RAY_DTYPE, "nbvh_hit": nb.HIT_DTYPE, "nbvh_neural_hit": nb.NEURAL_HIT_DTYPE,
                          "nbvh_segment": nb.SEGMENT_DTYPE}[name].itemsize
        else:
            assert C.sizeof(cls) == sz, name


def test_config_defaults(built):
    cfg = nb.default_config()
    assert cfg.abi_version == abi.NBVH_ABI_VERSION
    assert (cfg.hashgrid.n_levels, cfg.hashgrid.n_features_per_level, cfg.hashgrid.log2_hashmap_size) == (16, 2, 19)
    assert cfg.hashgrid.base_resolution == 16
    assert abs(cfg.hashgrid.per_level_scale - (2048 / 16) ** (1 / 15)) < 1e-6
    assert (cfg.network.n_neurons, cfg.network.n_hidden_layers) == (64, 4)
    assert cfg.module.input_segment_points == 4 and cfg.batch_size == 1 << 18
    assert abs(cfg.optimizer.learning_rate - 1e-2) < 1e-9 and cfg.optimizer.decay_start == 10000
    # NeuralBVHRendererConstants defaults (include/cuda/neural/neural_bvh_renderer_constants.cuh:24-31)
    assert cfg.bvh.inference_mint_epsilon == np.float32(1e-4) and cfg.bvh.fixed_node_dilation == np.float32(1e-5)
    assert abs(cfg.output.depth_epsilon - 0.2) < 1e-7 and cfg.output.visibility_loss == abi.LOSS["BinaryCrossEntropy"]
    L = nb.param_layout(cfg)
    assert L.n_inputs == 128 and L.n_network_params == 128 * 64 + 3 * 64 * 64 + 16 * 64
    assert list(L.level_resolution[:16])[0] == 16 and list(L.level_resolution[:16])[-1] == 2048
    assert L.n_params == L.n_network_params + 2 * L.n_grid_entries and L.n_features_per_level == 2


def test_config_validation(built):
    lib = nb.load_library()
    L = abi.ParamLayout()
    for key, val in (("hashgrid.n_features_per_level", 3), ("network.n_neurons", 128), ("batch_size", 1000),
                     ("module.input_segment_points", 5), ("network.precision", 3)):
        cfg = nb.default_config(**{key: val})
        assert lib.nbvh_param_layout_host(C.byref(cfg), C.byref(L)) == abi.NBVH_EINVAL, key
    for prec in (0, 1, 2):  # FP16, BF16, FP8
        cfg = nb.default_config(**{"network.precision": prec})
        assert lib.nbvh_param_layout_host(C.byref(cfg), C.byref(L)) == abi.NBVH_OK, prec


def test_status_strings_and_null_handles(built):
    lib = nb.load_library()
    for s in range(8):
        assert lib.nbvh_status_string(s)
    assert lib.nbvh_destroy(None) == abi.NBVH_EINVAL
    assert lib.nbvh_build_classic(None) == abi.NBVH_EINVAL
    assert lib.nbvh_query_closest_classic(None, None, 0, None, None) == abi.NBVH_EINVAL
    assert lib.nbvh_abi_version() == abi.NBVH_ABI_VERSION


def test_init_params_seeded(built):
    cfg = nb.default_config()
    a, b = nb.init_params(cfg), nb.init_params(cfg)
    assert np.array_equal(a, b)
    L = nb.param_layout(cfg)
    grid = a[L.n_network_params:]
    assert np.abs(grid).max() <= 1e-4
    out = a[L.n_network_params - 16 * 64:L.n_network_params].reshape(16, 64)
    assert np.all(out[8:] == 0) and np.abs(out[:8]).max() > 0
    c = nb.init_params(nb.default_config(seed=7))
    assert not np.array_equal(a, c)


def test_create_without_device_reports_edevice(built):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(nb.NBVHError) as e:
        nb.NBVH(nb.default_config())
    assert e.value.status == abi.NBVH_EDEVICE


def test_server_config_checked_before_the_device(built):
    """A query lane must leave at least one slot for renders; the configuration is refused with
    EINVAL before any device call (so this runs without a GPU)."""
    for n_slots, q in ((2, 2), (1, 1), (3, 5)):
        with pytest.raises(nb.NBVHError) as e:
            nb.Server(n_slots=n_slots, query_slots=q)
        assert e.value.status == abi.NBVH_EINVAL
    assert C.sizeof(abi.ServerConfig) == 56
