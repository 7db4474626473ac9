"""nbvh_gb300 -- Python bindings of libnbvh, the GB300-native N-BVH ray-query library.

The product is the C ABI in include/nbvh.h (host C++ over sm_103a CUDA kernels); this module is a
thin ctypes layer over it for tests, benchmarks and Python callers. Device buffers are torch CUDA
tensors (only their data pointers cross the boundary); host buffers are numpy arrays.

There is no CPU fallback: without the compiled library importing works, but every call raises,
and without a GPU the library answers NBVH_EDEVICE.
"""

import ctypes as C
import os

import numpy as np

from . import abi
from .abi import (Config, KernelProfile, ParamLayout, PathRequest, QueryStats, RenderRequest, Request, RequestResult,
                  ServerConfig, ServerStats, TrainStats)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libnbvh.so")

RAY_DTYPE = np.dtype([("o", np.float32, 3), ("tmin", np.float32), ("d", np.float32, 3), ("tmax", np.float32)])
HIT_DTYPE = np.dtype([("t", np.float32), ("u", np.float32), ("v", np.float32), ("prim", np.uint32)])
NEURAL_HIT_DTYPE = np.dtype([("t", np.float32), ("normal", np.float32, 3), ("albedo", np.float32, 3),
                             ("visibility", np.float32), ("flags", np.uint32), ("segments", np.uint32),
                             ("prim", np.uint32), ("reserved", np.uint32)])
SEGMENT_DTYPE = np.dtype([("mint", np.float32), ("maxt", np.float32), ("node", np.uint32), ("reserved", np.uint32)])
FLT_MAX = np.float32(3.4028234663852886e38)

_lib = None


class NBVHError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s: %s" % (abi.STATUS_NAMES.get(status, status), message))
        self.status = status


def load_library(path=None):
    """Loads libnbvh.so (built in-tree by nbvh_gb300.build) and binds every prototype."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise NBVHError(abi.NBVH_EDEVICE, "libnbvh.so not built (run nbvh_gb300.build.build())")
    lib = C.CDLL(p)
    for name, (res, args) in abi.PROTOTYPES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def default_config(**overrides):
    """nbvh_config_default() with keyword overrides using dotted names, e.g.
    default_config(**{"hashgrid.n_levels": 8, "batch_size": 1 << 16})."""
    lib = load_library()
    cfg = Config()
    _check(lib.nbvh_config_default(C.byref(cfg)), None)
    for key, val in overrides.items():
        obj = cfg
        parts = key.split(".")
        for part in parts[:-1]:
            obj = getattr(obj, part)
        setattr(obj, parts[-1], val)
    return cfg


def reference_default_config():
    """The configuration the reference renderer starts from before it reads a JSON file: this
    library's defaults (the benchmark's inference configuration) with the reference's own defaults
    where they differ: hash grid of 8 levels x 4 features x 2^18 entries, base resolution 8, level
    scale 2.0 (include/cuda/neural/utils/tcnn_config.h:70-74), 3 segment points
    (include/cuda/neural/neural_bvh_module.h:81) and a neural cut from the root
    (m_neural_bvh_min_depth = 0, include/cuda/neural/neural_bvh_renderer.h:206)."""
    cfg = default_config()
    cfg.hashgrid.n_levels = 8
    cfg.hashgrid.n_features_per_level = 4
    cfg.hashgrid.log2_hashmap_size = 18
    cfg.hashgrid.base_resolution = 8
    cfg.hashgrid.per_level_scale = 2.0
    cfg.module.input_segment_points = 3
    cfg.neural_bvh_max_depth = 0
    return cfg


def config_from_reference_json(js, base=None):
    """Builds a config from a reference-style JSON dict (neural_bvh_renderer section keys:
    bvh_constants, neural_module.{pt_output_constants, bvh_module_constants, network, optimizer,
    segment_encoding.hashgrid_options}, batch_size, neural_bvh_min_depth). Keys the dict leaves out
    take the reference's defaults (reference_default_config), as the reference's loaders do, unless
    `base` is given."""
    cfg = base if base is not None else reference_default_config()
    r = js.get("neural_bvh_renderer", js)
    nm = r.get("neural_module", {})
    bc = r.get("bvh_constants", {})
    for k in ("inference_mint_epsilon", "inference_maxt_epsilon", "learning_mint_epsilon", "learning_maxt_epsilon",
              "sampling_bbox_scaling", "fixed_node_dilation", "node_extent_dilation", "leaf_boundary_sampling_ratio"):
        if k in bc:
            setattr(cfg.bvh, k, float(bc[k]))
    for k in ("ignore_neural_blas", "max_training_bounces", "sample_cosine_weighted", "backface_bounce_training",
              "log2_bvh_max_traversals"):
        if k in bc:
            setattr(cfg.bvh, k, int(bc[k]))
    pt = nm.get("pt_output_constants", {})
    for k in ("visibility_loss", "depth_loss", "normal_loss", "albedo_loss"):
        if k in pt:
            setattr(cfg.output, k, abi.LOSS[pt[k]])
    for k in ("visibility_loss_scale", "depth_loss_scale", "normal_loss_scale", "albedo_loss_scale",
              "primary_visibility_threshold", "secondary_visibility_threshold", "depth_epsilon",
              "fixed_depth_epsilon"):
        if k in pt:
            setattr(cfg.output, k, float(pt[k]))
    for k in ("output_normal_linear_activation", "output_albedo_linear_activation", "visibility_masking_loss"):
        if k in pt:
            setattr(cfg.output, k, int(bool(pt[k])))
    if "output_normal_dim" in pt:
        cfg.output.learn_normal = int(pt["output_normal_dim"] == 3)
    if "output_albedo_dim" in pt:
        cfg.output.learn_albedo = int(pt["output_albedo_dim"] == 3)
    mc = nm.get("bvh_module_constants", {})
    if "input_segment_points" in mc:
        cfg.module.input_segment_points = int(mc["input_segment_points"])
    if "segment_distribution" in mc:
        cfg.module.segment_distribution = abi.SEGMENT[mc["segment_distribution"]]
    net = nm.get("network", {})
    if "n_neurons" in net:
        cfg.network.n_neurons = int(net["n_neurons"])
    if "n_hidden_layers" in net:
        cfg.network.n_hidden_layers = int(net["n_hidden_layers"])
    opt = nm.get("optimizer", {})
    for k in ("learning_rate", "beta1", "beta2", "epsilon", "l2_reg", "decay_base"):
        if k in opt:
            setattr(cfg.optimizer, k, float(opt[k]))
    for k in ("decay_start", "decay_interval"):
        if k in opt:
            setattr(cfg.optimizer, k, int(opt[k]))
    hg = nm.get("segment_encoding", {}).get("hashgrid_options", {})
    for k in ("n_levels", "n_features_per_level", "log2_hashmap_size", "base_resolution"):
        if k in hg:
            setattr(cfg.hashgrid, k, int(hg[k]))
    if "per_level_scale" in hg:
        cfg.hashgrid.per_level_scale = float(hg["per_level_scale"])
    if "batch_size" in r:
        cfg.batch_size = int(r["batch_size"])
    if "neural_bvh_min_depth" in r:
        cfg.neural_bvh_max_depth = int(r["neural_bvh_min_depth"])
    return cfg


def _check(status, handle, lib=None):
    if status != abi.NBVH_OK:
        lib = lib or load_library()
        msg = lib.nbvh_last_error(handle).decode() if handle else lib.nbvh_status_string(status).decode()
        raise NBVHError(status, msg)


def _ptr(x):
    """Data pointer of a torch tensor (device or host) or a numpy array."""
    if x is None:
        return None
    if isinstance(x, np.ndarray):
        return x.ctypes.data_as(C.c_void_p)
    return C.c_void_p(x.data_ptr())


def _stream(stream):
    if stream is None:
        import torch
        return C.c_void_p(torch.cuda.current_stream().cuda_stream)
    if isinstance(stream, int):
        return C.c_void_p(stream)
    return C.c_void_p(stream.cuda_stream)


def param_layout(cfg):
    lib = load_library()
    L = ParamLayout()
    _check(lib.nbvh_param_layout_host(C.byref(cfg), C.byref(L)), None)
    return L


def read_tcnn_params(path):
    """The parameters of a tcnn trainer JSON file as FP32 (no device needed)."""
    lib = load_library()
    n = C.c_uint64(0)
    _check(lib.nbvh_read_tcnn_params_host(str(path).encode(), None, 0, C.byref(n)), None)
    out = np.empty(n.value, np.float32)
    _check(lib.nbvh_read_tcnn_params_host(str(path).encode(), out.ctypes.data_as(C.POINTER(C.c_float)), n.value,
                                          C.byref(n)), None)
    return out


def write_tcnn_params(path, params):
    """Writes FP32 parameters as a tcnn trainer JSON file (no device needed)."""
    p = np.ascontiguousarray(params, np.float32)
    _check(load_library().nbvh_write_tcnn_params_host(str(path).encode(), p.ctypes.data_as(C.POINTER(C.c_float)),
                                                      p.size), None)


def device_level_scales(cfg, device=0):
    """The hash-grid level scales evaluated on the GPU the way tcnn's kernels do (CUDA's exp2f),
    for comparison with param_layout(cfg).level_scale (the host's exp2f)."""
    n = int(cfg.hashgrid.n_levels)
    out = (C.c_float * 32)()
    _check(load_library().nbvh_debug_device_level_scales(C.byref(cfg), device, out), None)
    return np.array(out[:n], np.float32)


def init_params(cfg):
    L = param_layout(cfg)
    p = np.empty(L.n_params, np.float32)
    _check(load_library().nbvh_init_params_host(C.byref(cfg), _ptr(p)), None)
    return p


def build_bvh2_host(vertices, indices):
    """Host BVH2 build (no device needed): returns (nodes uint32 [n, 8], prim_indices uint32)."""
    lib = load_library()
    v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
    t = np.ascontiguousarray(indices, np.uint32).reshape(-1, 3)
    nodes = np.empty((2 * len(t), 8), np.uint32)
    n = C.c_uint32(0)
    prims = np.empty(len(t), np.uint32)
    _check(lib.nbvh_build_bvh2_host(_ptr(v), len(v), _ptr(t), len(t), _ptr(nodes), C.byref(n), _ptr(prims)), None)
    return nodes[: n.value].copy(), prims


def build_neural_cut_host(nodes, max_depth):
    lib = load_library()
    nodes = np.ascontiguousarray(nodes, np.uint32)
    out = np.empty((max(1, 2 * len(nodes)), 8), np.uint32)
    n = C.c_uint32(len(out))
    _check(lib.nbvh_build_neural_cut_host(_ptr(nodes), len(nodes), max_depth, _ptr(out), C.byref(n)), None)
    return out[: n.value].copy()


class PinnedArray(np.ndarray):
    """numpy array in page-locked host memory (nbvh_host_alloc); the *_host queries read and write
    such buffers from the kernels directly."""

    def __array_finalize__(self, obj):
        if obj is not None and getattr(self, "_owner", None) is None:
            self._owner = getattr(obj, "_owner", None)


class _PinnedBlock:
    def __init__(self, nbytes):
        self.lib = load_library()
        self.ptr = C.c_void_p()
        _check(self.lib.nbvh_host_alloc(nbytes, C.byref(self.ptr)), None)

    def __del__(self):
        if self.ptr:
            self.lib.nbvh_host_free(self.ptr)
            self.ptr = C.c_void_p()


def pinned_empty(shape, dtype):
    """An uninitialised PinnedArray of the given shape and dtype."""
    dtype = np.dtype(dtype)
    shape = (shape,) if np.isscalar(shape) else tuple(shape)
    nbytes = int(np.prod(shape)) * dtype.itemsize
    block = _PinnedBlock(max(nbytes, 1))
    raw = (C.c_uint8 * max(nbytes, 1)).from_address(block.ptr.value)
    arr = np.frombuffer(raw, np.uint8, count=nbytes).view(dtype).reshape(shape).view(PinnedArray)
    arr._owner = block
    return arr


def pinned_copy(a):
    """A PinnedArray holding a copy of a."""
    a = np.ascontiguousarray(a)
    out = pinned_empty(a.shape, a.dtype)
    out[...] = a
    return out


def tree_cut_options(**kw):
    """nbvh_tree_cut_options with the reference defaults, fields overridden by keyword."""
    o = abi.TreeCutOptions()
    _check(load_library().nbvh_tree_cut_options_default(C.byref(o)), None)
    for k, v in kw.items():
        if not hasattr(o, k):
            raise AttributeError(k)
        setattr(o, k, v)
    return o


def tree_cut_options_from_reference_json(js, base=None):
    """Tree-cut options from a reference-style JSON dict, read as the reference renderer reads them
    (src/cuda/neural/neural_bvh_renderer_init.cu:705-712): `tree_cut_learning` and
    `bvh_split_scheduler.{splitting_interval, last_split_iteration, start_split_num, split_scaling,
    split_interval_scaling}` (include/cuda/neural/utils/bvh_split_scheduler.h:131-140) of the
    neural_bvh_renderer section, and `bvh_constants.{num_lods_learned, training_node_survival,
    survival_probability_scale, min_rr_survival_prob}` (include/cuda/neural/
    neural_bvh_renderer_constants.cuh:78-108). Missing keys keep the defaults."""
    o = base if base is not None else tree_cut_options()
    r = js.get("neural_bvh_renderer", js)
    if "tree_cut_learning" in r:
        o.tree_cut_learning = int(bool(r["tree_cut_learning"]))
    sch = r.get("bvh_split_scheduler", {})
    for k in ("splitting_interval", "last_split_iteration", "start_split_num"):
        if k in sch:
            setattr(o, k, int(sch[k]))
    for k in ("split_scaling", "split_interval_scaling"):
        if k in sch:
            setattr(o, k, float(sch[k]))
    bc = r.get("bvh_constants", {})
    for k in ("num_lods_learned", "training_node_survival"):
        if k in bc:
            setattr(o, k, int(bc[k]))
    for k in ("survival_probability_scale", "min_rr_survival_prob"):
        if k in bc:
            setattr(o, k, float(bc[k]))
    return o


def split_schedule(options, start_nodes, n_iterations):
    """Splits per iteration (capped by the leaves) and the node count reached (no device needed)."""
    splits = np.zeros(max(n_iterations, 1), np.uint32)
    nodes = C.c_uint32(0)
    _check(load_library().nbvh_split_schedule_host(C.byref(options), start_nodes, n_iterations, _ptr(splits),
                                                   C.byref(nodes)), None)
    return splits[:n_iterations], nodes.value


def read_nbvh(path):
    """Neural-cut nodes (uint32 [n, 8]) of a reference .nbvh file (no device needed)."""
    lib = load_library()
    n = C.c_uint32(0)
    _check(lib.nbvh_read_nbvh_host(str(path).encode(), None, C.byref(n)), None)
    nodes = np.empty((n.value, 8), np.uint32)
    _check(lib.nbvh_read_nbvh_host(str(path).encode(), _ptr(nodes), C.byref(n)), None)
    return nodes


def write_nbvh(path, nodes):
    """Writes neural-cut nodes (uint32 [n, 8]) as a reference .nbvh file."""
    nodes = np.ascontiguousarray(nodes, np.uint32)
    _check(load_library().nbvh_write_nbvh_host(str(path).encode(), _ptr(nodes), len(nodes)), None)


def nodes_to_float(nodes):
    """Bounding boxes of uint32 [n, 8] node records: (min [n,3], max [n,3]) float32."""
    f = nodes.view(np.float32)
    return f[:, 0:3].copy(), f[:, 4:7].copy()


class NBVH:
    """One library handle: scene, classic BVH, neural cut, network parameters and workspaces."""

    def __init__(self, config=None, device=0):
        self.lib = load_library()
        self.cfg = config if config is not None else default_config()
        h = C.c_void_p()
        _check(self.lib.nbvh_create(C.byref(self.cfg), device, C.byref(h)), None, self.lib)
        self.h = h
        self.device = device
        L = ParamLayout()
        self._check(self.lib.nbvh_get_param_layout(self.h, C.byref(L)))
        self.layout = L

    def _check(self, st):
        _check(st, self.h, self.lib)

    def close(self):
        if getattr(self, "h", None):
            self.lib.nbvh_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- scene ----
    def set_mesh(self, vertices, indices, albedo=None):
        v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
        t = np.ascontiguousarray(indices, np.uint32).reshape(-1, 3)
        a = None if albedo is None else np.ascontiguousarray(albedo, np.float32).reshape(-1, 3)
        self._keep = (v, t, a)
        self._check(self.lib.nbvh_set_mesh(self.h, _ptr(v), len(v), _ptr(t), len(t), _ptr(a)))

    def build_classic(self):
        self._check(self.lib.nbvh_build_classic(self.h))

    def classic_bvh(self):
        nn, np_ = C.c_uint32(0), C.c_uint32(0)
        self._check(self.lib.nbvh_get_classic_bvh(self.h, None, C.byref(nn), None, C.byref(np_)))
        nodes = np.empty((nn.value, 8), np.uint32)
        prims = np.empty(np_.value, np.uint32)
        self._check(self.lib.nbvh_get_classic_bvh(self.h, _ptr(nodes), C.byref(nn), _ptr(prims), C.byref(np_)))
        return nodes, prims

    def build_neural_cut(self, max_depth=None):
        self._check(self.lib.nbvh_build_neural_cut(self.h, self.cfg.neural_bvh_max_depth if max_depth is None else max_depth))

    def neural_bvh(self):
        nn = C.c_uint32(0)
        self._check(self.lib.nbvh_get_neural_bvh(self.h, None, C.byref(nn), None))
        nodes = np.empty((nn.value, 8), np.uint32)
        bbox = np.empty(6, np.float32)
        self._check(self.lib.nbvh_get_neural_bvh(self.h, _ptr(nodes), C.byref(nn), _ptr(bbox)))
        return nodes, bbox

    def set_non_neural_leaves(self, node_ids, flag=True):
        ids = np.ascontiguousarray(node_ids, np.uint32)
        self._check(self.lib.nbvh_set_non_neural_leaves(self.h, _ptr(ids), len(ids), int(bool(flag))))

    def set_ray_ordering(self, enable):
        self._check(self.lib.nbvh_set_ray_ordering(self.h, 1 if enable else 0))

    def set_ignore_neural_blas(self, ignore):
        self._check(self.lib.nbvh_set_ignore_neural_blas(self.h, int(bool(ignore))))

    # ---- queries on device tensors ----
    def _out(self, like, n, words):
        import torch
        return torch.empty((n, words), dtype=torch.int32, device=like.device)

    def query_closest_classic(self, rays, out=None, stream=None):
        n = rays.shape[0]
        out = self._out(rays, n, 4) if out is None else out
        self._check(self.lib.nbvh_query_closest_classic(self.h, _ptr(rays), n, _ptr(out), _stream(stream)))
        return out

    def query_any_classic(self, rays, out=None, stream=None):
        n = rays.shape[0]
        out = self._out(rays, n, 4) if out is None else out
        self._check(self.lib.nbvh_query_any_classic(self.h, _ptr(rays), n, _ptr(out), _stream(stream)))
        return out

    def query_closest_neural(self, rays, depth=1, out=None, stream=None):
        n = rays.shape[0]
        out = self._out(rays, n, 12) if out is None else out
        self._check(self.lib.nbvh_query_closest_neural(self.h, _ptr(rays), n, depth, _ptr(out), _stream(stream)))
        return out

    def query_visibility_neural(self, rays, depth=1, out=None, stream=None):
        n = rays.shape[0]
        out = self._out(rays, n, 12) if out is None else out
        self._check(self.lib.nbvh_query_visibility_neural(self.h, _ptr(rays), n, depth, _ptr(out), _stream(stream)))
        return out

    def query_segments(self, rays, max_segments, stream=None):
        import torch
        n = rays.shape[0]
        segs = torch.empty((n, max_segments, 4), dtype=torch.int32, device=rays.device)
        counts = torch.empty(n, dtype=torch.int32, device=rays.device)
        self._check(self.lib.nbvh_query_segments(self.h, _ptr(rays), n, max_segments, _ptr(segs), _ptr(counts),
                                                 _stream(stream)))
        return segs, counts

    # ---- queries on host arrays (pinned or pageable) ----
    @staticmethod
    def _host_rays(rays_np):
        if not (isinstance(rays_np, PinnedArray) and rays_np.flags.c_contiguous):
            rays_np = np.ascontiguousarray(rays_np)
        return rays_np, rays_np.nbytes // 32

    def query_closest_neural_host(self, rays_np, depth=1, out=None):
        rays_np, n = self._host_rays(rays_np)
        if out is None:
            out = pinned_empty(n, NEURAL_HIT_DTYPE) if isinstance(rays_np, PinnedArray) else np.empty(n, NEURAL_HIT_DTYPE)
        self._check(self.lib.nbvh_query_closest_neural_host(self.h, _ptr(rays_np), n, depth, _ptr(out)))
        return out

    def query_closest_classic_host(self, rays_np, out=None):
        rays_np, n = self._host_rays(rays_np)
        if out is None:
            out = pinned_empty(n, HIT_DTYPE) if isinstance(rays_np, PinnedArray) else np.empty(n, HIT_DTYPE)
        self._check(self.lib.nbvh_query_closest_classic_host(self.h, _ptr(rays_np), n, _ptr(out)))
        return out

    # ---- network ----
    def params(self):
        p = np.empty(self.layout.n_params, np.float32)
        self._check(self.lib.nbvh_get_params(self.h, _ptr(p)))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.layout.n_params
        self._check(self.lib.nbvh_set_params(self.h, _ptr(p)))

    def network_inference(self, positions, stream=None):
        import torch
        n = positions.shape[0]
        out = torch.empty((n, 8), dtype=torch.float32, device=positions.device)
        self._check(self.lib.nbvh_network_inference(self.h, _ptr(positions), n, _ptr(out), _stream(stream)))
        return out

    def mlp_inference(self, features, stream=None):
        """tcgen05 MLP on 16-bit encoded inputs ([n, n_inputs], contiguous): torch.float16, or
        torch.bfloat16 when the network precision is BF16."""
        import torch
        want = torch.bfloat16 if int(self.cfg.network.precision) == 1 else torch.float16
        assert features.dtype == want and features.is_contiguous()
        n = features.shape[0]
        out = torch.empty((n, 8), dtype=torch.float32, device=features.device)
        self._check(self.lib.nbvh_mlp_inference(self.h, _ptr(features), n, _ptr(out), _stream(stream)))
        return out

    def encode(self, positions, stream=None):
        import torch
        n = positions.shape[0]
        out = torch.empty((n, self.layout.n_inputs), dtype=torch.float32, device=positions.device)
        self._check(self.lib.nbvh_encode(self.h, _ptr(positions), n, _ptr(out), _stream(stream)))
        return out

    def compute_gradients(self, positions, targets, stream=None):
        import torch
        n = positions.shape[0]
        g = torch.empty(self.layout.n_params, dtype=torch.float32, device=positions.device)
        loss = C.c_float(0)
        self._check(self.lib.nbvh_compute_gradients(self.h, _ptr(positions), _ptr(targets), n, _ptr(g),
                                                    C.byref(loss), _stream(stream)))
        return g, loss.value

    def adam_step(self, gradients, stream=None):
        self._check(self.lib.nbvh_adam_step(self.h, _ptr(gradients), _stream(stream)))

    def generate_training_batch(self, training_step, n, stream=None):
        import torch
        P = self.cfg.module.input_segment_points
        dev = torch.device("cuda", self.device)
        pos = torch.empty((n, P, 3), dtype=torch.float32, device=dev)
        tgt = torch.empty((n, 8), dtype=torch.float32, device=dev)
        nodes = torch.empty(n, dtype=torch.int32, device=dev)
        self._check(self.lib.nbvh_generate_training_batch(self.h, training_step, n, _ptr(pos), _ptr(tgt),
                                                          _ptr(nodes), _stream(stream)))
        return pos, tgt, nodes

    def run_optimisation(self, steps):
        st = TrainStats()
        self._check(self.lib.nbvh_run_optimisation(self.h, steps, C.byref(st)))
        return st

    @property
    def training_step(self):
        return self.lib.nbvh_training_step(self.h)

    # ---- run-inference ----
    def camera_rays(self, req, stream=None):
        import torch
        rays = torch.empty((req.width * req.height, 8), dtype=torch.float32, device=torch.device("cuda", self.device))
        self._check(self.lib.nbvh_camera_rays(self.h, C.byref(req), _ptr(rays), _stream(stream)))
        return rays

    def run_inference(self, req, stream=None):
        import torch
        img = torch.empty((req.width * req.height, 12), dtype=torch.int32, device=torch.device("cuda", self.device))
        self._check(self.lib.nbvh_run_inference(self.h, C.byref(req), _ptr(img), _stream(stream)))
        return img

    def begin_tree_cut(self, options=None, start_depth=0):
        options = options if options is not None else tree_cut_options()
        self._check(self.lib.nbvh_begin_tree_cut(self.h, C.byref(options), start_depth))

    def tree_cut_info(self):
        info = abi.TreeCutInfo()
        self._check(self.lib.nbvh_get_tree_cut_info(self.h, C.byref(info)))
        return info

    def tree_cut(self):
        """(nodes uint32 [n, 8], stats uint32 [n, 4], node_map uint32 [n]) of the session."""
        n = C.c_uint32(0)
        self._check(self.lib.nbvh_get_tree_cut(self.h, None, None, None, C.byref(n)))
        nodes = np.empty((n.value, 8), np.uint32)
        stats = np.empty((n.value, 4), np.uint32)
        nmap = np.empty(n.value, np.uint32)
        self._check(self.lib.nbvh_get_tree_cut(self.h, _ptr(nodes), _ptr(stats), _ptr(nmap), C.byref(n)))
        return nodes, stats, nmap

    def set_tree_cut_stats(self, stats):
        st = np.ascontiguousarray(stats, np.uint32).reshape(-1, 4)
        self._check(self.lib.nbvh_set_tree_cut_stats(self.h, _ptr(st), len(st)))

    def training_batch(self, n=None):
        """(positions, targets, nodes, sample_loss) of the last run_optimisation step."""
        n = self.cfg.batch_size if n is None else n
        P = self.cfg.module.input_segment_points
        pos = np.empty((n, P, 3), np.float32)
        tgt = np.empty((n, 8), np.float32)
        nodes = np.empty(n, np.uint32)
        loss = np.empty(n, np.float32)
        self._check(self.lib.nbvh_get_training_batch(self.h, _ptr(pos), _ptr(tgt), _ptr(nodes), _ptr(loss), n))
        return pos, tgt, nodes, loss

    def import_neural_cut(self, path):
        self._check(self.lib.nbvh_import_neural_cut(self.h, str(path).encode()))

    def export_neural_cut(self, path):
        self._check(self.lib.nbvh_export_neural_cut(self.h, str(path).encode()))

    def import_tcnn_weights(self, path):
        """Parameters from a tcnn trainer JSON file (the reference's save_network_model format)."""
        self._check(self.lib.nbvh_import_tcnn_weights(self.h, str(path).encode()))

    def export_tcnn_weights(self, path):
        self._check(self.lib.nbvh_export_tcnn_weights(self.h, str(path).encode()))

    def render_path(self, req, stream=None):
        """Path-traced RGBA image (float32 [height * width, 4] on the device) and the rays traced."""
        import torch
        cam = req.camera
        img = torch.empty((cam.width * cam.height, 4), dtype=torch.float32, device=torch.device("cuda", self.device))
        traced = C.c_uint64(0)
        self._check(self.lib.nbvh_render_path(self.h, C.byref(req), _ptr(img), C.byref(traced), _stream(stream)))
        return img, traced.value

    # ---- checkpoints, stats ----
    def save(self, path):
        self._check(self.lib.nbvh_save(self.h, path.encode()))

    def load(self, path):
        self._check(self.lib.nbvh_load(self.h, path.encode()))
        L = ParamLayout()
        self._check(self.lib.nbvh_get_param_layout(self.h, C.byref(L)))
        self.layout = L

    def query_stats(self):
        s = QueryStats()
        self._check(self.lib.nbvh_last_query_stats(self.h, C.byref(s)))
        return s

    def set_kernel_profile(self, enable=True):
        """Time every wavefront-encoder launch of the following queries with CUDA events."""
        self._check(self.lib.nbvh_set_kernel_profile(self.h, 1 if enable else 0))

    def kernel_profile(self):
        """Encoder device time, launches and encoded segments of the last profiled query."""
        p = KernelProfile()
        self._check(self.lib.nbvh_last_kernel_profile(self.h, C.byref(p)))
        return p

    def last_kernel_time(self):
        ms = C.c_float(0)
        launches = C.c_uint32(0)
        self._check(self.lib.nbvh_last_kernel_time(self.h, C.byref(ms), C.byref(launches)))
        return ms.value, launches.value


def path_request(camera, spp=1, max_bounces=4, seed=0, ground_height=None, ground_albedo=(0.5, 0.5, 0.5),
                 sky_zenith=(0.35, 0.55, 1.0), sky_horizon=(1.0, 1.0, 1.0)):
    """nbvh_path_request over a render_request camera (ground plane off when ground_height is None)."""
    r = PathRequest()
    r.camera = camera
    r.spp, r.max_bounces, r.seed = spp, max_bounces, seed
    r.has_ground = 0 if ground_height is None else 1
    r.ground_height = 0.0 if ground_height is None else float(ground_height)
    for k in range(3):
        r.ground_albedo[k] = float(ground_albedo[k])
        r.sky_zenith[k] = float(sky_zenith[k])
        r.sky_horizon[k] = float(sky_horizon[k])
    return r


def render_request(width, height, origin, target, up=(0.0, 1.0, 0.0), yfov_degrees=45.0, sample_idx=0,
                   sample_offset=0):
    r = RenderRequest()
    r.width, r.height = width, height
    r.sample_idx, r.sample_offset = sample_idx, sample_offset
    for k in range(3):
        r.origin[k] = float(origin[k])
        r.target[k] = float(target[k])
        r.up[k] = float(up[k])
    r.yfov_degrees = float(yfov_degrees)
    return r


__all__ = [
    "NBVH", "NBVHError", "Config", "ParamLayout", "RenderRequest", "TrainStats", "QueryStats", "abi",
    "load_library", "default_config", "reference_default_config", "config_from_reference_json",
    "tree_cut_options_from_reference_json",
    "param_layout", "init_params",
    "build_bvh2_host", "build_neural_cut_host", "nodes_to_float", "render_request", "RAY_DTYPE", "HIT_DTYPE",
    "NEURAL_HIT_DTYPE", "SEGMENT_DTYPE", "FLT_MAX",
]


class Scene:
    """Instanced scene (nbvh_scene_*): models placed by 3x4 object-to-world transforms."""

    def __init__(self, device=0):
        self.lib = load_library()
        self.device = device
        self.s = C.c_void_p()
        _check(self.lib.nbvh_scene_create(device, C.byref(self.s)), None, self.lib)
        self.models = []  # keep the handles alive while the scene uses them

    def _check(self, st):
        if st != abi.NBVH_OK:
            raise NBVHError(st, self.lib.nbvh_scene_last_error(self.s).decode())

    def add_instance(self, model, object_to_world=None):
        m = np.eye(3, 4, dtype=np.float32) if object_to_world is None else np.ascontiguousarray(object_to_world,
                                                                                                np.float32)
        assert m.shape == (3, 4)
        iid = C.c_uint32(0)
        self._check(self.lib.nbvh_scene_add_instance(self.s, model.h, _ptr(m), C.byref(iid)))
        self.models.append(model)
        return iid.value

    def query_closest(self, rays, depth=1, out=None, stream=None):
        import torch
        n = rays.shape[0]
        out = torch.empty((n, 12), dtype=torch.int32, device=rays.device) if out is None else out
        self._check(self.lib.nbvh_scene_query_closest(self.s, _ptr(rays), n, depth, _ptr(out), _stream(stream)))
        return out

    def render_path(self, req, stream=None):
        import torch
        cam = req.camera
        img = torch.empty((cam.width * cam.height, 4), dtype=torch.float32, device=torch.device("cuda", self.device))
        traced = C.c_uint64(0)
        self._check(self.lib.nbvh_scene_render_path(self.s, C.byref(req), _ptr(img), C.byref(traced),
                                                    _stream(stream)))
        return img, traced.value

    def close(self):
        if self.s:
            self.lib.nbvh_scene_destroy(self.s)
            self.s = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """The serving loop (nbvh_server_*): continuous batching of query and render requests from
    many client threads against several resident models. Host buffers passed to submit must stay
    alive until wait returns."""

    def __init__(self, n_slots=4, hbm_budget_gb=150.0, max_batch_rays=1 << 22, use_graphs=True, autotune=True,
                 device=0, query_slots=0):
        self.lib = load_library()
        cfg = ServerConfig()
        _check(self.lib.nbvh_server_config_default(C.byref(cfg)), None)
        cfg.n_slots, cfg.max_batch_rays, cfg.query_slots = n_slots, max_batch_rays, query_slots
        cfg.hbm_budget_bytes = int(hbm_budget_gb * (1 << 30))
        cfg.use_graphs, cfg.autotune = int(use_graphs), int(autotune)
        s = C.c_void_p()
        st = self.lib.nbvh_server_create(C.byref(cfg), device, C.byref(s))
        if st != abi.NBVH_OK:
            raise NBVHError(st, self.lib.nbvh_status_string(st).decode())
        self.s = s
        self._keep = {}

    def _check(self, st):
        if st != abi.NBVH_OK:
            raise NBVHError(st, self.lib.nbvh_server_last_error(self.s).decode())

    def add_model(self, handle):
        mid = C.c_uint32(0)
        self._check(self.lib.nbvh_server_add_model(self.s, handle.h, C.byref(mid)))
        return mid.value

    def submit_query(self, model, rays_np, depth=1, hits=None):
        """`hits`: an optional caller-owned output array (len(rays) records of NEURAL_HIT_DTYPE, e.g. in
        page-locked memory); a new array is made otherwise."""
        rays = np.ascontiguousarray(rays_np, np.float32).reshape(-1, 8)
        if hits is None:
            hits = np.empty(len(rays), NEURAL_HIT_DTYPE)
        elif hits.dtype != NEURAL_HIT_DTYPE or hits.shape != (len(rays),) or not hits.flags.c_contiguous:
            raise ValueError("hits must be a contiguous array of len(rays) NEURAL_HIT_DTYPE records")
        r = Request()
        r.kind, r.model, r.n_rays, r.depth = 0, model, len(rays), depth
        r.h_rays, r.h_hits = rays.ctypes.data, hits.ctypes.data
        t = C.c_uint64(0)
        self._check(self.lib.nbvh_server_submit(self.s, C.byref(r), C.byref(t)))
        self._keep[t.value] = (rays, hits)
        return t.value

    def submit_render(self, model, path_req):
        cam = path_req.camera
        img = np.empty((cam.width * cam.height, 4), np.float32)
        r = Request()
        r.kind, r.model = 1, model
        r.render = path_req
        r.h_image = img.ctypes.data
        t = C.c_uint64(0)
        self._check(self.lib.nbvh_server_submit(self.s, C.byref(r), C.byref(t)))
        self._keep[t.value] = (img,)
        return t.value

    def wait(self, ticket, timeout_ms=60000):
        """(output array, RequestResult): hits for a query, the RGBA image for a render."""
        res = RequestResult()
        st = self.lib.nbvh_server_wait(self.s, ticket, timeout_ms, C.byref(res))
        if st != abi.NBVH_OK:
            raise NBVHError(st, self.lib.nbvh_server_last_error(self.s).decode())
        bufs = self._keep.pop(ticket)
        return bufs[-1], res

    def stats(self):
        st = ServerStats()
        self._check(self.lib.nbvh_server_get_stats(self.s, C.byref(st)))
        return st

    def reset_stats(self):
        self._check(self.lib.nbvh_server_reset_stats(self.s))

    def close(self):
        if getattr(self, "s", None):
            self.lib.nbvh_server_destroy(self.s)
            self.s = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
