"""TEST INFRASTRUCTURE ONLY: ctypes bindings of the CPU oracle (oracle/nbvh_oracle.c).

Imported by tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg; never by the
product. Parity status of the oracle: unpinned (see nbvh_oracle.h).
"""

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "nbvh_oracle.c")
LIB = os.path.join(HERE, "liboracle.so")
FLAGS = ["-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-std=c11"]


def build(force=False):
    """Compiles the oracle with gcc (no FMA contraction, no fast math)."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(
            os.path.getmtime(SRC), os.path.getmtime(os.path.join(HERE, "nbvh_oracle.h"))):
        return LIB
    subprocess.run(["gcc"] + FLAGS + ["-o", LIB, SRC, "-lm", "-lpthread"], check=True)
    return LIB


class ClassicScene(C.Structure):
    _fields_ = [("nodes", C.c_void_p), ("n_nodes", C.c_uint32), ("prim_indices", C.c_void_p),
                ("vertices", C.c_void_p), ("indices", C.c_void_p), ("n_triangles", C.c_uint32)]


class NeuralConsts(C.Structure):
    _fields_ = [("inference_mint_epsilon", C.c_float), ("inference_maxt_epsilon", C.c_float),
                ("learning_mint_epsilon", C.c_float), ("learning_maxt_epsilon", C.c_float),
                ("sampling_bbox_scaling", C.c_float), ("fixed_node_dilation", C.c_float),
                ("node_extent_dilation", C.c_float), ("leaf_boundary_sampling_ratio", C.c_float),
                ("primary_visibility_threshold", C.c_float), ("secondary_visibility_threshold", C.c_float),
                ("depth_epsilon", C.c_float), ("fixed_depth_epsilon", C.c_float),
                ("input_segment_points", C.c_int32), ("segment_distribution", C.c_int32),
                ("bvh_lod", C.c_uint32), ("max_traversal_steps", C.c_uint32)]


class Network(C.Structure):
    _fields_ = [("n_levels", C.c_uint32), ("n_points", C.c_uint32), ("n_inputs", C.c_uint32),
                ("n_neurons", C.c_uint32), ("n_hidden_layers", C.c_uint32), ("level_offset", C.c_void_p),
                ("level_size", C.c_void_p), ("level_resolution", C.c_void_p), ("level_scale", C.c_void_p),
                ("grid_f16", C.c_void_p), ("weights_f16", C.c_void_p), ("exact", C.c_int32),
                ("grid_f32", C.c_void_p), ("weights_f32", C.c_void_p), ("bf16", C.c_int32), ("fp8", C.c_int32),
                ("n_features", C.c_uint32)]


class PathParams(C.Structure):
    _fields_ = [("origin", C.c_float * 3), ("du", C.c_float * 3), ("dv", C.c_float * 3), ("tl", C.c_float * 3),
                ("width", C.c_uint32), ("height", C.c_uint32), ("spp", C.c_uint32), ("sample_base", C.c_uint32),
                ("sample_offset", C.c_uint32), ("seed", C.c_uint32), ("max_bounces", C.c_uint32),
                ("has_ground", C.c_uint32), ("ground_y", C.c_float), ("ground_albedo", C.c_float * 3),
                ("sky_zenith", C.c_float * 3), ("sky_horizon", C.c_float * 3)]


class NeuralScene(C.Structure):
    _fields_ = [("neural_nodes", C.c_void_p), ("scene_min", C.c_float * 3), ("scene_max", C.c_float * 3),
                ("non_neural", C.c_void_p)]


class LossConsts(C.Structure):
    _fields_ = [("visibility_loss", C.c_int32), ("depth_loss", C.c_int32), ("normal_loss", C.c_int32),
                ("albedo_loss", C.c_int32), ("visibility_loss_scale", C.c_float), ("depth_loss_scale", C.c_float),
                ("normal_loss_scale", C.c_float), ("albedo_loss_scale", C.c_float),
                ("output_normal_linear_activation", C.c_int32), ("output_albedo_linear_activation", C.c_int32),
                ("visibility_masking_loss", C.c_int32), ("learn_normal", C.c_int32), ("learn_albedo", C.c_int32)]


class NodeSurvival(C.Structure):
    _fields_ = [("stats", C.c_void_p), ("current_max_loss", C.c_float), ("survival_probability_scale", C.c_float),
                ("min_survival_prob", C.c_float), ("current_learned_lod", C.c_uint32), ("enabled", C.c_int32)]


class SplitScheduler:
    """BvhSplitScheduler (include/cuda/neural/utils/bvh_split_scheduler.h:13-145), restated."""

    def __init__(self, splitting_interval=50, last_split_iteration=2000, start_split_num=1, split_scaling=2.0,
                 split_interval_scaling=2.0, lod_decision_type=0):
        self.splitting_interval = splitting_interval
        self.last_split_iteration = last_split_iteration
        self.start_split_num = start_split_num
        self.split_scaling = np.float32(split_scaling)
        self.split_interval_scaling = np.float32(split_interval_scaling)
        self.lod_decision_type = lod_decision_type
        self.total_splits_expected = 0
        self._reset()

    def _reset(self):
        self.current_num_splits = self.start_split_num
        self.current_splitting_interval = self.splitting_interval
        self.current_total_splits = 0

    def get_bvh_splits(self, it):
        if it == 0:
            self._reset()
        if it > self.last_split_iteration:
            return 0
        n = 0
        if it % self.splitting_interval == 0:
            n = self.current_num_splits
            self.current_total_splits += n
        if it % self.current_splitting_interval == 0:
            # int *= float: the product in float, truncated back to int
            self.current_num_splits = int(np.float32(self.current_num_splits) * self.split_scaling)
            self.current_splitting_interval = int(np.float32(self.current_splitting_interval) *
                                                  self.split_interval_scaling)
        return n

    def expected(self, start_nodes, n_iterations):
        """update_stats_and_reset: splits per iteration (capped by the leaves) and the node count."""
        nodes, total, graph = start_nodes, 0, []
        for it in range(n_iterations):
            leaves = (nodes + 1) // 2
            k = self.get_bvh_splits(it)
            if k > 0:
                k = min(k, leaves)
                total += k
                nodes += 2 * k
            graph.append(total)
        self.total_splits_expected = total
        self._reset()
        return graph, nodes

    def should_assign_new_lod(self, it, current_lod, num_lods_learned, max_lods=7):
        if self.lod_decision_type == 0:
            nxt = (max_lods - current_lod) * self.last_split_iteration // num_lods_learned
            assign = nxt <= it
        else:
            nxt = (max_lods - current_lod) * self.total_splits_expected // num_lods_learned
            assign = nxt <= self.current_total_splits
        return assign or it >= self.last_split_iteration


def bf16_bits(x):
    """bfloat16 bits of float32 values, round to nearest even (finite values)."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = u + 0x7FFF + ((u >> 16) & 1)
    return (u >> 16).astype(np.uint16)


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Oracle:
    """Owns the oracle library plus the arrays referenced by the structs handed to it."""

    def __init__(self, path=None):
        self.lib = C.CDLL(path or build())
        L = self.lib
        L.orc_murmur_mix.restype = C.c_uint32
        L.orc_murmur_mix.argtypes = [C.c_uint32, C.c_uint32]
        L.orc_murmur_finalize.restype = C.c_uint32
        L.orc_murmur_finalize.argtypes = [C.c_uint32]
        L.orc_lcg_seed.restype = C.c_uint32
        L.orc_lcg_seed.argtypes = [C.c_uint32] * 3
        L.orc_lcg_randomf.restype = C.c_float
        L.orc_lcg_randomf.argtypes = [C.POINTER(C.c_uint32)]
        L.orc_sincos_turns.argtypes = [C.c_float, C.POINTER(C.c_float), C.POINTER(C.c_float)]
        L.orc_f32_to_f16.restype = C.c_uint16
        L.orc_f32_to_f16.argtypes = [C.c_float]
        L.orc_f16_to_f32.restype = C.c_float
        L.orc_f16_to_f32.argtypes = [C.c_uint16]
        L.orc_path_trace.restype = C.c_uint64
        self._keep = []

    # ---- RNG ----
    def lcg_seed(self, index, frame, linear):
        return self.lib.orc_lcg_seed(index, frame, linear)

    def lcg_stream(self, index, frame, linear, n):
        s = C.c_uint32(self.lcg_seed(index, frame, linear))
        return np.array([self.lib.orc_lcg_randomf(C.byref(s)) for _ in range(n)], np.float32)

    def sincos_turns(self, u):
        s, c = C.c_float(), C.c_float()
        self.lib.orc_sincos_turns(u, C.byref(s), C.byref(c))
        return s.value, c.value

    # ---- scenes ----
    def classic_scene(self, nodes, prims, vertices, indices):
        nodes = np.ascontiguousarray(nodes, np.uint32)
        prims = np.ascontiguousarray(prims, np.uint32)
        v = np.ascontiguousarray(vertices, np.float32)
        t = np.ascontiguousarray(indices, np.uint32)
        self._keep += [nodes, prims, v, t]
        return ClassicScene(_p(nodes).value, len(nodes), _p(prims).value, _p(v).value, _p(t).value, len(t))

    def neural_scene(self, neural_nodes, bbox, non_neural=None):
        nn = np.ascontiguousarray(neural_nodes, np.uint32)
        self._keep.append(nn)
        s = NeuralScene()
        s.neural_nodes = _p(nn).value
        for k in range(3):
            s.scene_min[k] = float(bbox[k])
            s.scene_max[k] = float(bbox[3 + k])
        if non_neural is not None:
            f = np.ascontiguousarray(non_neural, np.uint8)
            self._keep.append(f)
            s.non_neural = _p(f).value
        return s

    @staticmethod
    def neural_consts(cfg):
        c = NeuralConsts()
        for k in ("inference_mint_epsilon", "inference_maxt_epsilon", "learning_mint_epsilon",
                  "learning_maxt_epsilon", "sampling_bbox_scaling", "fixed_node_dilation", "node_extent_dilation",
                  "leaf_boundary_sampling_ratio"):
            setattr(c, k, getattr(cfg.bvh, k))
        for k in ("primary_visibility_threshold", "secondary_visibility_threshold", "depth_epsilon",
                  "fixed_depth_epsilon"):
            setattr(c, k, getattr(cfg.output, k))
        c.input_segment_points = cfg.module.input_segment_points
        c.segment_distribution = cfg.module.segment_distribution
        c.bvh_lod = 0
        c.max_traversal_steps = cfg.max_traversal_steps
        return c

    @staticmethod
    def loss_consts(cfg):
        lc = LossConsts()
        o = cfg.output
        for k in ("visibility_loss", "depth_loss", "normal_loss", "albedo_loss", "visibility_loss_scale",
                  "depth_loss_scale", "normal_loss_scale", "albedo_loss_scale", "output_normal_linear_activation",
                  "output_albedo_linear_activation", "visibility_masking_loss", "learn_normal", "learn_albedo"):
            setattr(lc, k, getattr(o, k))
        return lc

    def network(self, cfg, layout, params, exact=False):
        """Network struct over FP32 parameters: the network matrices rounded to the configured MLP
        precision (FP16; BF16 when cfg.network.precision is 1; FP8-E4M3 hidden matrices and their
        inputs when it is 2) and the grid to FP16, unless exact."""
        params = np.ascontiguousarray(params, np.float32)
        nl = layout.n_levels
        off = np.array(layout.level_offset[:nl], np.uint32)
        size = np.array(layout.level_size[:nl], np.uint32)
        res = np.array(layout.level_resolution[:nl], np.uint32)
        scale = np.array(layout.level_scale[:nl], np.float32)
        nnet = layout.n_network_params
        w32 = np.ascontiguousarray(params[:nnet])
        g32 = np.ascontiguousarray(params[nnet:])
        bf16 = int(cfg.network.precision) == 1
        w16 = bf16_bits(w32) if bf16 else w32.astype(np.float16).view(np.uint16)
        g16 = g32.astype(np.float16).view(np.uint16)
        self._keep += [off, size, res, scale, w32, g32, w16, g16]
        net = Network()
        net.n_levels = nl
        net.n_points = cfg.module.input_segment_points
        net.n_inputs = layout.n_inputs
        net.n_neurons = cfg.network.n_neurons
        net.n_hidden_layers = cfg.network.n_hidden_layers
        net.level_offset, net.level_size = _p(off).value, _p(size).value
        net.level_resolution, net.level_scale = _p(res).value, _p(scale).value
        net.grid_f16, net.weights_f16 = _p(g16).value, _p(w16).value
        net.exact = 1 if exact else 0
        net.grid_f32, net.weights_f32 = _p(g32).value, _p(w32).value
        net.bf16 = 1 if bf16 else 0
        net.fp8 = 1 if int(cfg.network.precision) == 2 else 0
        net.n_features = cfg.hashgrid.n_features_per_level
        return net

    # ---- queries ----
    def classic_query(self, scene, rays, any_hit=False, threads=1, stats=False):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        n = len(rays)
        hits = np.empty((n, 4), np.uint32)
        st = np.empty((n, 2), np.uint32) if stats else None
        self.lib.orc_classic_query(C.byref(scene), _p(rays), C.c_uint32(n), C.c_int(int(any_hit)), _p(hits), _p(st),
                                   C.c_int(threads))
        return (hits, st) if stats else hits

    def fp64_closest(self, scene, rays):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        n = len(rays)
        t = np.empty(n, np.float64)
        prim = np.empty(n, np.uint32)
        self.lib.orc_fp64_closest(C.byref(scene), _p(rays), C.c_uint32(n), _p(t), _p(prim))
        return t, prim

    def neural_segments(self, neural_nodes, consts, rays, max_segments):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        nn = np.ascontiguousarray(neural_nodes, np.uint32)
        n = len(rays)
        segs = np.zeros((n, max_segments, 4), np.uint32)
        counts = np.empty(n, np.uint32)
        self.lib.orc_neural_segments(_p(nn), C.byref(consts), _p(rays), C.c_uint32(n), C.c_uint32(max_segments),
                                     _p(segs), _p(counts))
        return segs, counts

    def encode(self, net, positions):
        pos = np.ascontiguousarray(positions, np.float32)
        n = pos.shape[0]
        out = np.empty((n, net.n_inputs), np.float32)
        self.lib.orc_encode(C.byref(net), _p(pos), C.c_uint32(n), _p(out))
        return out

    def network_inference(self, net, positions, threads=1):
        pos = np.ascontiguousarray(positions, np.float32)
        n = pos.shape[0]
        out = np.empty((n, 16), np.float32)
        self.lib.orc_network_inference(C.byref(net), _p(pos), C.c_uint32(n), _p(out), C.c_int(threads))
        return out

    def neural_query(self, nscene, net, consts, rays, depth=1, visibility_only=False, classic=None,
                     fallback_margin=0.0, threads=1):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        n = len(rays)
        hits = np.empty((n, 12), np.uint32)
        self.lib.orc_neural_query(C.byref(nscene), C.byref(net), C.byref(consts),
                                  C.byref(classic) if classic is not None else None, C.c_float(fallback_margin),
                                  _p(rays), C.c_uint32(n), C.c_uint32(depth), C.c_int(int(visibility_only)),
                                  _p(hits), C.c_int(threads))
        return hits

    def training_batch(self, nscene, cscene, albedo, consts, training_step, batch_size, n):
        P = consts.input_segment_points
        pos = np.empty((n, P, 3), np.float32)
        tgt = np.empty((n, 8), np.float32)
        nodes = np.empty(n, np.uint32)
        alb = None if albedo is None else np.ascontiguousarray(albedo, np.float32)
        self.lib.orc_generate_training_batch(C.byref(nscene), C.byref(cscene), _p(alb), C.byref(consts),
                                             C.c_uint32(training_step), C.c_uint32(batch_size), C.c_uint32(n),
                                             _p(pos), _p(tgt), _p(nodes))
        return pos, tgt, nodes

    def training_batch_rr(self, nscene, cscene, albedo, consts, training_step, batch_size, n, stats, max_loss,
                          prev_positions, prev_targets, scale=1.0, min_prob=0.005, learned_lod=6, enabled=True):
        """Training batch with node survival: rejected slots keep prev_positions / prev_targets."""
        pos = np.array(prev_positions, np.float32).reshape(n, consts.input_segment_points, 3)
        tgt = np.array(prev_targets, np.float32).reshape(n, 8)
        nodes = np.empty(n, np.uint32)
        st = np.ascontiguousarray(stats, np.uint32).reshape(-1, 4)
        rr = NodeSurvival(_p(st), float(max_loss), float(scale), float(min_prob), int(learned_lod), int(enabled))
        alb = None if albedo is None else np.ascontiguousarray(albedo, np.float32)
        self.lib.orc_generate_training_batch_rr(C.byref(nscene), C.byref(cscene), _p(alb), C.byref(consts),
                                                C.c_uint32(training_step), C.c_uint32(batch_size), C.c_uint32(n),
                                                _p(pos), _p(tgt), _p(nodes), C.byref(rr))
        return pos, tgt, nodes

    def e4m3_round(self, x):
        f = self.lib.orc_e4m3_round
        f.restype = C.c_float
        f.argtypes = [C.c_float]
        return np.array([f(float(v)) for v in np.asarray(x, np.float32).ravel()], np.float32)

    def loss_heuristic(self, stats):
        st = np.ascontiguousarray(stats, np.uint32).reshape(-1, 4)
        f = self.lib.orc_loss_heuristic
        f.restype = C.c_float
        return np.array([f(_p(st[i:i + 1])) for i in range(len(st))], np.float32)

    def tree_cut_accumulate(self, stats, values, sample_nodes, dims):
        st = np.array(stats, np.uint32).reshape(-1, 4)
        v = np.ascontiguousarray(values, np.float32)
        nd = np.ascontiguousarray(sample_nodes, np.uint32)
        self.lib.orc_tree_cut_accumulate(_p(st), _p(v), _p(nd), C.c_uint32(len(nd)), C.c_uint32(dims))
        return st

    def tree_cut_decisions(self, nodes, stats, k):
        nodes = np.ascontiguousarray(nodes, np.uint32)
        st = np.array(stats, np.uint32).reshape(-1, 4)
        mx = np.zeros(max(k, 1), np.float32)
        idx = np.zeros(max(k, 1), np.uint32)
        self.lib.orc_tree_cut_decisions(_p(nodes), C.c_uint32(len(nodes)), _p(st), C.c_uint32(k), _p(mx), _p(idx))
        return mx[:k], idx[:k], st

    def tree_cut_split(self, nodes, stats, node_map, classic_nodes, split_indices, k, lod, capacity):
        n = len(nodes)
        out = np.zeros((capacity, 8), np.uint32)
        out[:n] = nodes
        st = np.zeros((capacity, 4), np.uint32)
        st[:n] = np.asarray(stats, np.uint32).reshape(-1, 4)
        nm = np.zeros(capacity, np.uint32)
        nm[:n] = node_map
        cn = np.ascontiguousarray(classic_nodes, np.uint32)
        si = np.ascontiguousarray(split_indices, np.uint32)
        count = C.c_uint32(n)
        self.lib.orc_tree_cut_split.restype = C.c_uint32
        m = self.lib.orc_tree_cut_split(_p(out), C.byref(count), C.c_uint32(capacity), _p(st), _p(nm), _p(cn),
                                        _p(si), C.c_uint32(k), C.c_uint32(lod))
        c = count.value
        return out[:c], st[:c], nm[:c], m

    def tree_cut_assign_lod(self, nodes, lod):
        out = np.array(nodes, np.uint32)
        self.lib.orc_tree_cut_assign_lod(_p(out), C.c_uint32(len(out)), C.c_uint32(lod))
        return out

    def composite_loss(self, lc, predictions, targets, loss_scale=1.0):
        pred = np.ascontiguousarray(predictions, np.float32).reshape(-1, 16)
        tgt = np.ascontiguousarray(targets, np.float32).reshape(-1, 8)
        n = len(pred)
        vals = np.empty((n, 16), np.float32)
        grads = np.empty((n, 16), np.float32)
        self.lib.orc_composite_loss(C.byref(lc), _p(pred), _p(tgt), C.c_uint32(n), C.c_float(loss_scale), _p(vals),
                                    _p(grads))
        return vals, grads

    def compute_gradients(self, net, lc, positions, targets, n_params, loss_scale=128.0, fp16_backward=True):
        pos = np.ascontiguousarray(positions, np.float32)
        tgt = np.ascontiguousarray(targets, np.float32)
        g = np.empty(n_params, np.float64)
        loss = C.c_double(0)
        self.lib.orc_compute_gradients(C.byref(net), C.byref(lc), _p(pos), _p(tgt), C.c_uint32(len(pos)),
                                       C.c_float(loss_scale), _p(g), C.byref(loss), C.c_int(int(fp16_backward)))
        return g, loss.value

    def adam_step(self, params, m, v, grad, step, cfg):
        o = cfg.optimizer
        self.lib.orc_adam_step(_p(params), _p(m), _p(v), _p(np.ascontiguousarray(grad, np.float32)),
                               C.c_uint32(len(params)), C.c_uint32(step), C.c_float(o.learning_rate),
                               C.c_float(o.beta1), C.c_float(o.beta2), C.c_float(o.epsilon), C.c_float(o.l2_reg),
                               C.c_int32(o.decay_start), C.c_int32(o.decay_interval), C.c_float(o.decay_base))

    def grid_layout(self, n_levels, log2_hashmap_size, base_resolution, per_level_scale):
        """Level offsets, sizes, resolutions and position scales of the hash grid (tcnn's conventions)."""
        off, size, res = (np.empty(n_levels, np.uint32) for _ in range(3))
        scale = np.empty(n_levels, np.float32)
        total = C.c_uint32(0)
        self.lib.orc_grid_layout(C.c_uint32(n_levels), C.c_uint32(log2_hashmap_size), C.c_uint32(base_resolution),
                                 C.c_float(per_level_scale), _p(off), _p(size), _p(res), _p(scale), C.byref(total))
        return off, size, res, scale, total.value

    def path_trace(self, nscene, net, consts, req, sample_base=None, threads=1):
        """One path-traced frame of an nbvh_path_request (the library's k_path.cu restated): RGBA
        image [height * width, 4] and the rays traced. sample_base defaults to camera.sample_idx *
        spp, as nbvh_render_path uses."""
        cam = req.camera
        p = PathParams()
        du, dv, tl = (C.c_float * 3)(), (C.c_float * 3)(), (C.c_float * 3)()
        o = np.array(cam.origin[:], np.float32)
        t = np.array(cam.target[:], np.float32)
        u = np.array(cam.up[:], np.float32)
        self.lib.orc_camera_basis(C.c_uint32(cam.width), C.c_uint32(cam.height), _p(o), _p(t), _p(u),
                                  C.c_float(cam.yfov_degrees), du, dv, tl)
        for k in range(3):
            p.origin[k], p.du[k], p.dv[k], p.tl[k] = cam.origin[k], du[k], dv[k], tl[k]
            p.ground_albedo[k], p.sky_zenith[k], p.sky_horizon[k] = (req.ground_albedo[k], req.sky_zenith[k],
                                                                     req.sky_horizon[k])
        p.width, p.height, p.spp = cam.width, cam.height, req.spp
        p.sample_base = cam.sample_idx * req.spp if sample_base is None else sample_base
        p.sample_offset, p.seed, p.max_bounces = cam.sample_offset, req.seed, req.max_bounces
        p.has_ground, p.ground_y = 1 if req.has_ground else 0, req.ground_height
        img = np.empty((cam.width * cam.height, 4), np.float32)
        traced = self.lib.orc_path_trace(C.byref(nscene), C.byref(net), C.byref(consts), C.byref(p), _p(img),
                                         C.c_int(threads))
        return img, int(traced)

    def camera_rays(self, req):
        n = req.width * req.height
        rays = np.empty((n, 8), np.float32)
        o = np.array(req.origin[:], np.float32)
        t = np.array(req.target[:], np.float32)
        u = np.array(req.up[:], np.float32)
        self.lib.orc_camera_rays(C.c_uint32(req.width), C.c_uint32(req.height), C.c_uint32(req.sample_idx),
                                 C.c_uint32(req.sample_offset), _p(o), _p(t), _p(u), C.c_float(req.yfov_degrees),
                                 _p(rays))
        return rays
