"""ctypes mirror of include/nbvh.h (records, configuration structs and function prototypes)."""

import ctypes as C

NBVH_ABI_VERSION = 1

NBVH_OK, NBVH_EINVAL, NBVH_ENOMEM, NBVH_EDEVICE, NBVH_ETIMEOUT, NBVH_EOVERFLOW, NBVH_ESTATE, NBVH_EIO = range(8)
STATUS_NAMES = {
    0: "NBVH_OK", 1: "NBVH_EINVAL", 2: "NBVH_ENOMEM", 3: "NBVH_EDEVICE",
    4: "NBVH_ETIMEOUT", 5: "NBVH_EOVERFLOW", 6: "NBVH_ESTATE", 7: "NBVH_EIO",
}

HIT_VALID = 0x1
HIT_CLASSIC_FALLBACK = 0x2
HIT_STEP_CAP = 0x4

LOSS = {"RelativeL2": 0, "L2": 1, "RelativeL1": 2, "L1": 3, "BinaryCrossEntropy": 5, "LogL2": 6, "LHalf": 7}
SEGMENT = {"EquidistantInterior": 0, "EquidistantExterior": 1, "Uniform": 2}
PRECISION = {"fp16": 0, "bf16": 1, "fp8": 2}


class HashgridOptions(C.Structure):
    _fields_ = [("n_levels", C.c_int32), ("n_features_per_level", C.c_int32), ("log2_hashmap_size", C.c_int32),
                ("base_resolution", C.c_int32), ("per_level_scale", C.c_float)]


class NetworkOptions(C.Structure):
    _fields_ = [("n_neurons", C.c_int32), ("n_hidden_layers", C.c_int32), ("precision", C.c_int32)]


class OptimizerOptions(C.Structure):
    _fields_ = [("learning_rate", C.c_float), ("beta1", C.c_float), ("beta2", C.c_float), ("epsilon", C.c_float),
                ("l2_reg", C.c_float), ("decay_start", C.c_int32), ("decay_interval", C.c_int32),
                ("decay_base", C.c_float), ("loss_scale", C.c_float)]


class BvhConstants(C.Structure):
    _fields_ = [("inference_mint_epsilon", C.c_float), ("inference_maxt_epsilon", C.c_float),
                ("learning_mint_epsilon", C.c_float), ("learning_maxt_epsilon", C.c_float),
                ("sampling_bbox_scaling", C.c_float), ("fixed_node_dilation", C.c_float),
                ("node_extent_dilation", C.c_float), ("leaf_boundary_sampling_ratio", C.c_float),
                ("ignore_neural_blas", C.c_int32), ("max_training_bounces", C.c_int32),
                ("sample_cosine_weighted", C.c_int32), ("backface_bounce_training", C.c_int32),
                ("log2_bvh_max_traversals", C.c_int32)]


class OutputConstants(C.Structure):
    _fields_ = [("visibility_loss", C.c_int32), ("visibility_loss_scale", C.c_float),
                ("depth_loss", C.c_int32), ("depth_loss_scale", C.c_float),
                ("normal_loss", C.c_int32), ("normal_loss_scale", C.c_float),
                ("albedo_loss", C.c_int32), ("albedo_loss_scale", C.c_float),
                ("output_normal_linear_activation", C.c_int32), ("output_albedo_linear_activation", C.c_int32),
                ("visibility_masking_loss", C.c_int32), ("primary_visibility_threshold", C.c_float),
                ("secondary_visibility_threshold", C.c_float), ("depth_epsilon", C.c_float),
                ("fixed_depth_epsilon", C.c_float), ("learn_normal", C.c_int32), ("learn_albedo", C.c_int32)]


class ModuleConstants(C.Structure):
    _fields_ = [("input_segment_points", C.c_int32), ("segment_distribution", C.c_int32)]


class Config(C.Structure):
    _fields_ = [("abi_version", C.c_uint32), ("hashgrid", HashgridOptions), ("network", NetworkOptions),
                ("optimizer", OptimizerOptions), ("bvh", BvhConstants), ("output", OutputConstants),
                ("module", ModuleConstants), ("batch_size", C.c_uint32), ("neural_bvh_max_depth", C.c_uint32),
                ("max_traversal_steps", C.c_uint32), ("seed", C.c_uint32), ("fallback_margin", C.c_float),
                ("reserved", C.c_uint32 * 7)]


class ParamLayout(C.Structure):
    _fields_ = [("n_inputs", C.c_uint32), ("n_network_params", C.c_uint32), ("n_grid_entries", C.c_uint32),
                ("n_params", C.c_uint32), ("n_levels", C.c_uint32), ("level_offset", C.c_uint32 * 32),
                ("level_size", C.c_uint32 * 32), ("level_resolution", C.c_uint32 * 32),
                ("level_scale", C.c_float * 32), ("n_features_per_level", C.c_uint32)]


class TrainStats(C.Structure):
    _fields_ = [("steps_done", C.c_uint32), ("training_step", C.c_uint32), ("last_loss", C.c_float),
                ("mean_loss", C.c_float), ("learning_rate", C.c_float), ("ms_per_step", C.c_float)]


class TreeCutOptions(C.Structure):
    _fields_ = [("tree_cut_learning", C.c_int32), ("splitting_interval", C.c_int32),
                ("last_split_iteration", C.c_int32), ("start_split_num", C.c_int32), ("split_scaling", C.c_float),
                ("split_interval_scaling", C.c_float), ("num_lods_learned", C.c_int32),
                ("lod_decision_type", C.c_int32), ("training_node_survival", C.c_int32),
                ("survival_probability_scale", C.c_float), ("min_rr_survival_prob", C.c_float),
                ("reserved", C.c_uint32 * 5)]


class TreeCutInfo(C.Structure):
    _fields_ = [("active", C.c_uint32), ("learning", C.c_uint32), ("n_nodes", C.c_uint32), ("capacity", C.c_uint32),
                ("iteration", C.c_uint32), ("current_learned_lod", C.c_uint32), ("total_splits", C.c_uint32),
                ("max_depth", C.c_uint32), ("expected_nodes", C.c_uint32), ("max_node_loss", C.c_float),
                ("n_lod_nodes", C.c_uint32 * 7), ("reserved", C.c_uint32 * 3)]


class RenderRequest(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("sample_idx", C.c_uint32),
                ("sample_offset", C.c_uint32), ("origin", C.c_float * 3), ("target", C.c_float * 3),
                ("up", C.c_float * 3), ("yfov_degrees", C.c_float)]


class PathRequest(C.Structure):
    _fields_ = [("camera", RenderRequest), ("spp", C.c_uint32), ("max_bounces", C.c_uint32), ("seed", C.c_uint32),
                ("has_ground", C.c_int32), ("ground_height", C.c_float), ("ground_albedo", C.c_float * 3),
                ("sky_zenith", C.c_float * 3), ("sky_horizon", C.c_float * 3), ("reserved", C.c_uint32 * 4)]


class ServerConfig(C.Structure):
    _fields_ = [("n_slots", C.c_uint32), ("max_batch_rays", C.c_uint32), ("hbm_budget_bytes", C.c_uint64),
                ("use_graphs", C.c_uint32), ("autotune", C.c_uint32), ("query_slots", C.c_uint32),
                ("reserved", C.c_uint32 * 7)]


class Request(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("model", C.c_uint32), ("h_rays", C.c_void_p), ("n_rays", C.c_uint32),
                ("depth", C.c_uint32), ("h_hits", C.c_void_p), ("render", PathRequest), ("h_image", C.c_void_p)]


class RequestResult(C.Structure):
    _fields_ = [("status", C.c_int), ("latency_ms", C.c_double), ("queue_ms", C.c_double),
                ("rays_traced", C.c_uint64)]


class ServerStats(C.Structure):
    _fields_ = [("requests_done", C.c_uint64), ("rays_traced", C.c_uint64), ("batches", C.c_uint64),
                ("merged_requests", C.c_uint64), ("slot_capacity_rays", C.c_uint32),
                ("graphs_captured", C.c_uint64), ("graph_replays", C.c_uint64), ("p50_ms", C.c_double),
                ("p99_ms", C.c_double), ("mean_ms", C.c_double), ("max_ms", C.c_double), ("busy_seconds", C.c_double)]


class QueryStats(C.Structure):
    _fields_ = [("rays", C.c_uint32), ("segments", C.c_uint32), ("step_capped", C.c_uint32),
                ("stack_overflow", C.c_uint32), ("fallback", C.c_uint32)]


class KernelProfile(C.Structure):
    _fields_ = [("encode_ms", C.c_float), ("encode_launches", C.c_uint32), ("encoded_segments", C.c_uint32),
                ("segments", C.c_uint32), ("train_sample_ms", C.c_float), ("train_encode_ms", C.c_float),
                ("train_mlp_ms", C.c_float), ("train_scatter_ms", C.c_float), ("train_adam_ms", C.c_float),
                ("train_rows", C.c_uint32)]


P = C.c_void_p
U32 = C.c_uint32
I32 = C.c_int
ST = C.c_int
PU32 = C.POINTER(C.c_uint32)
PF = C.POINTER(C.c_float)
PCFG = C.POINTER(Config)

# name -> (restype, argtypes); every symbol declared in include/nbvh.h
PROTOTYPES = {
    "nbvh_config_default": (ST, [PCFG]),
    "nbvh_create": (ST, [PCFG, I32, C.POINTER(P)]),
    "nbvh_destroy": (ST, [P]),
    "nbvh_last_error": (C.c_char_p, [P]),
    "nbvh_status_string": (C.c_char_p, [ST]),
    "nbvh_abi_version": (U32, []),
    "nbvh_set_mesh": (ST, [P, P, U32, P, U32, P]),
    "nbvh_build_classic": (ST, [P]),
    "nbvh_get_classic_bvh": (ST, [P, P, PU32, P, PU32]),
    "nbvh_build_neural_cut": (ST, [P, U32]),
    "nbvh_get_neural_bvh": (ST, [P, P, PU32, P]),
    "nbvh_set_non_neural_leaves": (ST, [P, P, U32, I32]),
    "nbvh_set_ignore_neural_blas": (ST, [P, I32]),
    "nbvh_set_ray_ordering": (ST, [P, I32]),
    "nbvh_query_closest_classic": (ST, [P, P, U32, P, P]),
    "nbvh_query_any_classic": (ST, [P, P, U32, P, P]),
    "nbvh_query_closest_neural": (ST, [P, P, U32, U32, P, P]),
    "nbvh_query_closest_neural_noalloc": (ST, [P, P, U32, U32, P, P]),
    "nbvh_query_visibility_neural": (ST, [P, P, U32, U32, P, P]),
    "nbvh_query_closest_neural_host": (ST, [P, P, U32, U32, P]),
    "nbvh_query_closest_classic_host": (ST, [P, P, U32, P]),
    "nbvh_query_segments": (ST, [P, P, U32, U32, P, P, P]),
    "nbvh_get_param_layout": (ST, [P, C.POINTER(ParamLayout)]),
    "nbvh_get_params": (ST, [P, P]),
    "nbvh_set_params": (ST, [P, P]),
    "nbvh_network_inference": (ST, [P, P, U32, P, P]),
    "nbvh_mlp_inference": (ST, [P, P, U32, P, P]),
    "nbvh_encode": (ST, [P, P, U32, P, P]),
    "nbvh_compute_gradients": (ST, [P, P, P, U32, P, PF, P]),
    "nbvh_adam_step": (ST, [P, P, P]),
    "nbvh_generate_training_batch": (ST, [P, U32, U32, P, P, P, P]),
    "nbvh_run_optimisation": (ST, [P, U32, C.POINTER(TrainStats)]),
    "nbvh_scene_create": (ST, [C.c_int, C.POINTER(P)]),
    "nbvh_scene_destroy": (ST, [P]),
    "nbvh_scene_last_error": (C.c_char_p, [P]),
    "nbvh_scene_add_instance": (ST, [P, P, P, C.POINTER(C.c_uint32)]),
    "nbvh_scene_query_closest": (ST, [P, P, U32, U32, P, P]),
    "nbvh_scene_render_path": (ST, [P, C.POINTER(PathRequest), P, C.POINTER(C.c_uint64), P]),
    "nbvh_tree_cut_options_default": (ST, [C.POINTER(TreeCutOptions)]),
    "nbvh_split_schedule_host": (ST, [C.POINTER(TreeCutOptions), U32, U32, P, C.POINTER(C.c_uint32)]),
    "nbvh_begin_tree_cut": (ST, [P, C.POINTER(TreeCutOptions), U32]),
    "nbvh_get_tree_cut_info": (ST, [P, C.POINTER(TreeCutInfo)]),
    "nbvh_get_tree_cut": (ST, [P, P, P, P, C.POINTER(C.c_uint32)]),
    "nbvh_set_tree_cut_stats": (ST, [P, P, U32]),
    "nbvh_get_training_batch": (ST, [P, P, P, P, P, U32]),
    "nbvh_training_step": (U32, [P]),
    "nbvh_run_inference": (ST, [P, C.POINTER(RenderRequest), P, P]),
    "nbvh_camera_rays": (ST, [P, C.POINTER(RenderRequest), P, P]),
    "nbvh_render_path": (ST, [P, C.POINTER(PathRequest), P, C.POINTER(C.c_uint64), P]),
    "nbvh_import_neural_cut": (ST, [P, C.c_char_p]),
    "nbvh_export_neural_cut": (ST, [P, C.c_char_p]),
    "nbvh_read_nbvh_host": (ST, [C.c_char_p, P, C.POINTER(C.c_uint32)]),
    "nbvh_write_nbvh_host": (ST, [C.c_char_p, P, C.c_uint32]),
    "nbvh_server_config_default": (ST, [C.POINTER(ServerConfig)]),
    "nbvh_server_create": (ST, [C.POINTER(ServerConfig), C.c_int, C.POINTER(C.c_void_p)]),
    "nbvh_server_add_model": (ST, [P, P, C.POINTER(C.c_uint32)]),
    "nbvh_server_submit": (ST, [P, C.POINTER(Request), C.POINTER(C.c_uint64)]),
    "nbvh_server_wait": (ST, [P, C.c_uint64, C.c_uint32, C.POINTER(RequestResult)]),
    "nbvh_server_get_stats": (ST, [P, C.POINTER(ServerStats)]),
    "nbvh_server_reset_stats": (ST, [P]),
    "nbvh_server_last_error": (C.c_char_p, [P]),
    "nbvh_server_destroy": (ST, [P]),
    "nbvh_save": (ST, [P, C.c_char_p]),
    "nbvh_load": (ST, [P, C.c_char_p]),
    "nbvh_last_query_stats": (ST, [P, C.POINTER(QueryStats)]),
    "nbvh_last_kernel_time": (ST, [P, PF, PU32]),
    "nbvh_set_kernel_profile": (ST, [P, I32]),
    "nbvh_last_kernel_profile": (ST, [P, C.POINTER(KernelProfile)]),
    "nbvh_debug_set_wait_limit": (ST, [P, C.c_uint64]),
    "nbvh_debug_inject_stall": (ST, [P, I32]),
    "nbvh_debug_fail_allocations": (ST, [C.c_int64]),
    "nbvh_debug_alloc_count": (ST, [C.POINTER(C.c_uint64)]),
    "nbvh_debug_device_level_scales": (ST, [C.POINTER(Config), C.c_int, C.POINTER(C.c_float)]),
    "nbvh_import_tcnn_weights": (ST, [P, C.c_char_p]),
    "nbvh_export_tcnn_weights": (ST, [P, C.c_char_p]),
    "nbvh_read_tcnn_params_host": (ST, [C.c_char_p, PF, C.c_uint64, C.POINTER(C.c_uint64)]),
    "nbvh_write_tcnn_params_host": (ST, [C.c_char_p, PF, C.c_uint64]),
    "nbvh_build_bvh2_host": (ST, [P, U32, P, U32, P, PU32, P]),
    "nbvh_build_neural_cut_host": (ST, [P, U32, U32, P, PU32]),
    "nbvh_param_layout_host": (ST, [PCFG, C.POINTER(ParamLayout)]),
    "nbvh_init_params_host": (ST, [PCFG, P]),
    "nbvh_host_alloc": (ST, [C.c_size_t, C.POINTER(P)]),
    "nbvh_host_free": (ST, [P]),
}
