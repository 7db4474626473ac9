/*
 * nbvh.h -- C ABI of the GB300-native N-BVH ray-query library (libnbvh.so).
 *
 * This header is the drop-in boundary for the neural ray-query path of the N-BVH renderer
 * (WeiPhil/nbvh). The reference exposes that path as C++ classes whose state lives in CUDA
 * __constant__ globals; every entry point below replaces one member of that surface and cites it.
 *
 *   reference surface                                          entry point here
 *   --------------------------------------------------------   --------------------------------------
 *   NeuralBVHModule ctor / reinitialise_neural_model            nbvh_create
 *     (include/cuda/neural/neural_bvh_module.h:144-241,
 *      src/cuda/neural/neural_bvh_module.cu:118-263)
 *   CudaBackend::load_scene / build_blas                        nbvh_set_mesh, nbvh_build_classic
 *     (src/cuda/cuda_backend.cpp:138-310)
 *   NeuralBVHRenderer::build_and_upload_neural_bvh              nbvh_build_neural_cut
 *     (src/cuda/neural/neural_bvh_renderer_accel.cpp:504-557)
 *   non_neural_bvh_intersection -> CudaBVH2::intersect<false>   nbvh_query_closest_classic
 *     (src/cuda/neural/path/path_inference_kernels.cu:195-222,
 *      include/cuda/accel/bvh2.cuh:12-88)
 *   CudaBVH2::intersect<true> (shadow rays)                     nbvh_query_any_classic
 *   neural_bvh_traversal + process_neural_bvh_traversal_step    nbvh_query_closest_neural
 *     (src/cuda/neural/path/path_module.cu:54-137,
 *      src/cuda/neural/path/path_inference_kernels.cu:61-131)
 *   neural_node_traversal(visibility_query_only = true)         nbvh_query_visibility_neural
 *     (include/cuda/neural/neural_bvh_module_common.cuh:160-209)
 *   NeuralBVHRendererConstants::ignore_neural_blas              nbvh_set_ignore_neural_blas
 *     (include/cuda/neural/neural_bvh_renderer_constants.cuh:19,
 *      include/cuda/neural/neural_bvh_module_common.cuh:323)
 *   NeuralBVHRenderer::render, m_run_optimisation branch        nbvh_run_optimisation
 *     (src/cuda/neural/neural_bvh_renderer.cu:141-288)
 *   NeuralBVHRenderer::render, m_run_inference branch           nbvh_run_inference
 *     (src/cuda/neural/neural_bvh_renderer.cu:299-379)
 *   save_network_model / load_network_model (tcnn trainer      nbvh_export_tcnn_weights,
 *     JSON, src/cuda/neural/neural_bvh_renderer_init.cu:385-404) nbvh_import_tcnn_weights;
 *                                                               nbvh_save, nbvh_load (whole state)
 *   save_neural_bvh / load_neural_bvh (.nbvh neural cut)        nbvh_export_neural_cut,
 *     (src/cuda/neural/neural_bvh_renderer_accel.cpp:170-254)   nbvh_import_neural_cut
 *   tree-cut learning, BvhSplitScheduler, split / LoD steps      nbvh_begin_tree_cut,
 *     (src/cuda/neural/neural_bvh_renderer.cu:196-282,           nbvh_get_tree_cut_info,
 *      include/cuda/neural/utils/bvh_split_scheduler.h:13-145,   nbvh_split_schedule_host
 *      src/cuda/neural/neural_bvh_renderer_accel.cpp:256-441)
 *   tcnn FullyFusedMLP::inference (the network half)            nbvh_mlp_inference
 *     (src/cuda/neural/neural_bvh_module.cu:232-238)
 *   path module scatter + next traversal, Lambertian case       nbvh_render_path
 *   CudaTLAS instancing (include/cuda/accel/tlas.cuh:123-324)   nbvh_scene_* (instanced scenes)
 *     (src/cuda/neural/path/path_inference_kernels.cu:224-429)
 *   (no counterpart: one model per process)                     nbvh_server_* serving loop,
 *                                                               nbvh_query_closest_neural_noalloc
 *
 * Conventions.
 *  - Every call returns an nbvh_status; nothing throws or exits across this boundary. The
 *    reference throws (CUDA_CHECK, src/ntwr.h:30-39) or calls exit(2) (CUDA_SYNC_CHECK,
 *    src/ntwr.h:46-54); here the message of the last failure is kept per handle and returned by
 *    nbvh_last_error.
 *  - Buffers named d_* are device pointers on the handle's device; h_* are host pointers. Query
 *    calls are asynchronous on the given stream (NULL = the legacy default stream) unless stated.
 *  - A handle serialises its calls with an internal mutex: it is safe to call from several host
 *    threads, and two handles share no state (the reference keeps its state in __constant__
 *    globals, which allows one model per process).
 *  - The library has no CPU fallback: when the CUDA device is missing every call that needs it
 *    returns NBVH_EDEVICE.
 */
#ifndef NBVH_H
#define NBVH_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NBVH_ABI_VERSION 1u

typedef struct nbvh_handle nbvh_handle;
typedef struct CUstream_st *nbvh_stream; /* identical to cudaStream_t */

typedef enum nbvh_status {
    NBVH_OK        = 0,
    NBVH_EINVAL    = 1, /* bad argument, size or configuration */
    NBVH_ENOMEM    = 2, /* device or pinned-host allocation failed */
    NBVH_EDEVICE   = 3, /* CUDA runtime error or no usable device */
    NBVH_ETIMEOUT  = 4, /* a bounded device-side loop gave up (step cap reached) */
    NBVH_EOVERFLOW = 5, /* a traversal stack overflowed on the device */
    NBVH_ESTATE    = 6, /* call order violated (e.g. query before build) */
    NBVH_EIO       = 7  /* checkpoint file could not be read or written, or is malformed */
} nbvh_status;

/* ---------------------------------------------------------------------------------------------
 * Ray and hit records
 * ------------------------------------------------------------------------------------------- */

/* Ray3f (include/cuda/base/ray.cuh:65-77): origin, tmin (default 1e-4), direction, tmax
 * (default FLT_MAX). 32 bytes, 16-byte aligned arrays are loaded with two 128-bit loads. */
typedef struct nbvh_ray {
    float o[3];
    float tmin;
    float d[3];
    float tmax;
} nbvh_ray;

/* PreliminaryItsData (include/cuda/base/ray.cuh:22-35) without mesh_idx: t = FLT_MAX and
 * prim = 0xFFFFFFFF when the ray misses. u, v are the barycentrics of the reference's
 * Moller-Trumbore test (include/cuda/accel/bvh.cuh:98-136). 16 bytes. */
typedef struct nbvh_hit {
    float t;
    float u;
    float v;
    uint32_t prim;
} nbvh_hit;

#define NBVH_HIT_VALID 0x1u            /* the query found a surface */
#define NBVH_HIT_CLASSIC_FALLBACK 0x2u /* the answer came from the classic BLAS */
#define NBVH_HIT_STEP_CAP 0x4u         /* the neural loop hit max_traversal_steps for this ray */

/* NeuralTraversalResult (src/cuda/neural/path/path_inference_kernels.cu:14-32) plus the network
 * visibility of the accepted segment and the number of leaf segments inferred. 48 bytes. */
typedef struct nbvh_neural_hit {
    float t;          /* FLT_MAX when no hit */
    float normal[3];  /* normalize(2 * o[2:5] - 1) of the accepted segment */
    float albedo[3];  /* o[5:8] of the accepted segment */
    float visibility; /* sigmoid visibility output of the accepted segment (0 if none) */
    uint32_t flags;   /* NBVH_HIT_* */
    uint32_t segments;
    uint32_t prim;    /* classic prim id when NBVH_HIT_CLASSIC_FALLBACK, else 0xFFFFFFFF */
    uint32_t reserved;
} nbvh_neural_hit;

/* ---------------------------------------------------------------------------------------------
 * Configuration (keys mirror the reference JSON: bvh_constants, pt_output_constants,
 * bvh_module_constants, segment_encoding.hashgrid_options, network, optimizer)
 * ------------------------------------------------------------------------------------------- */

typedef enum nbvh_loss_type { /* loss_types, include/cuda/neural/utils/tcnn_config.h:23-36 */
    NBVH_LOSS_RELATIVE_L2 = 0,
    NBVH_LOSS_L2          = 1,
    NBVH_LOSS_RELATIVE_L1 = 2,
    NBVH_LOSS_L1          = 3,
    NBVH_LOSS_BCE         = 5,
    NBVH_LOSS_LOG_L2      = 6,
    NBVH_LOSS_L_HALF      = 7
} nbvh_loss_type;

typedef enum nbvh_segment_distribution { /* neural_bvh_module.h:23-25 */
    NBVH_SEGMENT_EQUIDISTANT_INTERIOR = 0,
    NBVH_SEGMENT_EQUIDISTANT_EXTERIOR = 1,
    NBVH_SEGMENT_UNIFORM              = 2
} nbvh_segment_distribution;

typedef enum nbvh_precision {
    NBVH_PRECISION_FP16 = 0, /* MLP operands FP16, FP32 accumulation */
    NBVH_PRECISION_BF16 = 1, /* MLP operands BF16, FP32 accumulation */
    NBVH_PRECISION_FP8  = 2  /* hidden 64x64 layers FP8-E4M3: weights e4m3(w * 2^6) / 2^6, their
                                input activations e4m3(a * 2^7) / 2^7 (ties to even, saturating);
                                first and last layers FP16. E4M3 values are exact in FP16, so the
                                FP16 tensor-core paths compute them; FP32 accumulation and master
                                weights, straight-through gradients */
} nbvh_precision;

/* HashGridOptions, include/cuda/neural/utils/tcnn_config.h:69-78. n_features_per_level is 2, 4 or
 * 8 (the reference default is 4); input_segment_points * n_levels * n_features_per_level must be a
 * multiple of 16 and at most 128. */
typedef struct nbvh_hashgrid_options {
    int32_t n_levels;
    int32_t n_features_per_level;
    int32_t log2_hashmap_size;
    int32_t base_resolution;
    float per_level_scale;
} nbvh_hashgrid_options;

/* NetworkOptions, tcnn_config.h:221-233: ReLU hidden layers, Sigmoid output, no biases.
 * n_neurons must be 64; n_hidden_layers in [1, 8]. */
typedef struct nbvh_network_options {
    int32_t n_neurons;
    int32_t n_hidden_layers;
    int32_t precision; /* nbvh_precision */
} nbvh_network_options;

/* OptimizerOptions (Adam wrapped in ExponentialDecay), tcnn_config.h:150-166 and
 * neural_bvh_module.cu:146-168. loss_scale multiplies the output gradient before the FP16
 * backward pass and is divided out in the Adam step. */
typedef struct nbvh_optimizer_options {
    float learning_rate;
    float beta1;
    float beta2;
    float epsilon;
    float l2_reg;
    int32_t decay_start;
    int32_t decay_interval;
    float decay_base;
    float loss_scale;
} nbvh_optimizer_options;

/* NeuralBVHRendererConstants, include/cuda/neural/neural_bvh_renderer_constants.cuh:13-46. */
typedef struct nbvh_bvh_constants {
    float inference_mint_epsilon;
    float inference_maxt_epsilon;
    float learning_mint_epsilon;
    float learning_maxt_epsilon;
    float sampling_bbox_scaling;
    float fixed_node_dilation;
    float node_extent_dilation;
    float leaf_boundary_sampling_ratio;
    int32_t ignore_neural_blas;
    int32_t max_training_bounces;
    int32_t sample_cosine_weighted;
    int32_t backface_bounce_training;
    int32_t log2_bvh_max_traversals;
} nbvh_bvh_constants;

/* PathTracingOutputConstants, include/cuda/neural/neural_bvh_module.h:243-302. The output
 * layout is fixed at visibility(1), LocalT depth(1), normal(3), albedo(3), padded to 16. */
typedef struct nbvh_output_constants {
    int32_t visibility_loss; /* nbvh_loss_type */
    float visibility_loss_scale;
    int32_t depth_loss;
    float depth_loss_scale;
    int32_t normal_loss;
    float normal_loss_scale;
    int32_t albedo_loss;
    float albedo_loss_scale;
    int32_t output_normal_linear_activation;
    int32_t output_albedo_linear_activation;
    int32_t visibility_masking_loss;
    float primary_visibility_threshold;
    float secondary_visibility_threshold;
    float depth_epsilon;
    float fixed_depth_epsilon;
    int32_t learn_normal; /* output_normal_dim == 3 */
    int32_t learn_albedo; /* output_albedo_dim == 3 */
} nbvh_output_constants;

/* NeuralBVHModuleConstants, include/cuda/neural/neural_bvh_module.h:79-131 (no direction input). */
typedef struct nbvh_module_constants {
    int32_t input_segment_points;
    int32_t segment_distribution; /* nbvh_segment_distribution */
} nbvh_module_constants;

typedef struct nbvh_config {
    uint32_t abi_version; /* NBVH_ABI_VERSION */
    nbvh_hashgrid_options hashgrid;
    nbvh_network_options network;
    nbvh_optimizer_options optimizer;
    nbvh_bvh_constants bvh;
    nbvh_output_constants output;
    nbvh_module_constants module;
    uint32_t batch_size;           /* training rays per step, power of two (renderer.h:193) */
    uint32_t neural_bvh_max_depth; /* fixed cut depth, m_neural_bvh_min_depth */
    uint32_t max_traversal_steps;  /* neural_bvh_module.h:200 (1000) */
    uint32_t seed;                 /* parameter initialisation and training-ray seed */
    float fallback_margin;         /* |visibility - threshold| < margin -> classic answer; 0 = off */
    uint32_t reserved[7];
} nbvh_config;

/* Fills the defaults of the reference (the tcnn_config.h / renderer-constant defaults) with the
 * hot-path network shape: 4 stratified points, 16 levels x 2 features x 2^19 entries,
 * resolution 16..2048, 64 x 4 ReLU MLP in FP16, batch 2^18, cut depth 10. */
nbvh_status nbvh_config_default(nbvh_config *cfg);

/* ---------------------------------------------------------------------------------------------
 * Lifetime, scene and acceleration structures
 * ------------------------------------------------------------------------------------------- */

nbvh_status nbvh_create(const nbvh_config *cfg, int device, nbvh_handle **out);
nbvh_status nbvh_destroy(nbvh_handle *h);
const char *nbvh_last_error(const nbvh_handle *h);
const char *nbvh_status_string(nbvh_status s);
uint32_t nbvh_abi_version(void);

/* Triangle mesh (host arrays; copied). albedo is per triangle (3 floats) or NULL for the
 * reference's default base colour 0.9 (include/base/material.h:54). */
nbvh_status nbvh_set_mesh(nbvh_handle *h, const float *h_vertices, uint32_t n_vertices,
                          const uint32_t *h_indices, uint32_t n_triangles, const float *h_albedo);

/* Builds the classic BVH2 on the host (binned SAH, leaves of 1-2 triangles, flat-axis boxes padded
 * by 1e-4 as cuda_backend.cpp:212-223) and uploads nodes plus pre-gathered triangle records. */
nbvh_status nbvh_build_classic(nbvh_handle *h);

/* Copies the classic BVH out (host): nodes as 8 x 32-bit words per node in the reference layout
 * {min.xyz, prim_count, max.xyz, left_or_prim_offset} (include/base/accel/bvh.h:66-72), and the
 * primitive index list. Pass NULL buffers to query the counts. */
nbvh_status nbvh_get_classic_bvh(const nbvh_handle *h, uint32_t *h_nodes, uint32_t *n_nodes,
                                 uint32_t *h_prim_indices, uint32_t *n_prim_indices);

/* Fixed tree cut of the classic BVH at max_depth (traverse_and_build_neural_bvh,
 * neural_bvh_renderer_accel.cpp:25-88): nodes with prim_count 0 (interior),
 * 1 (final leaf) or 8 (LoD-6 leaf). Also sets the neural scene box to the BVH root box. */
nbvh_status nbvh_build_neural_cut(nbvh_handle *h, uint32_t max_depth);
nbvh_status nbvh_get_neural_bvh(const nbvh_handle *h, uint32_t *h_nodes, uint32_t *n_nodes,
                                float *h_scene_bbox /* 6 floats: min, max */);

/* The reference's .nbvh neural-cut file (NeuralBVHRenderer::save_neural_bvh / load_neural_bvh,
 * src/cuda/neural/neural_bvh_renderer_accel.cpp:170-254; written through the madmann91/bvh v2
 * serializer): u64 node count, u64 1, per node 40 bytes {f32 min.x, max.x, min.y, max.y, min.z,
 * max.z, u64 first_id, u64 prim_count}, u64 0. Import replaces the handle's neural cut (the
 * classic BVH must be built: it gives the scene box); files that fail the size, header or tree
 * checks return NBVH_EIO. The host forms read / write 8 words per node in the nbvh_get_neural_bvh
 * layout (h_nodes NULL: count only; *n_nodes is the capacity on input). */
nbvh_status nbvh_import_neural_cut(nbvh_handle *h, const char *path);
nbvh_status nbvh_export_neural_cut(nbvh_handle *h, const char *path);
nbvh_status nbvh_read_nbvh_host(const char *path, uint32_t *h_nodes, uint32_t *n_nodes);
nbvh_status nbvh_write_nbvh_host(const char *path, const uint32_t *h_nodes, uint32_t n_nodes);

/* Marks neural leaves whose queries are answered by the classic BLAS (flag != 0). */
nbvh_status nbvh_set_non_neural_leaves(nbvh_handle *h, const uint32_t *h_node_ids, uint32_t n,
                                       int flag);
nbvh_status nbvh_set_ignore_neural_blas(nbvh_handle *h, int ignore);
/* Ray ordering (on by default; no counterpart in the reference): batches of 524,288 rays or more are
 * answered bin by bin, the bins being the direction octant x 8^3 cells of the ray origin over the
 * scene box grown by half its size on every side, so that the rays of a warp fetch the same nodes.
 * It changes no result, only the order in which the classic kernel and the neural query's first
 * pass take the rays. */
nbvh_status nbvh_set_ray_ordering(nbvh_handle *h, int enable);

/* ---------------------------------------------------------------------------------------------
 * Queries (device buffers, asynchronous on stream)
 * ------------------------------------------------------------------------------------------- */

nbvh_status nbvh_query_closest_classic(nbvh_handle *h, const nbvh_ray *d_rays, uint32_t n,
                                       nbvh_hit *d_hits, nbvh_stream stream);
nbvh_status nbvh_query_any_classic(nbvh_handle *h, const nbvh_ray *d_rays, uint32_t n,
                                   nbvh_hit *d_hits, nbvh_stream stream);

/* Neural closest hit. Rays with tmin != 1e-4 are accepted; the neural traversal always restarts
 * from -FLT_MAX as the reference does (neural_bvh2.cuh:185-189). depth: 1 = primary ray
 * (primary_visibility_threshold), > 1 = secondary. When ignore_neural_blas is set the call
 * answers from the classic BLAS and sets NBVH_HIT_CLASSIC_FALLBACK on every valid hit.
 * The neural queries are wavefronts whose length depends on the data: the host reads the count of
 * rays still traversing every few steps, so these two calls return after the work is done on the
 * stream (like the reference's host loop, path_module.cu:54-137), not asynchronously. */
nbvh_status nbvh_query_closest_neural(nbvh_handle *h, const nbvh_ray *d_rays, uint32_t n,
                                      uint32_t depth, nbvh_neural_hit *d_hits, nbvh_stream stream);
nbvh_status nbvh_query_visibility_neural(nbvh_handle *h, const nbvh_ray *d_rays, uint32_t n,
                                         uint32_t depth, nbvh_neural_hit *d_hits,
                                         nbvh_stream stream);

/* Same queries from host buffers, returning when h_hits is filled. Page-locked buffers (both
 * h_rays and h_hits from cudaHostAlloc / cudaHostRegister) are read and written by the kernels
 * directly over the host link, so the transfers overlap the query; other host memory is staged
 * through device buffers in chunks on two internal streams. */
nbvh_status nbvh_query_closest_neural_host(nbvh_handle *h, const nbvh_ray *h_rays, uint32_t n,
                                           uint32_t depth, nbvh_neural_hit *h_hits);
nbvh_status nbvh_query_closest_classic_host(nbvh_handle *h, const nbvh_ray *h_rays, uint32_t n,
                                            nbvh_hit *h_hits);

/* Leaf segments each ray enters, in traversal order, with current_maxt = FLT_MAX (the N-BVH
 * traversal alone, NeuralBVH2::intersect, neural_bvh2.cuh:170-292). Per ray up to max_segments
 * records {mint, maxt, node}; d_counts receives the total number entered. */
typedef struct nbvh_segment {
    float mint;
    float maxt;
    uint32_t node;
    uint32_t reserved;
} nbvh_segment;
nbvh_status nbvh_query_segments(nbvh_handle *h, const nbvh_ray *d_rays, uint32_t n,
                                uint32_t max_segments, nbvh_segment *d_segments,
                                uint32_t *d_counts, nbvh_stream stream);

/* ---------------------------------------------------------------------------------------------
 * Network: parameters, forward/backward kernels, optimisation
 * ------------------------------------------------------------------------------------------- */

/* Parameter layout (one flat FP32 vector, network first as tcnn orders it):
 *   W_0   [n_neurons][n_inputs]     n_inputs = input_segment_points * n_levels * F
 *   W_1.. [n_neurons][n_neurons]    (n_hidden_layers - 1 matrices)
 *   W_out [16][n_neurons]           rows 8..15 are padding and stay zero
 *   grid  [n_grid_entries][F]       levels concatenated; F = n_features_per_level
 */
typedef struct nbvh_param_layout {
    uint32_t n_inputs;
    uint32_t n_network_params;
    uint32_t n_grid_entries;
    uint32_t n_params; /* n_network_params + F * n_grid_entries */
    uint32_t n_levels;
    uint32_t level_offset[32];     /* in entries */
    uint32_t level_size[32];       /* entries in the level (hashed levels: 2^log2_hashmap_size) */
    uint32_t level_resolution[32]; /* grid points per axis */
    float level_scale[32];         /* position scale: pos = scale * x + 0.5 */
    uint32_t n_features_per_level; /* F: values per grid entry (2, 4 or 8) */
} nbvh_param_layout;
nbvh_status nbvh_get_param_layout(const nbvh_handle *h, nbvh_param_layout *out);

/* FP32 master parameters; set also refreshes the FP16 (or BF16/FP8) copies and resets Adam. */
nbvh_status nbvh_get_params(nbvh_handle *h, float *h_params);
nbvh_status nbvh_set_params(nbvh_handle *h, const float *h_params);

/* tcnn trainer weights as the reference saves and loads them (NeuralBVHRenderer::save_network_model /
 * load_network_model, src/cuda/neural/neural_bvh_renderer_init.cu:385-404: the JSON text of
 * trainer->serialize(false)): {"n_params": N, "params_type": "float" | "__half", "params_binary":
 * {"bytes": [...], "subtype": null}}, the binary value in nlohmann's text form (a bare byte array is
 * read too). The parameters are in tcnn's NetworkWithInputEncoding order, which is this library's:
 * the network matrices [out][in] row-major (first, hidden, output padded to 16 rows), then the hash
 * grid level by level, F values per entry. FP16 files are widened to FP32; export writes FP32.
 * Import replaces the handle's parameters like nbvh_set_params (N must equal its layout's
 * n_params, else NBVH_EINVAL; a malformed file gives NBVH_EIO). The host forms need no device:
 * read gives *n_params and, when h_params is not NULL and capacity suffices, the values. */
nbvh_status nbvh_import_tcnn_weights(nbvh_handle *h, const char *path);
nbvh_status nbvh_export_tcnn_weights(nbvh_handle *h, const char *path);
nbvh_status nbvh_read_tcnn_params_host(const char *path, float *h_params, uint64_t capacity, uint64_t *n_params);
nbvh_status nbvh_write_tcnn_params_host(const char *path, const float *h_params, uint64_t n_params);

/* Network inference on explicit inputs: d_positions holds n x points x 3 encoded positions in
 * [0,1]^3; d_outputs receives n x 8 sigmoid outputs. (Hash-grid encoding + fused MLP.) */
nbvh_status nbvh_network_inference(nbvh_handle *h, const float *d_positions, uint32_t n,
                                   float *d_outputs, nbvh_stream stream);

/* The fully fused MLP alone on encoded inputs (tcnn FullyFusedMLP::inference, configured at
 * src/cuda/neural/neural_bvh_module.cu:232-238; the network half of the reference's
 * NetworkWithInputEncoding): d_features holds n rows of n_inputs FP16 values (row-major, 16-byte
 * aligned); d_outputs receives n x 8 sigmoid outputs. Runs on the tcgen05 tensor cores with
 * TMA-fed tiles; returns after the kernel has finished (it reads back the kernel's status word). */
nbvh_status nbvh_mlp_inference(nbvh_handle *h, const uint16_t *d_features, uint32_t n, float *d_outputs,
                               nbvh_stream stream);

/* Hash-grid encoding alone: n x points x 3 positions -> n x n_inputs features (FP32 values of the
 * FP16 features fed to the MLP). */
nbvh_status nbvh_encode(nbvh_handle *h, const float *d_positions, uint32_t n, float *d_features,
                        nbvh_stream stream);

/* One forward + loss + backward pass on an explicit batch without the optimiser: writes the FP32
 * gradient of the mean loss w.r.t. every parameter (n_params floats, loss scale removed) and the
 * mean loss. targets: n x 8. */
nbvh_status nbvh_compute_gradients(nbvh_handle *h, const float *d_positions, const float *d_targets,
                                   uint32_t n, float *d_gradients, float *h_loss,
                                   nbvh_stream stream);

/* One Adam + ExponentialDecay step from an explicit FP32 gradient (n_params floats). */
nbvh_status nbvh_adam_step(nbvh_handle *h, const float *d_gradients, nbvh_stream stream);

/* Training rays generated and labelled on the device for a training step
 * (granular_sample_bvh_network_input_data, src/cuda/neural/neural_bvh_module_kernels.cu:119-264
 * with n_sub_batch = 2^log2_bvh_max_traversals). d_positions: n x points x 3, d_targets: n x 8,
 * d_nodes: sampled neural node per sample (may be NULL). */
nbvh_status nbvh_generate_training_batch(nbvh_handle *h, uint32_t training_step, uint32_t n,
                                         float *d_positions, float *d_targets, uint32_t *d_nodes,
                                         nbvh_stream stream);

typedef struct nbvh_train_stats {
    uint32_t steps_done;
    uint32_t training_step; /* total steps after the call */
    float last_loss;        /* mean loss of the last step */
    float mean_loss;        /* mean over the steps of this call */
    float learning_rate;    /* effective rate of the last step */
    float ms_per_step;      /* device time per step */
} nbvh_train_stats;

/* run-optimisation: `steps` training steps on device-generated, classic-labelled rays
 * (sample generation -> fused forward/loss/backward -> Adam). Synchronous; stats may be NULL. */
nbvh_status nbvh_run_optimisation(nbvh_handle *h, uint32_t steps, nbvh_train_stats *stats);
uint32_t nbvh_training_step(const nbvh_handle *h);

/* ---------------------------------------------------------------------------------------------
 * Learned tree cut (tree_cut_learning of NeuralBVHRenderer::render, neural_bvh_renderer.cu:196-282;
 * BvhSplitScheduler, include/cuda/neural/utils/bvh_split_scheduler.h:13-145; node survival,
 * neural_bvh_module_kernels.cu:184-199; split_neural_bvh_at / assign_lod_to_current_neural_leaf_nodes,
 * neural_bvh_renderer_accel.cpp:256-441)
 * ------------------------------------------------------------------------------------------- */

typedef struct nbvh_tree_cut_options {
    int32_t tree_cut_learning;        /* split leaves on the schedule below (m_tree_cut_learning) */
    int32_t splitting_interval;       /* bvh_split_scheduler: 50 */
    int32_t last_split_iteration;     /* 2000 */
    int32_t start_split_num;          /* 1 */
    float split_scaling;              /* 2 */
    float split_interval_scaling;     /* 2 */
    int32_t num_lods_learned;         /* bvh_constants.num_lods_learned: 1, at most 7 */
    int32_t lod_decision_type;        /* 0 EqualIterations, 1 EqualSplits */
    int32_t training_node_survival;   /* bvh_constants: 1 */
    float survival_probability_scale; /* 1 */
    float min_rr_survival_prob;       /* 0.005 */
    uint32_t reserved[5];
} nbvh_tree_cut_options;

typedef struct nbvh_tree_cut_info {
    uint32_t active;              /* a tree-cut session exists on the handle */
    uint32_t learning;            /* splits still scheduled */
    uint32_t n_nodes;
    uint32_t capacity;            /* classic node count: a cut never holds more */
    uint32_t iteration;           /* training steps since nbvh_begin_tree_cut */
    uint32_t current_learned_lod;
    uint32_t total_splits;
    uint32_t max_depth;
    uint32_t expected_nodes;      /* the scheduler's node count after last_split_iteration */
    float max_node_loss;          /* heuristic maximum the next step's node survival uses */
    uint32_t n_lod_nodes[7];      /* n_bvh_lod_nodes: node count when each LoD was assigned */
    uint32_t reserved[3];
} nbvh_tree_cut_info;

/* The reference defaults (tree_cut_learning and training_node_survival on). */
nbvh_status nbvh_tree_cut_options_default(nbvh_tree_cut_options *o);

/* The split schedule alone (BvhSplitScheduler::update_stats_and_reset): splits requested at each
 * of n_iterations steps, capped by the leaves of the growing cut (h_splits may be NULL), and the
 * node count reached from start_nodes. No device needed. */
nbvh_status nbvh_split_schedule_host(const nbvh_tree_cut_options *o, uint32_t start_nodes, uint32_t n_iterations,
                                     uint32_t *h_splits, uint32_t *expected_nodes);

/* Starts a tree-cut session: the cut is rebuilt at start_depth (m_neural_bvh_min_depth, 0 = the
 * root alone) with its leaves at the coarsest LoD, per-node statistics are reset, and every later
 * nbvh_run_optimisation step also accounts each sample's loss to its node, applies node survival
 * to the sampler and, while learning, splits the leaves with the largest loss heuristic on the
 * schedule (and assigns LoDs when num_lods_learned > 1). The session ends when the cut is replaced
 * (nbvh_build_neural_cut, nbvh_import_neural_cut, nbvh_load, a new mesh). */
nbvh_status nbvh_begin_tree_cut(nbvh_handle *h, const nbvh_tree_cut_options *o, uint32_t start_depth);
nbvh_status nbvh_get_tree_cut_info(nbvh_handle *h, nbvh_tree_cut_info *info);

/* The session's device state: nodes (8 words each), statistics (4 words each: f32 loss,
 * iter_alive, depth, samples) and the classic node of each neural node; any pointer may be NULL;
 * *n_nodes is the capacity on input and the node count on output. */
nbvh_status nbvh_get_tree_cut(nbvh_handle *h, uint32_t *h_nodes, uint32_t *h_stats, uint32_t *h_node_map,
                              uint32_t *n_nodes);
/* Replaces the per-node statistics (n_nodes must be the session's node count), e.g. to resume. */
nbvh_status nbvh_set_tree_cut_stats(nbvh_handle *h, const uint32_t *h_stats, uint32_t n_nodes);

/* The batch of the last nbvh_run_optimisation step (host copies; any pointer may be NULL):
 * positions n x points x 3, targets n x 8, sampled node per sample, and per sample the sum of its
 * output channels' loss values (tcnn's L matrix summed over channels, already divided by n_total). */
nbvh_status nbvh_get_training_batch(nbvh_handle *h, float *h_positions, float *h_targets, uint32_t *h_nodes,
                                    float *h_sample_loss, uint32_t n);

/* run-inference: renders one frame of primary rays from a pinhole camera (camera_raygen,
 * include/cuda/neural/neural_bvh_renderer_kernels.cuh:74-79; CudaBackend::update_camera,
 * src/cuda/cuda_backend.cpp:595-611) through the neural query, into a headless buffer. */
typedef struct nbvh_render_request {
    uint32_t width, height;
    uint32_t sample_idx; /* get_lcg_rng(sample_idx, sample_offset, pixel) jitter */
    uint32_t sample_offset;
    float origin[3];
    float target[3];
    float up[3];
    float yfov_degrees;
} nbvh_render_request;
/* d_image: width*height nbvh_neural_hit records (row-major, y down). */
nbvh_status nbvh_run_inference(nbvh_handle *h, const nbvh_render_request *req,
                               nbvh_neural_hit *d_image, nbvh_stream stream);
/* The primary rays run_inference traces (for checking against a host restatement). */
nbvh_status nbvh_camera_rays(nbvh_handle *h, const nbvh_render_request *req, nbvh_ray *d_rays,
                             nbvh_stream stream);

/* Hybrid path tracing over the neural BLAS: the Lambertian case of the reference's path module
 * (scatter + next traversal, src/cuda/neural/path/path_inference_kernels.cu:224-429; raygen
 * 540-567) as a wavefront. spp camera paths per pixel (camera_raygen jitter with the sample index
 * running over the spp samples), up to max_bounces Lambertian bounces (cosine-sampled) on neural
 * surfaces (network albedo and normal) and on an optional classic ground plane y = ground_height,
 * lit only by an analytic sky (horizon colour to zenith colour with the direction's height). */
typedef struct nbvh_path_request {
    nbvh_render_request camera;
    uint32_t spp;
    uint32_t max_bounces; /* bounces after the camera ray's first hit */
    uint32_t seed;
    int32_t has_ground;
    float ground_height;
    float ground_albedo[3];
    float sky_zenith[3];
    float sky_horizon[3];
    uint32_t reserved[4];
} nbvh_path_request;
/* d_image: width*height RGBA float32 (row-major, y down), the mean over the spp paths of each
 * pixel. rays_traced (may be NULL) receives the number of rays queried over all bounces.
 * Synchronous: returns when the image is written. */
nbvh_status nbvh_render_path(nbvh_handle *h, const nbvh_path_request *req, float *d_image, uint64_t *rays_traced,
                             nbvh_stream stream);

/* ---------------------------------------------------------------------------------------------
 * Instanced scenes: several models (handles) placed by affine transforms and queried or path
 * traced together. The reference renders one neural BLAS with pre-transformed vertices
 * (src/cuda/neural/neural_bvh_renderer_init.cu:23-25, src/base/scene.cpp:38-44); its TLAS walk is
 * include/cuda/accel/tlas.cuh:123-324. Each query tests the rays against every instance's world
 * box and answers those that enter it with the instance's model in object space; the record kept
 * is the closest hit in world space, with the instance in `reserved` (~0 when nothing is hit) and
 * the segment counts of all instances summed. Models must not change while a scene call runs.
 * ------------------------------------------------------------------------------------------- */

typedef struct nbvh_scene nbvh_scene;

nbvh_status nbvh_scene_create(int device, nbvh_scene **out);
nbvh_status nbvh_scene_destroy(nbvh_scene *scene);
const char *nbvh_scene_last_error(const nbvh_scene *scene);
/* object_to_world: row-major 3x4 [A | b], A invertible; world = A * object + b. */
nbvh_status nbvh_scene_add_instance(nbvh_scene *scene, nbvh_handle *model, const float *object_to_world,
                                    uint32_t *instance_id);
nbvh_status nbvh_scene_query_closest(nbvh_scene *scene, const nbvh_ray *d_rays, uint32_t n, uint32_t depth,
                                     nbvh_neural_hit *d_hits, nbvh_stream stream);
/* The Lambertian path tracer of nbvh_render_path over the instanced scene (plus the classic ground
 * plane and the sky of the request). */
nbvh_status nbvh_scene_render_path(nbvh_scene *scene, const nbvh_path_request *req, float *d_image,
                                   uint64_t *rays_traced, nbvh_stream stream);


/* ---------------------------------------------------------------------------------------------
 * Serving loop (no counterpart in the reference, which renders one model in one process).
 *
 * A server takes ray-query and render requests of uneven size from many client threads against
 * several resident models and runs them with continuous batching on one GPU: n_slots worker
 * threads, each with its own stream and buffers sized from hbm_budget_bytes, take the oldest
 * pending work as soon as they are free; pending queries for the same model and depth are merged
 * into one batch up to a slot's capacity, larger requests are split. Query batches are padded to
 * power-of-two buckets whose first part runs as a captured CUDA graph; launch parameters per
 * bucket are chosen by timing when a model is added (autotune). Models must be added before the
 * first request; while the server holds a handle, the handle's own calls must not run.
 * ------------------------------------------------------------------------------------------- */
typedef struct nbvh_server nbvh_server;

typedef struct nbvh_server_config {
    uint32_t n_slots;          /* batches in flight at once (default 4) */
    uint32_t max_batch_rays;   /* rays (or render paths) one batch may hold (default 2^22) */
    uint64_t hbm_budget_bytes; /* device memory all slots' buffers may take together (default 150 GiB) */
    uint32_t use_graphs;       /* replay captured CUDA graphs per batch-size bucket (default 1) */
    uint32_t autotune;         /* time the launch-parameter candidates per bucket (default 1) */
    uint32_t query_slots;      /* of the n_slots, how many take query requests only, on streams of the
                                  device's highest priority (default 0; must be < n_slots when renders
                                  are submitted). Every slot takes pending query work before renders. */
    uint32_t reserved[7];
} nbvh_server_config;

typedef enum nbvh_request_kind { NBVH_REQUEST_QUERY = 0, NBVH_REQUEST_RENDER = 1 } nbvh_request_kind;

typedef struct nbvh_request {
    uint32_t kind;  /* nbvh_request_kind */
    uint32_t model; /* id from nbvh_server_add_model */
    /* NBVH_REQUEST_QUERY: closest-hit neural query of n_rays host rays into host hits */
    const nbvh_ray *h_rays;
    uint32_t n_rays;
    uint32_t depth; /* 1 = primary threshold, > 1 secondary (0 is taken as 1) */
    nbvh_neural_hit *h_hits;
    /* NBVH_REQUEST_RENDER: nbvh_render_path into h_image (width * height RGBA float32) */
    nbvh_path_request render;
    float *h_image;
} nbvh_request;

typedef struct nbvh_request_result {
    nbvh_status status;
    double latency_ms; /* submit -> done */
    double queue_ms;   /* submit -> first batch started */
    uint64_t rays_traced;
} nbvh_request_result;

typedef struct nbvh_server_stats {
    uint64_t requests_done;
    uint64_t rays_traced;
    uint64_t batches;
    uint64_t merged_requests; /* requests that joined another request's batch */
    uint32_t slot_capacity_rays;
    uint64_t graphs_captured; /* query shapes running from a captured CUDA graph */
    uint64_t graph_replays;   /* batches answered by replaying one */
    double p50_ms, p99_ms, mean_ms, max_ms; /* request latency, submit -> done */
    double busy_seconds;                    /* first submit -> last completion */
} nbvh_server_stats;

nbvh_status nbvh_server_config_default(nbvh_server_config *cfg);
nbvh_status nbvh_server_create(const nbvh_server_config *cfg, int device, nbvh_server **out);
/* Registers a built handle (scene, cuts and parameters stay on the device); sizes every slot
 * for it and autotunes its buckets. The handle must not be changed while requests for it are in
 * flight; between requests it may be (more training, a new or learned cut): a slot whose captured
 * graphs hold arrays that moved since then drops and recaptures them. */
nbvh_status nbvh_server_add_model(nbvh_server *s, nbvh_handle *model, uint32_t *model_id);
/* Queues a request (the host buffers must stay valid until it is done); returns at once. */
nbvh_status nbvh_server_submit(nbvh_server *s, const nbvh_request *req, uint64_t *ticket);
/* Waits up to timeout_ms for a request; NBVH_ETIMEOUT if it is not done yet (wait again). */
nbvh_status nbvh_server_wait(nbvh_server *s, uint64_t ticket, uint32_t timeout_ms, nbvh_request_result *result);
nbvh_status nbvh_server_get_stats(nbvh_server *s, nbvh_server_stats *out);
nbvh_status nbvh_server_reset_stats(nbvh_server *s);
const char *nbvh_server_last_error(nbvh_server *s);
/* Finishes the queued work, stops the workers and frees the server (not the models). */
nbvh_status nbvh_server_destroy(nbvh_server *s);

/* Checkpoint: config, mesh, both BVHs, FP32 parameters, Adam moments and step (own format). */
nbvh_status nbvh_save(nbvh_handle *h, const char *path);
nbvh_status nbvh_load(nbvh_handle *h, const char *path);

/* Counters of the last query call (device-side step caps and stack overflows). */
typedef struct nbvh_query_stats {
    uint32_t rays;
    uint32_t segments;       /* leaf segments inferred */
    uint32_t step_capped;    /* rays stopped by max_traversal_steps */
    uint32_t stack_overflow; /* rays whose traversal stack overflowed */
    uint32_t fallback;       /* rays answered by the classic BLAS */
} nbvh_query_stats;
nbvh_status nbvh_last_query_stats(nbvh_handle *h, nbvh_query_stats *out);

/* Device time (ms, CUDA events on the launching stream) of the dominant kernel of the last query
 * or training call, and the number of kernels that call launched. */
nbvh_status nbvh_last_kernel_time(nbvh_handle *h, float *ms, uint32_t *launches);

/* Per-kernel timing of the dominant kernel of the neural query, the wavefront hash-grid encoder
 * (no counterpart in the reference, whose kernels are timed by external profilers). While enabled,
 * every neural query on the handle's own first context records a CUDA event pair around each
 * encoder launch on the query's stream (up to 32 launches), and the last step of each
 * nbvh_run_optimisation call records its phases; nbvh_last_kernel_profile waits for the events
 * and reports the summed device time, the launches and the segments they encoded, and the
 * training step's phases. Disabled by default (the events cost a few microseconds per query). */
typedef struct nbvh_kernel_profile {
    float encode_ms;           /* summed device time of the encoder launches */
    uint32_t encode_launches;  /* encoder launches of the last query */
    uint32_t encoded_segments; /* leaf segments those launches encoded */
    uint32_t segments;         /* all leaf segments of the last query (the tail kernel encodes the rest) */
    /* the last step of the last nbvh_run_optimisation call made while profiling was on (device
     * time of each phase; train_rows = 0 if there was none) */
    float train_sample_ms;     /* training-ray generation and labels */
    float train_encode_ms;     /* hash-grid encoding of the rows (and the packing of the matrices) */
    float train_mlp_ms;        /* tensor-core forward, loss, backward and weight gradients */
    float train_scatter_ms;    /* hash-grid gradient scatter */
    float train_adam_ms;       /* Adam */
    uint32_t train_rows;
} nbvh_kernel_profile;
nbvh_status nbvh_set_kernel_profile(nbvh_handle *h, int enable);
nbvh_status nbvh_last_kernel_profile(nbvh_handle *h, nbvh_kernel_profile *out);

/* Failure-path testing (no counterpart in the reference, which stops the process on a CUDA error,
 * include/ntwr.h:30-54).
 * nbvh_debug_set_wait_limit: time limit of the phase waits inside this handle's tensor-core
 * kernels (the fused MLP of the queries and of nbvh_mlp_inference, the training kernel), in
 * nanoseconds; 0 restores the default of one second. A wait that runs out makes the kernel record
 * the failure, let the copies and MMAs it has in flight finish, release its tensor memory and
 * return; the call then fails with NBVH_ETIMEOUT and the handle stays usable.
 * nbvh_debug_inject_stall: while enabled, every tensor-core kernel this handle launches first waits
 * on an mbarrier that nothing arrives at, so that its wait runs out after the wait limit (a wait
 * that would otherwise never end, made on purpose and bounded).
 * nbvh_debug_fail_allocations: every device allocation the library makes after the next `after`
 * ones fails as if the device were out of memory (the call reports NBVH_ENOMEM); a negative value
 * switches this off. Process-wide.
 * nbvh_debug_alloc_count: device allocations the library has made so far (process-wide).
 * nbvh_debug_device_level_scales: the configuration's hash-grid level scales (n_levels values)
 * evaluated on `device` the way tcnn's encoding kernels do, exp2f(l * log2f(per_level_scale)) *
 * base_resolution - 1 with CUDA's exp2f; the library itself takes them from the host's exp2f
 * (nbvh_get_param_layout, level_scale), so that a layout needs no GPU. A test compares the two. */
nbvh_status nbvh_debug_set_wait_limit(nbvh_handle *h, uint64_t ns);
nbvh_status nbvh_debug_inject_stall(nbvh_handle *h, int enable);
nbvh_status nbvh_debug_fail_allocations(int64_t after);
nbvh_status nbvh_debug_alloc_count(uint64_t *out);
nbvh_status nbvh_debug_device_level_scales(const nbvh_config *cfg, int device, float *out);

/* ---------------------------------------------------------------------------------------------
 * Allocation-free neural query. This entry point has no counterpart in the reference.
 *
 * Same result as nbvh_query_closest_neural, for callers that must not allocate memory while they
 * trace: a renderer whose GPU memory is reserved up front and must not grow mid-frame, or a host
 * thread that may not take the device-wide synchronisation an allocation can cause. The ordinary
 * query grows per-handle buffers to the largest batch seen; this one allocates nothing. Its
 * scratch (the per-ray traversal state, the network inputs and outputs of a step, the node order,
 * the fallback list and the counters: about 660 bytes per ray, 10.8 MB in all) is one fixed buffer
 * of NBVH_NOALLOC_MAX_RAYS rays compiled into the library, one copy per device, created when the
 * library's device code is loaded.
 *  - n must be at most NBVH_NOALLOC_MAX_RAYS; a larger n returns NBVH_EINVAL and launches nothing.
 *    Split larger batches into several calls.
 *  - The call cannot be captured into a CUDA graph: it reads the list lengths back to the host
 *    between steps and synchronises its stream before it returns.
 *  - The first call on each device loads the library's device code there if nothing has yet
 *    (setup); a first call with n = 0 does only that, so a caller can take the setup's latency
 *    before its first frame. Every call looks the buffer's address up again (no allocation), so
 *    handles created after a reset of the device (cudaDeviceReset) find it where the reloaded
 *    code put it; handles created before the reset are invalid, as for every call.
 *  - Each call zeroes the counters it uses before its first kernel; nothing relies on the buffer's
 *    contents from an earlier call.
 *  - There is one buffer per device, shared by every handle on it. Calls that overlap in time on
 *    the same device (several host threads, or several handles) race on it: serialise them. A call
 *    returns only after its work on the stream is complete, so consecutive calls are safe.
 *  - nbvh_last_query_stats and nbvh_last_kernel_time do not report this call.
 * ------------------------------------------------------------------------------------------- */
#define NBVH_NOALLOC_MAX_RAYS 16384u
nbvh_status nbvh_query_closest_neural_noalloc(nbvh_handle *h, const nbvh_ray *d_rays, uint32_t n,
                                              uint32_t depth, nbvh_neural_hit *d_hits,
                                              nbvh_stream stream);

/* ---------------------------------------------------------------------------------------------
 * Host-only utilities (no CUDA device needed)
 * ------------------------------------------------------------------------------------------- */

/* The classic BVH builder of nbvh_build_classic, run on host arrays. h_nodes receives
 * 8 words per node (capacity 2 * n_triangles nodes), h_prim_indices n_triangles entries. */
nbvh_status nbvh_build_bvh2_host(const float *h_vertices, uint32_t n_vertices, const uint32_t *h_indices,
                                 uint32_t n_triangles, uint32_t *h_nodes, uint32_t *n_nodes,
                                 uint32_t *h_prim_indices);
/* The fixed neural cut of nbvh_build_neural_cut; *n_neural_nodes is the capacity on input. */
nbvh_status nbvh_build_neural_cut_host(const uint32_t *h_nodes, uint32_t n_nodes, uint32_t max_depth,
                                       uint32_t *h_neural_nodes, uint32_t *n_neural_nodes);
/* Parameter layout and seeded initial parameters (Xavier-uniform matrices, grid U(-1e-4, 1e-4))
 * that nbvh_create would produce for cfg. */
nbvh_status nbvh_param_layout_host(const nbvh_config *cfg, nbvh_param_layout *out);
nbvh_status nbvh_init_params_host(const nbvh_config *cfg, float *h_params);

/* Page-locked host memory for the *_host queries (cudaHostAlloc / cudaFreeHost). */
nbvh_status nbvh_host_alloc(size_t bytes, void **out);
nbvh_status nbvh_host_free(void *ptr);

#ifdef __cplusplus
}
#endif

#endif /* NBVH_H */
