/*
 * nbvh_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of the N-BVH ray-query path of WeiPhil/nbvh, used by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg as the checker of libnbvh. Nothing in
 * the product links or calls this library.
 *
 * Parity status: UNPINNED. The reference ships no tests, golden vectors or fixtures, and its path
 * cannot be compiled here (glm, madmann91/bvh and the tiny-cuda-nn fork are empty submodules), so
 * this restatement is checked against its own independent Python restatement of the same
 * reference lines (tests/golden/make_golden.py) and against mathematical identities (FP64
 * brute-force ray/triangle, finite-difference gradients), not against reference outputs.
 *
 * Arithmetic is FP32 with a fixed operation order and no contraction (-ffp-contract=off); where
 * the reference writes a double literal (1e-3 in the LocalT depth code) the expression is
 * evaluated in double as C++ does. Network accumulation is in double.
 */
#ifndef NBVH_ORACLE_H
#define NBVH_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* --- RNG: include/cuda/utils/lcg_rng.cuh:12-79 --- */
uint32_t orc_murmur_mix(uint32_t hash, uint32_t k);
uint32_t orc_murmur_finalize(uint32_t hash);
uint32_t orc_lcg_seed(uint32_t index, uint32_t frame, uint32_t linear);
float orc_lcg_randomf(uint32_t *state);
void orc_sincos_turns(float u, float *s, float *c);

/* --- classic BVH2 closest / any hit: include/cuda/accel/bvh2.cuh:12-88, bvh.cuh:98-136 --- */
typedef struct orc_classic_scene {
    const uint32_t *nodes; /* 8 words per node: min.xyz, prim_count, max.xyz, left_or_prim_offset */
    uint32_t n_nodes;
    const uint32_t *prim_indices;
    const float *vertices;    /* 3 per vertex */
    const uint32_t *indices;  /* 3 per triangle */
    uint32_t n_triangles;
} orc_classic_scene;

/* rays: 8 floats each {o, tmin, d, tmax}; hits: 4 words each {t, u, v, prim}.
 * stats (optional, 2 per ray): child boxes tested, triangles tested. */
void orc_classic_query(const orc_classic_scene *scene, const float *rays, uint32_t n, int any_hit,
                       uint32_t *hits, uint32_t *stats, int n_threads);

/* FP64 Moller-Trumbore over every triangle (adjudicator for grazing/tie rays):
 * hit t (FLT_MAX-like 1e300 on miss) and the lowest prim index at the minimum t. */
void orc_fp64_closest(const orc_classic_scene *scene, const float *rays, uint32_t n, double *t,
                      uint32_t *prim);

/* --- neural BVH2 traversal: include/cuda/neural/accel/neural_bvh2.cuh:170-292 --- */
typedef struct orc_neural_consts {
    float inference_mint_epsilon, inference_maxt_epsilon;
    float learning_mint_epsilon, learning_maxt_epsilon;
    float sampling_bbox_scaling;
    float fixed_node_dilation, node_extent_dilation;
    float leaf_boundary_sampling_ratio;
    float primary_visibility_threshold, secondary_visibility_threshold;
    float depth_epsilon, fixed_depth_epsilon;
    int32_t input_segment_points, segment_distribution;
    uint32_t bvh_lod;
    uint32_t max_traversal_steps;
} orc_neural_consts;

/* Segments entered (current_maxt = FLT_MAX), as nbvh_query_segments. segs: 4 words per record. */
void orc_neural_segments(const uint32_t *neural_nodes, const orc_neural_consts *c, const float *rays,
                         uint32_t n, uint32_t max_segments, uint32_t *segs, uint32_t *counts);

/* --- hash grid + MLP (behaviour of the tcnn calls at neural_bvh_module.cu:170-262) --- */
typedef struct orc_network {
    uint32_t n_levels;
    uint32_t n_points;
    uint32_t n_inputs;   /* n_points * n_levels * n_features */
    uint32_t n_neurons;  /* 64 */
    uint32_t n_hidden_layers;
    const uint32_t *level_offset;
    const uint32_t *level_size;
    const uint32_t *level_resolution;
    const float *level_scale;
    const uint16_t *grid_f16;   /* n_grid_entries x n_features half bits */
    const uint16_t *weights_f16; /* network matrices as laid out by nbvh_param_layout */
    /* exact mode (finite-difference checks): FP32 parameters, no FP16 rounding anywhere */
    int32_t exact;
    const float *grid_f32;
    const float *weights_f32;
    /* MLP precision: 0 = FP16 operands (weights_f16 holds FP16 bits), 1 = BF16 operands
     * (weights_f16 holds BF16 bits; encoded features, hidden activations and backward gradients are
     * rounded to BF16). The grid table is FP16 either way. */
    int32_t bf16;
    /* FP8 mode (MLP operands FP16 otherwise): the hidden 64x64 matrices hold FP8-E4M3 values at
     * scale 2^6 (e4m3(w * 64) / 64 of the FP32 weights) and the activations entering them are
     * FP8-E4M3 values at scale 2^7 (e4m3(a * 128) / 128). */
    int32_t fp8;
    /* features per hash-grid level (HashGridOptions::n_features_per_level): 2, 4 or 8; 0 reads as 2 */
    uint32_t n_features;
} orc_network;

/* Nearest FP8-E4M3 value (ties to even, saturating at +-448, subnormals on the 2^-9 grid). */
float orc_e4m3_round(float x);

void orc_grid_layout(uint32_t n_levels, uint32_t log2_hashmap_size, uint32_t base_resolution,
                     float per_level_scale, uint32_t *offset, uint32_t *size, uint32_t *resolution,
                     float *scale, uint32_t *total_entries);

uint16_t orc_f32_to_f16(float f);
float orc_f16_to_f32(uint16_t h);
uint16_t orc_f32_to_bf16(float f);
float orc_bf16_to_f32(uint16_t b);

/* positions: n x points x 3; features: n x n_inputs (FP32 values before FP16 rounding) */
void orc_encode(const orc_network *net, const float *positions, uint32_t n, float *features);
/* features rounded to FP16 then the MLP; outputs: n x 16 (sigmoid), hidden activations FP16. */
void orc_network_inference(const orc_network *net, const float *positions, uint32_t n,
                           float *outputs, int n_threads);

/* --- full neural queries: path_module.cu:54-137, path_inference_kernels.cu:61-131,
 *     neural_bvh_module_common.cuh:23-209, neural_bvh_module_kernels.cu:10-97,266-303 --- */
typedef struct orc_neural_scene {
    const uint32_t *neural_nodes;
    float scene_min[3], scene_max[3];
    const uint8_t *non_neural; /* per node flag or NULL */
} orc_neural_scene;

/* hits: 12 words per ray, the nbvh_neural_hit layout. classic answers for fallback rays come from
 * `classic` (may be NULL when no fallback is configured). */
void orc_neural_query(const orc_neural_scene *scene, const orc_network *net,
                      const orc_neural_consts *c, const orc_classic_scene *classic,
                      float fallback_margin, const float *rays, uint32_t n, uint32_t depth,
                      int visibility_only, uint32_t *hits, int n_threads);

/* decode_depth_estimate, LocalT branch (neural_bvh_module_common.cuh:23-58) */
float orc_decode_local_t(float out_depth, float mint, float maxt, int inside, float depth_epsilon,
                         float fixed_depth_epsilon);

/* --- training: neural_bvh_module_kernels.cu:119-264, neural_bvh_module_common.cuh:586-861 --- */
void orc_generate_training_batch(const orc_neural_scene *scene, const orc_classic_scene *classic,
                                 const float *albedo, const orc_neural_consts *c,
                                 uint32_t training_step, uint32_t batch_size, uint32_t n,
                                 float *positions, float *targets, uint32_t *nodes);

/* --- learned tree cut (NeuralBVH2Node LoD encoding, include/cuda/neural/accel/neural_bvh2.cuh:14-30) --- */
#define ORC_NUM_BVH_LODS 7u
#define ORC_LEAF_FINAL 1u
#define ORC_LEAF_LOD(l) (2u + (l))
#define ORC_NO_NEURAL_CHILD 0xFFFFFFFFu

/* Per-node tree-cut statistics are 4 words: f32 loss, u32 iter_alive, u32 depth, u32 samples
 * (NeuralTreeCutData, include/cuda/neural/neural_bvh_renderer.h:36-47). */
float orc_loss_heuristic(const uint32_t *stats);

/* Node survival of the training sampler (neural_bvh_module_kernels.cu:184-199) and the sampled
 * LoD (common.cuh:719-721). A rejected sample leaves positions / targets of its slot unchanged. */
typedef struct orc_node_survival {
    const uint32_t *stats;
    float current_max_loss;
    float survival_probability_scale;
    float min_survival_prob;
    uint32_t current_learned_lod;
    int32_t enabled;
} orc_node_survival;

void orc_generate_training_batch_rr(const orc_neural_scene *scene, const orc_classic_scene *classic,
                                    const float *albedo, const orc_neural_consts *c,
                                    uint32_t training_step, uint32_t batch_size, uint32_t n,
                                    float *positions, float *targets, uint32_t *nodes,
                                    const orc_node_survival *rr);

/* update_neural_tree_cut_loss (renderer_kernels.cu:202-230): values are n x dims loss values. */
void orc_tree_cut_accumulate(uint32_t *stats, const float *values, const uint32_t *sample_nodes,
                             uint32_t n, uint32_t dims);

/* The k + 1 launches of update_neural_tree_cut_decisions (renderer_kernels.cu:232-287), in node
 * order: iter_alive of every leaf + 1, then the k largest distinct heuristics of the non-final
 * leaves (max_losses, floored at 0) and for each the last node in index order holding it. */
void orc_tree_cut_decisions(const uint32_t *nodes, uint32_t n_nodes, uint32_t *stats, uint32_t k,
                            float *max_losses, uint32_t *split_indices);

/* split_neural_bvh_at (accel.cpp:256-392); returns the number of nodes split. */
uint32_t orc_tree_cut_split(uint32_t *nodes, uint32_t *n_nodes, uint32_t capacity, uint32_t *stats,
                            uint32_t *node_map, const uint32_t *classic_nodes,
                            const uint32_t *split_indices, uint32_t k, uint32_t current_lod);

/* assign_lod_to_current_neural_leaf_nodes (accel.cpp:394-441) */
void orc_tree_cut_assign_lod(uint32_t *nodes, uint32_t n_nodes, uint32_t lod);

typedef struct orc_loss_consts {
    int32_t visibility_loss, depth_loss, normal_loss, albedo_loss;
    float visibility_loss_scale, depth_loss_scale, normal_loss_scale, albedo_loss_scale;
    int32_t output_normal_linear_activation, output_albedo_linear_activation;
    int32_t visibility_masking_loss;
    int32_t learn_normal, learn_albedo;
} orc_loss_consts;

/* composite_pt_loss, include/cuda/neural/utils/pt_composite_loss.cuh:18-123: per element of the
 * n x 16 prediction matrix, loss value and d loss / d prediction (loss_scale applied). */
void orc_composite_loss(const orc_loss_consts *lc, const float *predictions, const float *targets,
                        uint32_t n, float loss_scale, float *values, float *gradients);

/* Mean loss and the gradient of the mean loss w.r.t. all parameters (network then grid, FP32
 * master layout), for the FP16 forward of orc_network_inference; gradients of the output rounded
 * to FP16 after loss scaling as the FP16 backward does, loss scale removed at the end. */
void orc_compute_gradients(const orc_network *net, const orc_loss_consts *lc, const float *positions,
                           const float *targets, uint32_t n, float loss_scale, double *gradients,
                           double *mean_loss, int fp16_backward);

/* Adam + ExponentialDecay step over n params (FP32); step = steps completed before this one. */
void orc_adam_step(float *params, float *m, float *v, const float *grad, uint32_t n, uint32_t step,
                   float lr, float beta1, float beta2, float eps, float l2_reg, int32_t decay_start,
                   int32_t decay_interval, float decay_base);

/* Pinhole camera rays of run_inference (renderer_kernels.cuh:74-79, cuda_backend.cpp:595-611). */
void orc_camera_rays(uint32_t width, uint32_t height, uint32_t sample_idx, uint32_t sample_offset,
                     const float *origin, const float *target, const float *up, float yfov_degrees,
                     float *rays);

#ifdef __cplusplus
}
#endif

/* --- hybrid path tracer (the library's wavefront path tracer, k_path.cu, after the reference's
 *     Lambertian case of path_inference_kernels.cu:224-429 and material.cuh:101-200) --- */
typedef struct orc_path_params {
    float origin[3], du[3], dv[3], tl[3]; /* pinhole camera: d = normalize(du * x + dv * y + tl) */
    uint32_t width, height, spp, sample_base, sample_offset, seed, max_bounces, has_ground;
    float ground_y;
    float ground_albedo[3], sky_zenith[3], sky_horizon[3];
} orc_path_params;

/* Camera basis of CudaBackend::update_camera (cuda_backend.cpp:595-611), as orc_camera_rays. */
void orc_camera_basis(uint32_t width, uint32_t height, const float *origin, const float *target, const float *up,
                      float yfov_degrees, float *du, float *dv, float *tl);

/* One frame: image receives width x height RGBA values; returns the rays traced. */
uint64_t orc_path_trace(const orc_neural_scene *scene, const orc_network *net, const orc_neural_consts *c,
                        const orc_path_params *p, float *image, int n_threads);

#endif
