// k_misc.cu -- pinhole camera ray generation for run-inference, and the hash-grid level scales
// as the GPU evaluates them (a check of the host's values).
//
// camera_raygen (include/cuda/neural/neural_bvh_renderer_kernels.cuh:74-79) with the pixel jitter of
// camera_raygen_and_intersect_neural_bvh (include/cuda/neural/neural_bvh_module_common.cuh:222-228):
// rng = get_lcg_rng(sample_idx, sample_offset, pixel), x = (px + u) / width, y = (py + u') / height,
// d = normalize(x * du + y * dv + dir_top_left).
#include "device_math.cuh"
#include "nbvh_internal.h"

namespace nbvh {

namespace {

struct CameraArgs {
    float origin[3], du[3], dv[3], tl[3];
    uint32_t width, height, sample_idx, sample_offset;
    nbvh_ray *rays;
};

__global__ void __launch_bounds__(256) k_camera_rays(const __grid_constant__ CameraArgs a)
{
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.width * a.height)
        return;
    const uint32_t px = p % a.width, py = p / a.width;
    uint32_t rng = lcg_seed(a.sample_idx, a.sample_offset, p);
    const float jx = lcg_randomf(rng);
    const float jy = lcg_randomf(rng);
    const float xf = __fdiv_rn(__fadd_rn((float)px, jx), (float)a.width);
    const float yf = __fdiv_rn(__fadd_rn((float)py, jy), (float)a.height);
    const V3 du = mk3(a.du[0], a.du[1], a.du[2]), dv = mk3(a.dv[0], a.dv[1], a.dv[2]),
             tl = mk3(a.tl[0], a.tl[1], a.tl[2]);
    const V3 d = normalize3(add3(add3(scale3(du, xf), scale3(dv, yf)), tl));
    float4 *out = reinterpret_cast<float4 *>(a.rays + p);
    out[0] = make_float4(a.origin[0], a.origin[1], a.origin[2], 1e-4f);
    out[1] = make_float4(d.x, d.y, d.z, FLT_MAX);
}

// tcnn's grid_scale evaluated on the device, as tcnn's encoding kernels do:
// exp2f(level * log2_per_level_scale) * base_resolution - 1 (nvcc contracts the multiply and the
// subtraction into one FMA by default; written out here as that FMA).
__global__ void k_level_scales(float log2_scale, float base, uint32_t n, float *out)
{
    const uint32_t l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l < n)
        out[l] = __fmaf_rn(exp2f(__fmul_rn((float)l, log2_scale)), base, -1.0f);
}

} // namespace

cudaError_t launch_level_scales(float log2_scale, float base, uint32_t n, float *out, cudaStream_t s)
{
    if (n == 0)
        return cudaSuccess;
    k_level_scales<<<1, 32, 0, s>>>(log2_scale, base, n, out);
    return cudaGetLastError();
}

cudaError_t launch_camera_rays(uint32_t width, uint32_t height, uint32_t sample_idx, uint32_t sample_offset,
                               const float *origin, const float *du, const float *dv, const float *top_left,
                               nbvh_ray *rays, cudaStream_t s)
{
    CameraArgs a;
    for (int k = 0; k < 3; k++) {
        a.origin[k] = origin[k];
        a.du[k] = du[k];
        a.dv[k] = dv[k];
        a.tl[k] = top_left[k];
    }
    a.width = width;
    a.height = height;
    a.sample_idx = sample_idx;
    a.sample_offset = sample_offset;
    a.rays = rays;
    const uint32_t n = width * height;
    if (n == 0)
        return cudaSuccess;
    k_camera_rays<<<(n + 255u) / 256u, 256, 0, s>>>(a);
    return cudaGetLastError();
}

} // namespace nbvh
