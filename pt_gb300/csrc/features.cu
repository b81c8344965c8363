// features.cu — first-hit features for the denoiser and the packing of the
// network's input and output.
//
// The feature rays are the camera rays of the plain tracer (same sampler
// state: pixel, sample index, seed 0; the first two 2-D samples give the
// pixel and lens offsets), so features of samples [s, s + k) describe exactly
// the primary hits of those samples.
#include <cuda_bf16.h>

#include "device/render.cuh"
#include "kernels.h"

namespace pt {

namespace {

__global__ void __launch_bounds__(128) k_features(RenderArgs a, float4* feat_a, float4* feat_n)
{
    const uint32_t h = a.fp16_features;
    const uint32_t pixels = a.width * a.height;
    TraceCounters tc{0u, 0u};
    for (uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x; pix < pixels; pix += gridDim.x * blockDim.x) {
        const uint32_t px = pix % a.width, py = pix / a.width;
        f3 alb = mk3(0.0f, 0.0f, 0.0f), nrm = mk3(0.0f, 0.0f, 0.0f);
        float depth = 0.0f;
        for (uint32_t k = 0; k < a.samples; k++) {
            Sampler smp;
            sampler_start(smp, px, py, a.sample_index + k, 0);
            f2 u_pixel = sample_2d(smp);
            f2 u_lens = sample_2d(smp);
            f3 ro, rd;
            camera_ray(a, px, py, u_pixel, u_lens, ro, rd);
            Hit h;
            if (!trace_closest(a.s, ro, rd, a.near_plane, a.far_plane, h, tc))
                continue;
            f3 ha, hn;
            hit_features(a.s, h, rd, ha, hn);
            alb = alb + ha;
            nrm = nrm + hn;
            depth += h.t;
        }
        const float inv = 1.0f / (float)a.samples;
        feat_store(feat_a, pix, make_float4(alb.x * inv, alb.y * inv, alb.z * inv, depth * inv), h);
        feat_store(feat_n, pix, make_float4(nrm.x * inv, nrm.y * inv, nrm.z * inv, 0.0f), h);
    }
}

__device__ __forceinline__ uint32_t bf2(float a, float b)
{
    __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&v);
}

// Noise estimate: the mean of the first samples minus the mean of all of them
// (half the difference of two independent half-sample means), signed log.
__device__ __forceinline__ float slog(float x)
{
    return copysignf(log1pf(fabsf(x)), x);
}

__global__ void k_denoise_input(const float4* img, const float4* half, const float4* fa, const float4* fn, uint32_t pixels,
                                float spp_feature, uint16_t* out, float4* base, uint32_t feat_h, uint32_t half_h)
{
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < pixels; p += gridDim.x * blockDim.x) {
        const float4 c = img[p], a = feat_load(fa, p, feat_h), n = feat_load(fn, p, feat_h);
        const float r = log1pf(fmaxf(c.x, 0.0f)), g = log1pf(fmaxf(c.y, 0.0f)), b = log1pf(fmaxf(c.z, 0.0f));
        float dr = 0.0f, dg = 0.0f, db = 0.0f, have = 0.0f;
        if (half) {
            const float4 h = feat_load(half, p, half_h);
            dr = slog(h.x - c.x);
            dg = slog(h.y - c.y);
            db = slog(h.z - c.z);
            have = 1.0f;
        }
        uint4* o = reinterpret_cast<uint4*>(out + (size_t)p * 16);
        o[0] = make_uint4(bf2(r, g), bf2(b, a.x), bf2(a.y, a.z), bf2(n.x, n.y));
        o[1] = make_uint4(bf2(n.z, log1pf(a.w) * 0.25f), bf2(spp_feature, dr), bf2(dg, db), bf2(have, 0.0f));
        if (base)
            base[p] = make_float4(r, g, b, 0.0f);
    }
}

__global__ void k_denoise_output(const float* out32, uint32_t pixels, float4* img)
{
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < pixels; p += gridDim.x * blockDim.x) {
        const float4 y = *reinterpret_cast<const float4*>(out32 + (size_t)p * 16);
        img[p] = make_float4(expm1f(fmaxf(y.x, 0.0f)), expm1f(fmaxf(y.y, 0.0f)), expm1f(fmaxf(y.z, 0.0f)), 1.0f);
    }
}

unsigned grid_for(uint32_t n, int threads)
{
    uint32_t b = (n + threads - 1) / threads;
    return b > 152 * 16 ? 152 * 16 : (b ? b : 1);
}

} // namespace

// This unit's copies of the sampler's direction numbers and the sRGB table.
cudaError_t features_init_tables(const uint32_t* table128, const float* srgb256, cudaStream_t stream)
{
    uint32_t bytes[4][4][256];
    sobol_byte_tables(table128, bytes);
    cudaError_t e = cudaMemcpyToSymbol(g_sobol_bytes, bytes, sizeof(bytes)); // synchronous: `bytes` is local
    if (e == cudaSuccess)
        e = cudaMemcpyToSymbolAsync(c_srgb, srgb256, sizeof(float) * 256, 0, cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess)
        return e;
    return cudaStreamSynchronize(stream);
}

cudaError_t launch_features(const RenderArgs& a, float4* feat_a, float4* feat_n, cudaStream_t st)
{
    k_features<<<grid_for(a.width * a.height, 128), 128, 0, st>>>(a, feat_a, feat_n);
    return cudaGetLastError();
}

cudaError_t launch_denoise_input(const float4* img, const float4* half, const float4* fa, const float4* fn, uint32_t pixels,
                                 float spp_feature, uint16_t* out, float* base, uint32_t feat_fp16, uint32_t half_fp16,
                                 cudaStream_t st)
{
    k_denoise_input<<<grid_for(pixels, 256), 256, 0, st>>>(img, half, fa, fn, pixels, spp_feature, out,
                                                           reinterpret_cast<float4*>(base), feat_fp16, half_fp16);
    return cudaGetLastError();
}

cudaError_t launch_denoise_output(const float* out32, uint32_t pixels, float4* img, cudaStream_t st)
{
    k_denoise_output<<<grid_for(pixels, 256), 256, 0, st>>>(out32, pixels, img);
    return cudaGetLastError();
}

} // namespace pt
