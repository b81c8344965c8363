// post.cu — output stage on the device: ACES tone map (tonemap.cs.hlsl:17-77)
// and the util/meansq mean squared error (meansq.cpp:34-43) as an FP64
// reduction.
#include <cuda_runtime.h>

#include "kernels.h"

namespace pt {

namespace {

__device__ __forceinline__ float to_srgb(float x) { return x <= 0.00031308f ? 12.92f * x : 1.055f * powf(x, 1.0f / 2.4f) - 0.055f; }

// src_is_srgb = false, dst_is_srgb = true (ptdispatch.cpp:29): encode, RRT,
// rational fit, ODT, saturate (NaN -> 0).  In place, alpha untouched.
__global__ void k_tonemap(float4* img, uint32_t n)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    float4 c = img[i];
    float s0 = to_srgb(c.x), s1 = to_srgb(c.y), s2 = to_srgb(c.z);
    float r[3] = {(0.59719f * s0 + 0.35458f * s1) + 0.04823f * s2, (0.07600f * s0 + 0.90834f * s1) + 0.01566f * s2,
                  (0.02840f * s0 + 0.13383f * s1) + 0.83777f * s2};
#pragma unroll
    for (int k = 0; k < 3; k++) {
        float v = r[k];
        float a = v * (v + 0.0245786f) - 0.000090537f;
        float b = v * (0.983729f * v + 0.4329510f) + 0.238081f;
        r[k] = a / b;
    }
    float o0 = (1.60475f * r[0] + -0.53108f * r[1]) + -0.07367f * r[2];
    float o1 = (-0.10208f * r[0] + 1.10813f * r[1]) + -0.00605f * r[2];
    float o2 = (-0.00327f * r[0] + -0.07276f * r[1]) + 1.07602f * r[2];
    c.x = isnan(o0) ? 0.0f : fminf(fmaxf(o0, 0.0f), 1.0f);
    c.y = isnan(o1) ? 0.0f : fminf(fmaxf(o1, 0.0f), 1.0f);
    c.z = isnan(o2) ? 0.0f : fminf(fmaxf(o2, 0.0f), 1.0f);
    img[i] = c;
}

// Per-block partial sums of squared RGB differences (difference in float,
// square and sum in FP64, as meansq.cpp:39-41), then one block adds the
// partials in index order so the result does not depend on scheduling.
constexpr int MSE_THREADS = 256;

__device__ __forceinline__ double block_sum(double v)
{
    __shared__ double warp_part[MSE_THREADS / 32];
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0)
        warp_part[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < MSE_THREADS / 32; w++)
            t += warp_part[w];
    return t;
}

__global__ void __launch_bounds__(MSE_THREADS) k_sse_partial(const float4* img, const float4* ref, uint32_t n, double* partial)
{
    double acc = 0.0;
    for (uint32_t i = blockIdx.x * MSE_THREADS + threadIdx.x; i < n; i += gridDim.x * MSE_THREADS) {
        float4 a = img[i], b = ref[i];
        double ex = (double)(a.x - b.x), ey = (double)(a.y - b.y), ez = (double)(a.z - b.z);
        acc += ex * ex;
        acc += ey * ey;
        acc += ez * ez;
    }
    double t = block_sum(acc);
    if (threadIdx.x == 0)
        partial[blockIdx.x] = t;
}

__global__ void __launch_bounds__(MSE_THREADS) k_sse_final(const double* partial, uint32_t blocks, double denom, double* out)
{
    double acc = 0.0;
    for (uint32_t i = threadIdx.x; i < blocks; i += MSE_THREADS)
        acc += partial[i];
    double t = block_sum(acc);
    if (threadIdx.x == 0)
        *out = t / denom;
}

} // namespace

cudaError_t launch_tonemap(float4* img, uint32_t n, cudaStream_t st)
{
    if (n == 0)
        return cudaSuccess;
    k_tonemap<<<(n + 255) / 256, 256, 0, st>>>(img, n);
    return cudaGetLastError();
}

uint32_t mse_blocks(uint32_t n)
{
    uint32_t b = (n + MSE_THREADS - 1) / MSE_THREADS;
    return b < MSE_MAX_BLOCKS ? (b == 0 ? 1 : b) : MSE_MAX_BLOCKS;
}

cudaError_t launch_mse(const float4* img, const float4* ref, uint32_t width, uint32_t height, double* partial, double* out, cudaStream_t st)
{
    uint32_t n = width * height;
    uint32_t blocks = mse_blocks(n);
    k_sse_partial<<<blocks, MSE_THREADS, 0, st>>>(img, ref, n, partial);
    double denom = (double)width * height * 3 - 1;
    k_sse_final<<<1, MSE_THREADS, 0, st>>>(partial, blocks, denom, out);
    return cudaGetLastError();
}

} // namespace pt
