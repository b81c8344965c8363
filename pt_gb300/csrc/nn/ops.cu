// ops.cu — memory-bound kernels of the denoiser: 2x2 average pooling and
// nearest upsampling with their backward passes (ReLU masks fused), bias
// gradients, weight packing for the tensor-core layouts and Adam.  Each
// thread moves 8 channels (one 16-byte vector) of one pixel.
#include <cuda_bf16.h>

#include "nn.h"

namespace pt {
namespace nn {

namespace {

__device__ __forceinline__ void unpack8(uint4 q, float (&v)[8])
{
    const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
    for (int k = 0; k < 4; k++) {
        v[2 * k] = __uint_as_float(w[k] << 16);
        v[2 * k + 1] = __uint_as_float(w[k] & 0xFFFF0000u);
    }
}

__device__ __forceinline__ uint32_t pack2(float a, float b)
{
    __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&v);
}

__device__ __forceinline__ uint4 pack8(const float (&v)[8])
{
    return make_uint4(pack2(v[0], v[1]), pack2(v[2], v[3]), pack2(v[4], v[5]), pack2(v[6], v[7]));
}

__device__ __forceinline__ uint4 ld8(const Act& a, size_t pix, int c)
{
    return *reinterpret_cast<const uint4*>(a.p + pix * a.pitch + c);
}

__device__ __forceinline__ void st8(const Act& a, size_t pix, int c, uint4 v)
{
    *reinterpret_cast<uint4*>(a.p + pix * a.pitch + c) = v;
}

__device__ __forceinline__ size_t pixel(const Act& a, int img, int y, int x)
{
    return ((size_t)img * a.h + y) * a.w + x;
}

// grid-stride over (output pixel, 8-channel group)
#define PT_FOR_PIXEL_GROUPS(out, groups)                                                                                          \
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x, n_ = (out).pixels() * (groups); i < n_;                       \
         i += (size_t)gridDim.x * blockDim.x)

__global__ void k_pool2(Act in, int in_c0, int groups, Act out, int out_c0)
{
    PT_FOR_PIXEL_GROUPS(out, groups)
    {
        const int g = (int)(i % groups);
        size_t q = i / groups;
        const int x = (int)(q % out.w);
        q /= out.w;
        const int y = (int)(q % out.h);
        const int img = (int)(q / out.h);
        float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int dy = 0; dy < 2; dy++)
            for (int dx = 0; dx < 2; dx++) {
                float v[8];
                unpack8(ld8(in, pixel(in, img, 2 * y + dy, 2 * x + dx), in_c0 + 8 * g), v);
#pragma unroll
                for (int k = 0; k < 8; k++)
                    acc[k] += v[k];
            }
#pragma unroll
        for (int k = 0; k < 8; k++)
            acc[k] *= 0.25f;
        st8(out, pixel(out, img, y, x), out_c0 + 8 * g, pack8(acc));
    }
}

__global__ void k_upsample2(Act in, int in_c0, int groups, Act out, int out_c0)
{
    PT_FOR_PIXEL_GROUPS(out, groups)
    {
        const int g = (int)(i % groups);
        size_t q = i / groups;
        const int x = (int)(q % out.w);
        q /= out.w;
        const int y = (int)(q % out.h);
        const int img = (int)(q / out.h);
        st8(out, pixel(out, img, y, x), out_c0 + 8 * g, ld8(in, pixel(in, img, y / 2, x / 2), in_c0 + 8 * g));
    }
}

__device__ __forceinline__ void relu_mask(float (&v)[8], uint4 zq)
{
    float z[8];
    unpack8(zq, z);
#pragma unroll
    for (int k = 0; k < 8; k++)
        if (!(z[k] > 0.0f))
            v[k] = 0.0f;
}

__global__ void k_upsample2_backward(Act gh, int g_c0, int groups, Act z, int z_c0, Act gl)
{
    PT_FOR_PIXEL_GROUPS(gl, groups)
    {
        const int g = (int)(i % groups);
        size_t q = i / groups;
        const int x = (int)(q % gl.w);
        q /= gl.w;
        const int y = (int)(q % gl.h);
        const int img = (int)(q / gl.h);
        float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int dy = 0; dy < 2; dy++)
            for (int dx = 0; dx < 2; dx++) {
                float v[8];
                unpack8(ld8(gh, pixel(gh, img, 2 * y + dy, 2 * x + dx), g_c0 + 8 * g), v);
#pragma unroll
                for (int k = 0; k < 8; k++)
                    acc[k] += v[k];
            }
        const size_t pl = pixel(gl, img, y, x);
        relu_mask(acc, ld8(z, pl, z_c0 + 8 * g));
        st8(gl, pl, 8 * g, pack8(acc));
    }
}

__global__ void k_pool2_backward(Act gs, int s_c0, Act gp, int groups, Act z, int z_c0, Act g_out)
{
    PT_FOR_PIXEL_GROUPS(g_out, groups)
    {
        const int g = (int)(i % groups);
        size_t q = i / groups;
        const int x = (int)(q % g_out.w);
        q /= g_out.w;
        const int y = (int)(q % g_out.h);
        const int img = (int)(q / g_out.h);
        const size_t ph = pixel(g_out, img, y, x);
        float a[8], b[8];
        unpack8(ld8(gs, ph, s_c0 + 8 * g), a);
        unpack8(ld8(gp, pixel(gp, img, y / 2, x / 2), 8 * g), b);
#pragma unroll
        for (int k = 0; k < 8; k++)
            a[k] += 0.25f * b[k];
        relu_mask(a, ld8(z, ph, z_c0 + 8 * g));
        st8(g_out, ph, 8 * g, pack8(a));
    }
}

// One block reduces a pixel range for all channels: thread t owns the 8-channel
// group t % groups and strides over pixels by blockDim / groups.
__global__ void k_bias_grad(Act g, int c0, int groups, float* db, size_t pixels_per_block)
{
    extern __shared__ float red[];
    const int rows = blockDim.x / groups;
    const int grp = threadIdx.x % groups, row = threadIdx.x / groups;
    float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    const size_t p0 = blockIdx.x * pixels_per_block;
    const size_t p1 = min(p0 + pixels_per_block, g.pixels());
    if (row < rows)
        for (size_t p = p0 + row; p < p1; p += rows) {
            float v[8];
            unpack8(ld8(g, p, c0 + 8 * grp), v);
#pragma unroll
            for (int k = 0; k < 8; k++)
                acc[k] += v[k];
        }
    for (int k = 0; k < 8; k++)
        red[threadIdx.x * 8 + k] = row < rows ? acc[k] : 0.0f;
    __syncthreads();
    if (threadIdx.x < groups * 8) {
        const int gg = threadIdx.x / 8, k = threadIdx.x % 8;
        float s = 0.0f;
        for (int r = 0; r < rows; r++)
            s += red[(r * groups + gg) * 8 + k];
        atomicAdd(db + 8 * gg + k, s);
    }
}

__global__ void k_pack_weights(const float* w, int cin, int cout, uint16_t* fwd, uint16_t* bwd)
{
    const size_t n = (size_t)9 * cin * cout;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        // i enumerates w[tap][ci][co]
        const int co = (int)(i % cout);
        const int ci = (int)((i / cout) % cin);
        const int tap = (int)(i / ((size_t)cout * cin));
        __nv_bfloat16 b = __float2bfloat16_rn(w[i]);
        const uint16_t bits = *reinterpret_cast<uint16_t*>(&b);
        // forward: [tap][ci/8][co][ci%8]
        fwd[(((size_t)tap * (cin / 8) + ci / 8) * cout + co) * 8 + ci % 8] = bits;
        // data gradient: tap' = 8 - tap, [tap'][co/8][ci][co%8]
        bwd[(((size_t)(8 - tap) * (cout / 8) + co / 8) * cin + ci) * 8 + co % 8] = bits;
    }
}

__global__ void k_adam(float* p, const float* g, float* m, float* v, size_t n, float lr, float b1, float b2, float eps, float bc1,
                       float bc2)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.0f - b1) * gi;
        const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    }
}

unsigned grid_for(size_t n, int threads)
{
    size_t b = (n + threads - 1) / threads;
    if (b > 152 * 32)
        b = 152 * 32;
    return (unsigned)(b ? b : 1);
}

bool shape_ok(const Act& a, int c0, int c)
{
    return a.p && c > 0 && c % 8 == 0 && c0 % 8 == 0 && c0 + c <= a.pitch && a.pitch % 8 == 0;
}

} // namespace

cudaError_t pool2(const Act& in, int in_c0, int c, const Act& out, int out_c0, cudaStream_t st)
{
    if (!shape_ok(in, in_c0, c) || !shape_ok(out, out_c0, c) || in.h != 2 * out.h || in.w != 2 * out.w || in.n != out.n)
        return cudaErrorInvalidValue;
    k_pool2<<<grid_for(out.pixels() * (c / 8), 256), 256, 0, st>>>(in, in_c0, c / 8, out, out_c0);
    return cudaGetLastError();
}

cudaError_t upsample2(const Act& in, int in_c0, int c, const Act& out, int out_c0, cudaStream_t st)
{
    if (!shape_ok(in, in_c0, c) || !shape_ok(out, out_c0, c) || out.h != 2 * in.h || out.w != 2 * in.w || in.n != out.n)
        return cudaErrorInvalidValue;
    k_upsample2<<<grid_for(out.pixels() * (c / 8), 256), 256, 0, st>>>(in, in_c0, c / 8, out, out_c0);
    return cudaGetLastError();
}

cudaError_t upsample2_backward(const Act& g_high, int g_c0, int c, const Act& z, int z_c0, const Act& g_low, cudaStream_t st)
{
    if (!shape_ok(g_high, g_c0, c) || !shape_ok(z, z_c0, c) || !shape_ok(g_low, 0, c) || g_high.h != 2 * g_low.h ||
        g_high.w != 2 * g_low.w || z.h != g_low.h || z.w != g_low.w)
        return cudaErrorInvalidValue;
    k_upsample2_backward<<<grid_for(g_low.pixels() * (c / 8), 256), 256, 0, st>>>(g_high, g_c0, c / 8, z, z_c0, g_low);
    return cudaGetLastError();
}

cudaError_t pool2_backward(const Act& g_skip, int s_c0, const Act& g_pool, int c, const Act& z, int z_c0, const Act& g,
                           cudaStream_t st)
{
    if (!shape_ok(g_skip, s_c0, c) || !shape_ok(g_pool, 0, c) || !shape_ok(z, z_c0, c) || !shape_ok(g, 0, c) ||
        g.h != 2 * g_pool.h || g.w != 2 * g_pool.w || g_skip.h != g.h || z.h != g.h)
        return cudaErrorInvalidValue;
    k_pool2_backward<<<grid_for(g.pixels() * (c / 8), 256), 256, 0, st>>>(g_skip, s_c0, g_pool, c / 8, z, z_c0, g);
    return cudaGetLastError();
}

cudaError_t bias_grad(const Act& g, int c0, int c, float* db, cudaStream_t st)
{
    if (!shape_ok(g, c0, c) || c > 256)
        return cudaErrorInvalidValue;
    const int groups = c / 8;
    const int threads = 256;
    const size_t blocks = 152 * 4;
    size_t per = (g.pixels() + blocks - 1) / blocks;
    if (per == 0)
        per = 1;
    const size_t nb = (g.pixels() + per - 1) / per;
    if (nb == 0)
        return cudaSuccess;
    k_bias_grad<<<(unsigned)nb, threads, threads * 8 * sizeof(float), st>>>(g, c0, groups, db, per);
    return cudaGetLastError();
}

cudaError_t pack_weights(const float* w, int cin, int cout, uint16_t* fwd, uint16_t* bwd, cudaStream_t st)
{
    if (cin % 8 || cout % 8)
        return cudaErrorInvalidValue;
    k_pack_weights<<<grid_for((size_t)9 * cin * cout, 256), 256, 0, st>>>(w, cin, cout, fwd, bwd);
    return cudaGetLastError();
}

cudaError_t adam_step(float* p, const float* g, float* m, float* v, size_t n, float lr, float beta1, float beta2, float eps,
                      float bc1, float bc2, cudaStream_t st)
{
    k_adam<<<grid_for(n, 256), 256, 0, st>>>(p, g, m, v, n, lr, beta1, beta2, eps, bc1, bc2);
    return cudaGetLastError();
}

} // namespace nn
} // namespace pt
