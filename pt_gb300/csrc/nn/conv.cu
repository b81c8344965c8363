// conv.cu — 3x3 convolutions of the denoiser on the tcgen05 tensor core.
//
// conv3x3 (forward and data gradient) is an implicit GEMM: M = 128 pixels of
// one image (a tx x ty tile), N = output channels, K = 9 taps x input
// channels.  Per tap, one TMA tensor load per 8 input channels brings the
// shifted 128-pixel tile (zero-filled outside the image, which is the conv's
// zero padding) into a K-major no-swizzle layout, and one bulk copy brings
// the tap's pre-packed weights.  Warp 0 produces, warp 1 issues tcgen05.mma
// into a TMEM accumulator, and all four warps run the epilogue (bias, ReLU,
// gradient mask, BF16 or FP32 store) from TMEM.
//
// conv3x3_wgrad is a GEMM with M = 128 (tap, input channel) rows, N = output
// channels and K = pixels: both operands come straight from NHWC buffers in
// MN-major layout (8 channels of one pixel per 16-byte row), K is split over
// CTAs and the partial sums are added to the FP32 gradient with atomics.
#include <cuda_bf16.h>

#include <algorithm>

#include "nn.h"
#include "tc.cuh"

namespace pt {
namespace nn {

namespace {

struct ConvParams {
    int cin, c0, nout;
    const uint16_t* wpk;
    const float* bias;
    int relu;
    uint16_t* out;
    int out_pitch, out_c0;
    float* out_f32;
    const uint16_t* mask;
    int mask_pitch, mask_c0;
    const float* residual;
    int n, h, w, tx, ty, tiles_x, tiles_y;
    int stages;
    uint32_t tmem_cols;
    uint32_t* error;
};

__device__ __forceinline__ bool bf16_positive(uint16_t b)
{
    return (b & 0x8000u) == 0 && (b & 0x7FFFu) != 0;
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b)
{
    __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&v);
}

__global__ void __launch_bounds__(128) k_conv3x3(const __grid_constant__ CUtensorMap amap, ConvParams p)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    const uint32_t a_bytes = (uint32_t)p.cin * 256u;
    const uint32_t b_bytes = (uint32_t)p.nout * (uint32_t)p.cin * 2u;
    const uint32_t stage_bytes = a_bytes + b_bytes;
    const int S = p.stages;
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + (size_t)S * stage_bytes);
    uint64_t* empty = full + S;
    uint64_t* done = empty + S;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(done + 1);
    uint32_t* fail = tslot + 1;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    int t = blockIdx.x;
    const int txi = t % p.tiles_x;
    t /= p.tiles_x;
    const int tyi = t % p.tiles_y;
    const int img = t / p.tiles_y;
    const int x0 = txi * p.tx, y0 = tyi * p.ty;

    if (threadIdx.x == 0) {
        for (int s = 0; s < S; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(done, 1);
        *fail = 0;
        mbar_init_fence();
    }
    if (warp == 0) {
        tmem_alloc(tslot, p.tmem_cols);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    bool ok = true;

    if (warp == 0 && lane == 0) {
        // producer: the shifted input tile and the weights of each tap
        for (int tap = 0; tap < 9 && ok; tap++) {
            const int s = tap % S;
            if (tap >= S && !mbar_wait(&empty[s], (uint32_t)((tap / S) - 1) & 1u)) {
                ok = false;
                break;
            }
            uint8_t* sa = smem + (size_t)s * stage_bytes;
            mbar_expect_tx(&full[s], stage_bytes);
            const int dy = tap / 3 - 1, dx = tap % 3 - 1;
            for (int kg = 0; kg < p.cin / 8; kg++)
                tma_load_4d(sa + kg * 2048, &amap, &full[s], p.c0 + 8 * kg, x0 + dx, y0 + dy, img);
            bulk_load(sa + a_bytes, p.wpk + (size_t)tap * p.nout * p.cin, b_bytes, &full[s]);
        }
    } else if (warp == 1 && lane == 0) {
        // MMA issuer
        const uint32_t idesc = idesc_bf16(128, (uint32_t)p.nout, false, false);
        const uint32_t b_lbo = (uint32_t)p.nout * 16u;
        for (int tap = 0; tap < 9; tap++) {
            const int s = tap % S;
            if (!mbar_wait(&full[s], (uint32_t)(tap / S) & 1u)) {
                ok = false;
                break;
            }
            tc_fence_after();
            const uint32_t sa = smem_addr(smem + (size_t)s * stage_bytes);
            const uint32_t sb = sa + a_bytes;
            for (int ks = 0; ks < p.cin / 16; ks++) {
                uint64_t ad = smem_desc(sa + (uint32_t)ks * 4096u, 2048u, 128u);
                uint64_t bd = smem_desc(sb + (uint32_t)ks * 2u * b_lbo, b_lbo, 128u);
                mma_bf16(tmem, ad, bd, idesc, (tap | ks) != 0);
            }
            mma_commit(&empty[s]);
        }
        mma_commit(done);
    }
    if (!ok)
        atomicOr(fail, 1u);
    __syncwarp();
    if (!mbar_wait(done, 0))
        atomicOr(fail, 1u);
    __syncthreads();
    ok = *fail == 0;
    tc_fence_after();

    // epilogue: TMEM lane = pixel of the tile, columns = output channels
    const int m = warp * 32 + lane;
    const int px = x0 + m % p.tx, py = y0 + m / p.tx;
    const bool valid = ok && px < p.w && py < p.h;
    const size_t pix = ((size_t)img * p.h + py) * p.w + px;
    for (int j = 0; j < p.nout / 16; j++) {
        uint32_t r[16];
        tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(j * 16), r);
        if (!valid)
            continue;
        float v[16];
#pragma unroll
        for (int k = 0; k < 16; k++) {
            v[k] = __uint_as_float(r[k]);
            if (p.bias)
                v[k] += p.bias[j * 16 + k];
            if (p.relu)
                v[k] = fmaxf(v[k], 0.0f);
        }
        if (p.mask) {
            const uint4* mp = reinterpret_cast<const uint4*>(p.mask + pix * p.mask_pitch + p.mask_c0 + j * 16);
            uint4 q0 = mp[0], q1 = mp[1];
            const uint32_t mw[8] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w};
#pragma unroll
            for (int k = 0; k < 8; k++) {
                if (!bf16_positive((uint16_t)(mw[k] & 0xFFFFu)))
                    v[2 * k] = 0.0f;
                if (!bf16_positive((uint16_t)(mw[k] >> 16)))
                    v[2 * k + 1] = 0.0f;
            }
        }
        if (p.out_f32) {
            if (p.residual && j == 0) {
                const float4 r4 = *reinterpret_cast<const float4*>(p.residual + pix * 4);
                v[0] += r4.x;
                v[1] += r4.y;
                v[2] += r4.z;
                v[3] += r4.w;
            }
            float4* o = reinterpret_cast<float4*>(p.out_f32 + pix * p.out_pitch + j * 16);
#pragma unroll
            for (int k = 0; k < 4; k++)
                o[k] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
        } else {
            uint4* o = reinterpret_cast<uint4*>(p.out + pix * p.out_pitch + p.out_c0 + j * 16);
            o[0] = make_uint4(pack_bf16(v[0], v[1]), pack_bf16(v[2], v[3]), pack_bf16(v[4], v[5]), pack_bf16(v[6], v[7]));
            o[1] = make_uint4(pack_bf16(v[8], v[9]), pack_bf16(v[10], v[11]), pack_bf16(v[12], v[13]), pack_bf16(v[14], v[15]));
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, p.tmem_cols);
    }
    if (!ok && threadIdx.x == 0)
        atomicOr(p.error, 1u);
}

struct WgradParams {
    int cin, x_c0, cout, g_c0;
    int groups;     // 9 * cin / 8 row groups of the GEMM
    int n, h, w, tx, ty, chunks_x, chunks_y, chunks, chunks_per_cta;
    int stages;
    uint32_t tmem_cols;
    float* dw;
    uint32_t* error;
};

__global__ void __launch_bounds__(128) k_wgrad(const __grid_constant__ CUtensorMap xmap, const __grid_constant__ CUtensorMap gmap,
                                               WgradParams p)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    const int mt = blockIdx.x;
    const int c_lo = blockIdx.y * p.chunks_per_cta;
    const int c_hi = min(p.chunks, c_lo + p.chunks_per_cta);
    if (c_lo >= c_hi)
        return;
    const int g_lo = mt * 16;
    const int g_n = min(16, p.groups - g_lo);
    const uint32_t a_bytes = 16u * 1024u;
    const uint32_t b_bytes = (uint32_t)p.cout * 128u;
    const uint32_t stage_bytes = a_bytes + b_bytes;
    const uint32_t tx_bytes = (uint32_t)g_n * 1024u + b_bytes;
    const int S = p.stages;
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + (size_t)S * stage_bytes);
    uint64_t* empty = full + S;
    uint64_t* done = empty + S;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(done + 1);
    uint32_t* fail = tslot + 1;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int cpt = p.cin / 8; // channel groups per tap

    if (threadIdx.x == 0) {
        for (int s = 0; s < S; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(done, 1);
        *fail = 0;
        mbar_init_fence();
    }
    if (warp == 0) {
        tmem_alloc(tslot, p.tmem_cols);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    bool ok = true;
    const int nchunks = c_hi - c_lo;

    if (warp == 0 && lane == 0) {
        for (int i = 0; i < nchunks; i++) {
            const int s = i % S;
            if (i >= S && !mbar_wait(&empty[s], (uint32_t)((i / S) - 1) & 1u)) {
                ok = false;
                break;
            }
            int c = c_lo + i;
            const int cx = c % p.chunks_x;
            c /= p.chunks_x;
            const int cy = c % p.chunks_y;
            const int img = c / p.chunks_y;
            const int x0 = cx * p.tx, y0 = cy * p.ty;
            uint8_t* sa = smem + (size_t)s * stage_bytes;
            mbar_expect_tx(&full[s], tx_bytes);
            for (int g = 0; g < g_n; g++) {
                const int G = g_lo + g;
                const int tap = G / cpt, cc = G % cpt;
                tma_load_4d(sa + g * 1024, &xmap, &full[s], p.x_c0 + 8 * cc, x0 + tap % 3 - 1, y0 + tap / 3 - 1, img);
            }
            for (int ng = 0; ng < p.cout / 8; ng++)
                tma_load_4d(sa + a_bytes + ng * 1024, &gmap, &full[s], p.g_c0 + 8 * ng, x0, y0, img);
        }
    } else if (warp == 1 && lane == 0) {
        const uint32_t idesc = idesc_bf16(128, (uint32_t)p.cout, true, true);
        for (int i = 0; i < nchunks; i++) {
            const int s = i % S;
            if (!mbar_wait(&full[s], (uint32_t)(i / S) & 1u)) {
                ok = false;
                break;
            }
            tc_fence_after();
            const uint32_t sa = smem_addr(smem + (size_t)s * stage_bytes);
            const uint32_t sb = sa + a_bytes;
            for (int ks = 0; ks < 4; ks++) {
                // MN-major, no swizzle: lbo = 128 between 8-pixel groups of K,
                // sbo = 1024 between 8-channel groups of M/N
                uint64_t ad = smem_desc(sa + (uint32_t)ks * 256u, 128u, 1024u);
                uint64_t bd = smem_desc(sb + (uint32_t)ks * 256u, 128u, 1024u);
                mma_bf16(tmem, ad, bd, idesc, (i | ks) != 0);
            }
            mma_commit(&empty[s]);
        }
        mma_commit(done);
    }
    if (!ok)
        atomicOr(fail, 1u);
    __syncwarp();
    if (!mbar_wait(done, 0))
        atomicOr(fail, 1u);
    __syncthreads();
    ok = *fail == 0;
    tc_fence_after();

    const int m = warp * 32 + lane;
    const int G = g_lo + m / 8;
    const bool valid = ok && G < p.groups;
    const int tap = G / cpt, ci = (G % cpt) * 8 + (m & 7);
    float* row = p.dw + ((size_t)tap * p.cin + ci) * p.cout;
    for (int j = 0; j < p.cout / 16; j++) {
        uint32_t r[16];
        tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(j * 16), r);
        if (!valid)
            continue;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            float4 v = make_float4(__uint_as_float(r[4 * k]), __uint_as_float(r[4 * k + 1]), __uint_as_float(r[4 * k + 2]),
                                   __uint_as_float(r[4 * k + 3]));
            atomicAdd(reinterpret_cast<float4*>(row + j * 16 + 4 * k), v);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, p.tmem_cols);
    }
    if (!ok && threadIdx.x == 0)
        atomicOr(p.error, 1u);
}

uint32_t tmem_columns(int n)
{
    uint32_t c = 32;
    while (c < (uint32_t)n)
        c <<= 1;
    return c;
}

// Dynamic shared memory that keeps at most 512 / cols CTAs on one SM, so that
// every resident CTA's TMEM allocation fits the SM's 512 columns.
size_t smem_for_residency(size_t need, uint32_t cols)
{
    const size_t per_sm = 233472; // 228 KB of shared memory per SM
    const size_t per_cta_reserved = 1024;
    size_t max_ctas = 512 / cols;
    size_t floor_bytes = per_sm / (max_ctas + 1) + 1 - per_cta_reserved;
    return std::max(need, floor_bytes);
}

constexpr size_t SMEM_LIMIT = 232448; // 227 KB per CTA

typedef CUresult (*EncodeTiled)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*, const cuuint64_t*,
                                const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encoder()
{
    static EncodeTiled fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiled>(p);
    }
    return fn;
}

} // namespace

void conv_tile_shape(int w, int& tx, int& ty)
{
    tx = 16;
    while (tx < 128 && tx < w)
        tx <<= 1;
    ty = 128 / tx;
}

void wgrad_chunk_shape(int w, int& tx, int& ty)
{
    tx = 8;
    while (tx < 64 && tx < w)
        tx <<= 1;
    ty = 64 / tx;
}

bool encode_act_map(CUtensorMap* map, const Act& a, int tx, int ty, const char** why)
{
    EncodeTiled enc = encoder();
    if (!enc) {
        *why = "cuTensorMapEncodeTiled is not available from the driver";
        return false;
    }
    if (((uintptr_t)a.p & 15u) || a.pitch % 8 != 0) {
        *why = "activation buffer not 16-byte aligned";
        return false;
    }
    cuuint64_t dims[4] = {(cuuint64_t)a.pitch, (cuuint64_t)a.w, (cuuint64_t)a.h, (cuuint64_t)a.n};
    cuuint64_t strides[3] = {(cuuint64_t)a.pitch * 2, (cuuint64_t)a.pitch * 2 * a.w, (cuuint64_t)a.pitch * 2 * a.w * a.h};
    cuuint32_t box[4] = {8, (cuuint32_t)tx, (cuuint32_t)ty, 1};
    cuuint32_t estr[4] = {1, 1, 1, 1};
    CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, a.p, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                     CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        *why = "cuTensorMapEncodeTiled rejected the activation layout";
        return false;
    }
    return true;
}

cudaError_t conv3x3(const ConvCall& c, uint32_t* error, cudaStream_t st)
{
    if (c.cin % 16 || c.nout % 16 || c.nout < 16 || c.nout > 256 || c.c0 % 8 || c.out_c0 % 8 || (c.mask && c.mask_c0 % 8))
        return cudaErrorInvalidValue;
    if (c.out.n != c.in.n || c.out.h != c.in.h || c.out.w != c.in.w)
        return cudaErrorInvalidValue;
    if (c.out_f32 ? c.out.pitch < c.nout || c.out.pitch % 4 : c.out_c0 + c.nout > c.out.pitch)
        return cudaErrorInvalidValue;
    ConvParams p{};
    p.cin = c.cin;
    p.c0 = c.c0;
    p.nout = c.nout;
    p.wpk = c.wpk;
    p.bias = c.bias;
    p.relu = c.relu ? 1 : 0;
    p.out = c.out.p;
    p.out_pitch = c.out.pitch;
    p.out_c0 = c.out_c0;
    p.out_f32 = c.out_f32;
    p.mask = c.mask ? c.mask->p : nullptr;
    p.mask_pitch = c.mask ? c.mask->pitch : 0;
    p.mask_c0 = c.mask_c0;
    p.residual = c.out_f32 ? c.residual : nullptr;
    p.n = c.in.n;
    p.h = c.in.h;
    p.w = c.in.w;
    conv_tile_shape(p.w, p.tx, p.ty);
    p.tiles_x = (p.w + p.tx - 1) / p.tx;
    p.tiles_y = (p.h + p.ty - 1) / p.ty;
    p.tmem_cols = tmem_columns(p.nout);
    p.error = error;
    const size_t stage = (size_t)p.cin * 256 + (size_t)p.nout * p.cin * 2;
    const size_t extra = 8 * (2 * 4 + 1) + 32;
    int S = 4;
    while (S > 2 && S * stage + extra > SMEM_LIMIT)
        S--;
    if (S * stage + extra > SMEM_LIMIT)
        return cudaErrorInvalidValue;
    p.stages = S;
    size_t smem = smem_for_residency(S * stage + extra, p.tmem_cols);
    if (smem > SMEM_LIMIT)
        smem = SMEM_LIMIT;
    cudaError_t e = cudaFuncSetAttribute(k_conv3x3, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_LIMIT);
    if (e != cudaSuccess)
        return e;
    const long long tiles = (long long)p.tiles_x * p.tiles_y * p.n;
    if (tiles <= 0)
        return cudaSuccess;
    k_conv3x3<<<(unsigned)tiles, 128, smem, st>>>(*c.in_map, p);
    return cudaGetLastError();
}

cudaError_t conv3x3_wgrad(const WgradCall& c, int sm_count, uint32_t* error, cudaStream_t st)
{
    if (c.cin % 8 || c.cout % 16 || c.cout > 128 || c.x_c0 % 8 || c.g_c0 % 8)
        return cudaErrorInvalidValue;
    WgradParams p{};
    p.cin = c.cin;
    p.x_c0 = c.x_c0;
    p.cout = c.cout;
    p.g_c0 = c.g_c0;
    p.groups = 9 * c.cin / 8;
    p.n = c.n;
    p.h = c.h;
    p.w = c.w;
    wgrad_chunk_shape(p.w, p.tx, p.ty);
    p.chunks_x = (p.w + p.tx - 1) / p.tx;
    p.chunks_y = (p.h + p.ty - 1) / p.ty;
    p.chunks = p.chunks_x * p.chunks_y * p.n;
    if (p.chunks <= 0)
        return cudaSuccess;
    const int m_tiles = (p.groups + 15) / 16;
    int splits = std::max(1, (2 * sm_count + m_tiles - 1) / m_tiles);
    splits = std::min(splits, p.chunks);
    p.chunks_per_cta = (p.chunks + splits - 1) / splits;
    splits = (p.chunks + p.chunks_per_cta - 1) / p.chunks_per_cta;
    p.tmem_cols = tmem_columns(p.cout);
    p.dw = c.dw;
    p.error = error;
    const size_t stage = 16 * 1024 + (size_t)p.cout * 128;
    const size_t extra = 8 * (2 * 3 + 1) + 32;
    p.stages = 3;
    size_t smem = smem_for_residency(p.stages * stage + extra, p.tmem_cols);
    cudaError_t e = cudaFuncSetAttribute(k_wgrad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_LIMIT);
    if (e != cudaSuccess)
        return e;
    k_wgrad<<<dim3((unsigned)m_tiles, (unsigned)splits), 128, smem, st>>>(*c.x_map, *c.g_map, p);
    return cudaGetLastError();
}

} // namespace nn
} // namespace pt
