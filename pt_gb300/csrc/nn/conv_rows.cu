// conv_rows.cu — persistent 3x3 convolution on tcgen05 with halo reuse.
//
// A work tile is MT image rows x 128 pixels.  For each 16-channel slice of
// the input, one TMA load per 8 channels brings the (MT + 2) x 130-pixel halo
// of the tile into shared memory as rows of 16 bytes (8 channels of one
// pixel).  In that layout 128 consecutive pixels of one row are a valid
// K-major operand (8-pixel core matrices 128 bytes apart), so the nine taps of
// the 3x3 stencil are nine descriptors into the same halo: offsets of
// (row + ky) * 130 + kx rows of 16 bytes.  The slice's weights for all nine
// taps arrive by one bulk copy.  Accumulators (MT x N fp32 columns) live in
// TMEM.
//
// Warp roles: warp 0 produces (TMA), warp 1 allocates TMEM and issues the
// MMAs, warps 2-5 drain the accumulators (bias, ReLU, gradient mask, store).
// One persistent CTA per SM with as many pipeline stages as shared memory
// holds; the accumulators are double-buffered in TMEM (2 x MT x N columns),
// so the MMAs of the next tile run while the epilogue drains this one.
#include <cuda_bf16.h>

#include <algorithm>
#include <cstdlib>

#include "nn.h"
#include "tc.cuh"

namespace pt {
namespace nn {

namespace {

constexpr int HALO_W = 130; // 128 pixels + one on each side
constexpr int KC = 16;      // input channels per pipeline stage

struct RowsParams {
    int cin, c0, nout, mt;
    const uint16_t* wpk; // [cin/16][9][2][nout][8]
    const float* bias;
    int relu;
    uint16_t* out;
    int out_pitch, out_c0;
    float* out_f32;
    const float* residual;
    const uint16_t* mask;
    int mask_pitch, mask_c0;
    int n, h, w, tiles_x, tiles_y, tiles;
    int stages;
    uint32_t tmem_cols; // one accumulator buffer; the CTA allocates two
    uint32_t* error;
};

__device__ __forceinline__ bool bf16_pos(uint16_t b)
{
    return (b & 0x8000u) == 0 && (b & 0x7FFFu) != 0;
}

__device__ __forceinline__ uint32_t pack2(float a, float b)
{
    __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&v);
}

__device__ __forceinline__ bool failed(volatile uint32_t* fail)
{
    return *fail != 0;
}

__global__ void __launch_bounds__(192) k_conv3x3_rows(const __grid_constant__ CUtensorMap amap, RowsParams p)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    const int MT = p.mt;
    // one 8-channel halo, rounded up so every TMA destination is 128-byte aligned
    const uint32_t a_real = (uint32_t)(MT + 2) * HALO_W * 16; // bytes one halo load delivers
    const uint32_t a_box = (a_real + 127u) & ~127u;
    const uint32_t a_bytes = 2 * a_box;
    const uint32_t b_tap = (uint32_t)p.nout * 32; // 16 channels x N x 2 bytes
    const uint32_t b_bytes = 9 * b_tap;
    const uint32_t stage_bytes = a_bytes + b_bytes;
    const int S = p.stages;
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + (size_t)S * stage_bytes);
    uint64_t* empty = full + S;
    uint64_t* acc_full = empty + S;     // [2]: buffer b holds a finished tile
    uint64_t* acc_empty = acc_full + 2; // [2]: buffer b was drained
    uint32_t* tslot = reinterpret_cast<uint32_t*>(acc_empty + 2);
    volatile uint32_t* fail = tslot + 1;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int chunks = p.cin / KC;

    if (threadIdx.x == 0) {
        for (int s = 0; s < S; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; b++) {
            mbar_init(&acc_full[b], 1);
            mbar_init(&acc_empty[b], 4);
        }
        *fail = 0;
        mbar_init_fence();
    }
    if (warp == 1) {
        tmem_alloc(tslot, 2 * p.tmem_cols);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;

    if (warp == 0) {
        if (lane == 0) {
            uint32_t it = 0;
            for (int t = blockIdx.x; t < p.tiles && !failed(fail); t += gridDim.x) {
                int q = t;
                const int txi = q % p.tiles_x;
                q /= p.tiles_x;
                const int tyi = q % p.tiles_y;
                const int img = q / p.tiles_y;
                const int x0 = txi * 128, y0 = tyi * MT;
                for (int c = 0; c < chunks; c++, it++) {
                    const uint32_t s = it % S;
                    if (it >= (uint32_t)S && !mbar_wait(&empty[s], ((it / S) - 1) & 1u)) {
                        atomicOr((uint32_t*)fail, 1u);
                        break;
                    }
                    uint8_t* sa = smem + (size_t)s * stage_bytes;
                    mbar_expect_tx(&full[s], 2 * a_real + b_bytes);
                    tma_load_4d(sa, &amap, &full[s], p.c0 + KC * c, x0 - 1, y0 - 1, img);
                    tma_load_4d(sa + a_box, &amap, &full[s], p.c0 + KC * c + 8, x0 - 1, y0 - 1, img);
                    bulk_load(sa + a_bytes, p.wpk + (size_t)c * 9 * 2 * p.nout * 8, b_bytes, &full[s]);
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            const uint32_t idesc = idesc_bf16(128, (uint32_t)p.nout, false, false);
            const uint32_t b_lbo = (uint32_t)p.nout * 16;
            uint32_t it = 0, tc = 0;
            for (int t = blockIdx.x; t < p.tiles && !failed(fail); t += gridDim.x, tc++) {
                // buffer b's previous tile (two tiles back) must have been drained
                const uint32_t b = tc & 1u, use = tc >> 1;
                if (use > 0 && !mbar_wait(&acc_empty[b], (use - 1) & 1u)) {
                    atomicOr((uint32_t*)fail, 1u);
                    break;
                }
                tc_fence_after();
                const uint32_t acc = tmem + b * p.tmem_cols;
                for (int c = 0; c < chunks; c++, it++) {
                    const uint32_t s = it % S;
                    if (!mbar_wait(&full[s], (it / S) & 1u)) {
                        atomicOr((uint32_t*)fail, 1u);
                        break;
                    }
                    tc_fence_after();
                    const uint32_t sa = smem_addr(smem + (size_t)s * stage_bytes);
                    const uint32_t sb = sa + a_bytes;
                    for (int r = 0; r < MT; r++) {
                        for (int tap = 0; tap < 9; tap++) {
                            const int ky = tap / 3, kx = tap % 3;
                            const uint32_t a_off = (uint32_t)((r + ky) * HALO_W + kx) * 16u;
                            const uint64_t ad = smem_desc(sa + a_off, a_box, 128u);
                            const uint64_t bd = smem_desc(sb + (uint32_t)tap * b_tap, b_lbo, 128u);
                            mma_bf16(acc + (uint32_t)(r * p.nout), ad, bd, idesc, (c | tap) != 0);
                        }
                    }
                    mma_commit(&empty[s]);
                }
                mma_commit(&acc_full[b]);
            }
        }
    } else {
        // epilogue warps 2..5 drain TMEM lanes 32 * (warp % 4) ..
        const int quarter = warp & 3;
        const int m = quarter * 32 + lane;
        uint32_t tc = 0;
        for (int t = blockIdx.x; t < p.tiles; t += gridDim.x, tc++) {
            const uint32_t b = tc & 1u, use = tc >> 1;
            const bool ok = !failed(fail) && mbar_wait(&acc_full[b], use & 1u);
            // warp-uniform decision before the warp-collective TMEM loads
            if (__any_sync(0xffffffffu, !ok)) {
                if (lane == 0)
                    atomicOr((uint32_t*)fail, 1u);
                break;
            }
            tc_fence_after();
            int q = t;
            const int txi = q % p.tiles_x;
            q /= p.tiles_x;
            const int tyi = q % p.tiles_y;
            const int img = q / p.tiles_y;
            const int px = txi * 128 + m;
            for (int r = 0; r < MT; r++) {
                const int py = tyi * MT + r;
                const bool valid = px < p.w && py < p.h;
                const size_t pix = ((size_t)img * p.h + py) * p.w + px;
                for (int j = 0; j < p.nout / 16; j++) {
                    uint32_t v32[16];
                    tmem_ld16(tmem + b * p.tmem_cols + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(r * p.nout + j * 16), v32);
                    if (!valid)
                        continue;
                    float v[16];
#pragma unroll
                    for (int k = 0; k < 16; k++) {
                        v[k] = __uint_as_float(v32[k]);
                        if (p.bias)
                            v[k] += p.bias[j * 16 + k];
                        if (p.relu)
                            v[k] = fmaxf(v[k], 0.0f);
                    }
                    if (p.mask) {
                        const uint4* mp = reinterpret_cast<const uint4*>(p.mask + pix * p.mask_pitch + p.mask_c0 + j * 16);
                        const uint4 q0 = mp[0], q1 = mp[1];
                        const uint32_t mw[8] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w};
#pragma unroll
                        for (int k = 0; k < 8; k++) {
                            if (!bf16_pos((uint16_t)(mw[k] & 0xFFFFu)))
                                v[2 * k] = 0.0f;
                            if (!bf16_pos((uint16_t)(mw[k] >> 16)))
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
                        o[0] = make_uint4(pack2(v[0], v[1]), pack2(v[2], v[3]), pack2(v[4], v[5]), pack2(v[6], v[7]));
                        o[1] = make_uint4(pack2(v[8], v[9]), pack2(v[10], v[11]), pack2(v[12], v[13]), pack2(v[14], v[15]));
                    }
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0)
                asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(&acc_empty[b])) : "memory");
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        tmem_dealloc(tmem, 2 * p.tmem_cols);
    }
    if (threadIdx.x == 0 && *fail)
        atomicOr(p.error, 1u);
}

__global__ void k_pack_rows(const float* w, int cin, int cout, uint16_t* fwd, uint16_t* bwd)
{
    const size_t n = (size_t)9 * cin * cout;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int co = (int)(i % cout);
        const int ci = (int)((i / cout) % cin);
        const int tap = (int)(i / ((size_t)cout * cin));
        __nv_bfloat16 b = __float2bfloat16_rn(w[i]);
        const uint16_t bits = *reinterpret_cast<uint16_t*>(&b);
        // forward GEMM: K = ci, N = co -> [ci/16][tap][(ci/8)%2][co][ci%8]
        fwd[((((size_t)(ci / 16) * 9 + tap) * 2 + (ci / 8) % 2) * cout + co) * 8 + ci % 8] = bits;
        // data gradient: K = co, N = ci, mirrored taps -> [co/16][8-tap][(co/8)%2][ci][co%8]
        bwd[((((size_t)(co / 16) * 9 + (8 - tap)) * 2 + (co / 8) % 2) * cin + ci) * 8 + co % 8] = bits;
    }
}

uint32_t pow2_cols(uint32_t n)
{
    uint32_t c = 32;
    while (c < n)
        c <<= 1;
    return c;
}

typedef CUresult (*EncodeTiled)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*, const cuuint64_t*,
                                const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

} // namespace

bool use_rows_kernel()
{
    const char* e = getenv("PT_CONV_KERNEL");
    return !(e && e[0] == 't');
}

int rows_per_tile(int nout)
{
    int mt = 256 / nout;
    return std::max(1, std::min(8, mt));
}

cudaError_t pack_weights_rows(const float* w, int cin, int cout, uint16_t* fwd, uint16_t* bwd, cudaStream_t st)
{
    if (cin % 16 || cout % 16)
        return cudaErrorInvalidValue;
    size_t n = (size_t)9 * cin * cout;
    unsigned blocks = (unsigned)std::min<size_t>((n + 255) / 256, 152 * 32);
    k_pack_rows<<<blocks ? blocks : 1, 256, 0, st>>>(w, cin, cout, fwd, bwd);
    return cudaGetLastError();
}

cudaError_t conv3x3_rows(const ConvCall& c, const CUtensorMap* halo_map, int sm_count, uint32_t* error, cudaStream_t st)
{
    if (c.cin % 16 || c.nout % 16 || c.nout < 16 || c.nout > 256 || c.c0 % 8 || c.out_c0 % 8 || (c.mask && c.mask_c0 % 8))
        return cudaErrorInvalidValue;
    if (c.out.n != c.in.n || c.out.h != c.in.h || c.out.w != c.in.w)
        return cudaErrorInvalidValue;
    RowsParams p{};
    p.cin = c.cin;
    p.c0 = c.c0;
    p.nout = c.nout;
    p.mt = rows_per_tile(c.nout);
    p.wpk = c.wpk;
    p.bias = c.bias;
    p.relu = c.relu ? 1 : 0;
    p.out = c.out.p;
    p.out_pitch = c.out.pitch;
    p.out_c0 = c.out_c0;
    p.out_f32 = c.out_f32;
    p.residual = c.out_f32 ? c.residual : nullptr;
    p.mask = c.mask ? c.mask->p : nullptr;
    p.mask_pitch = c.mask ? c.mask->pitch : 0;
    p.mask_c0 = c.mask_c0;
    p.n = c.in.n;
    p.h = c.in.h;
    p.w = c.in.w;
    p.tiles_x = (p.w + 127) / 128;
    p.tiles_y = (p.h + p.mt - 1) / p.mt;
    p.tiles = p.tiles_x * p.tiles_y * p.n;
    p.tmem_cols = pow2_cols((uint32_t)(p.mt * p.nout));
    p.error = error;
    if (p.tiles <= 0)
        return cudaSuccess;
    const size_t a_box = ((size_t)(p.mt + 2) * HALO_W * 16 + 127) & ~(size_t)127;
    const size_t stage = 2 * a_box + (size_t)9 * p.nout * 32;
    const size_t extra = 8 * (2 * 8 + 4) + 64;
    const size_t smem_max = 232448; // one CTA per SM: all of its shared memory
    int S = 8;
    while (S > 2 && S * stage + extra > smem_max)
        S--;
    if (S * stage + extra > smem_max || 2 * p.tmem_cols > 512)
        return cudaErrorInvalidValue;
    p.stages = S;
    const size_t smem = S * stage + extra;
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(k_conv3x3_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, 232448);
        if (e == cudaSuccess) // all of L1 as shared memory
            e = cudaFuncSetAttribute(k_conv3x3_rows, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
        if (e != cudaSuccess)
            return e;
        attr = true;
    }
    // one CTA per SM (its two accumulator buffers may take all 512 TMEM columns)
    const int grid = std::min(p.tiles, sm_count);
    k_conv3x3_rows<<<grid, 192, smem, st>>>(*halo_map, p);
    return cudaGetLastError();
}

} // namespace nn
} // namespace pt
