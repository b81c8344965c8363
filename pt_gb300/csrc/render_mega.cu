// render_mega.cu — megakernel path tracer: one thread owns one pixel and runs
// its samples back to back, tracing closest-hit and shadow rays inline.
#include "device/render.cuh"
#include "kernels.h"

namespace pt {

__device__ __forceinline__ void shade_segment(const DevScene& s, PathState& pl, f3 ro, f3 rd, bool hit, const Hit& h, uint32_t& shadow_rays,
                                              TraceCounters& tc)
{
    if (!hit) {
        shade_miss(s, pl);
        return;
    }
    NeeRequest nee;
    nee.add = false;
    nee.trace = false;
    NeeKeep keep{nee};
    shade_hit(s, pl, ro, rd, h, keep);
    float vis = 0.0f;
    if (nee.trace) {
        shadow_rays++;
        vis = trace_shadow(s, nee.origin, nee.dir, 0.0f, nee.tmax, tc);
    }
    finish_nee(pl.radiance, nee, vis);
}

// One block = a TW x (128 / TW) pixel tile.
template <int TW>
__global__ void __launch_bounds__(128) k_megakernel(RenderArgs a)
{
    const uint32_t px = blockIdx.x * TW + (threadIdx.x % TW);
    const uint32_t py = blockIdx.y * (128 / TW) + (threadIdx.x / TW);
    uint32_t segments = 0, shadow_rays = 0, paths = 0;
    TraceCounters tc{0u, 0u};
    if (px < a.width && py < a.height) {
        const size_t pix = (size_t)py * a.width + px;
        float4 acc = a.image[pix];
        // FP64 sums are added sample by sample in the oracle's order.
        double s64[3] = {0.0, 0.0, 0.0};
        if (a.sum64) {
            s64[0] = a.sum64[4 * pix + 0];
            s64[1] = a.sum64[4 * pix + 1];
            s64[2] = a.sum64[4 * pix + 2];
        }
        const DevScene& s = a.s;
        float4 fa = make_float4(0.0f, 0.0f, 0.0f, 0.0f), fn = fa;
        if (a.feat_a) {
            fa = feat_load(a.feat_a, pix, a.fp16_features);
            fn = feat_load(a.feat_n, pix, a.fp16_features);
        }
        for (uint32_t si = a.sample_index; si < a.sample_index + a.samples; si++) {
            PathState pl;
            pl.radiance = mk3(0.0f, 0.0f, 0.0f);
            sampler_start(pl.smp, px, py, si, 0);
            f2 u_pixel = sample_2d(pl.smp);
            f2 u_lens = sample_2d(pl.smp);
            f3 ro, rd;
            camera_ray(a, px, py, u_pixel, u_lens, ro, rd);
            sampler_start(pl.smp, px, py, si, 1);
            pl.throughput = mk3(1.0f, 1.0f, 1.0f);
            pl.brdf_pdf = -1.0f;
            pl.final_segment = (a.max_bounces == 0);
            paths++;
            segments++;
            Hit h;
            bool hit = trace_closest(s, ro, rd, a.near_plane, a.far_plane, h, tc);
            if (a.feat_a) {
                f3 alb = mk3(0.0f, 0.0f, 0.0f), nrm = alb;
                if (hit)
                    hit_features(s, h, rd, alb, nrm);
                feature_mean(fa, make_float4(alb.x, alb.y, alb.z, hit ? h.t : 0.0f), si);
                feature_mean(fn, make_float4(nrm.x, nrm.y, nrm.z, 0.0f), si);
            }
            shade_segment(s, pl, ro, rd, hit, h, shadow_rays, tc);
            if (!pl.final_segment) {
                for (uint32_t seg = 1; seg <= a.max_bounces; seg++) {
                    sampler_start(pl.smp, px, py, si, seg + 1);
                    ro = pl.next_o;
                    rd = pl.next_d;
                    pl.final_segment = seg >= a.max_bounces;
                    segments++;
                    hit = trace_closest(s, ro, rd, 0.0f, __int_as_float(0x7f800000), h, tc);
                    shade_segment(s, pl, ro, rd, hit, h, shadow_rays, tc);
                    if (pl.final_segment)
                        break;
                    if (seg >= a.rr_start && russian_roulette(pl))
                        break;
                }
            }
            f3 r = correct_radiance(pl.radiance * a.exposure);
            accumulate(acc, r, si);
            if (a.snapshot && si + 1 == a.snapshot_after)
                feat_store(a.snapshot, pix, acc, a.fp16_features);
            s64[0] += (double)r.x;
            s64[1] += (double)r.y;
            s64[2] += (double)r.z;
        }
        a.image[pix] = acc;
        if (a.feat_a) {
            feat_store(a.feat_a, pix, fa, a.fp16_features);
            feat_store(a.feat_n, pix, fn, a.fp16_features);
        }
        if (a.sum64) {
            double* d = a.sum64 + 4 * pix;
            d[0] = s64[0];
            d[1] = s64[1];
            d[2] = s64[2];
            d[3] += (double)a.samples;
        }
    }
    // warp-aggregated counters
    unsigned mask = 0xffffffffu;
    segments = __reduce_add_sync(mask, segments);
    shadow_rays = __reduce_add_sync(mask, shadow_rays);
    paths = __reduce_add_sync(mask, paths);
    uint32_t nodes = __reduce_add_sync(mask, tc.nodes);
    uint32_t tris = __reduce_add_sync(mask, tc.tris);
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(a.counters + 0, (unsigned long long)segments);
        atomicAdd(a.counters + 1, (unsigned long long)shadow_rays);
        atomicAdd(a.counters + 2, (unsigned long long)paths);
        atomicAdd(a.counters + 3, (unsigned long long)nodes);
        atomicAdd(a.counters + 4, (unsigned long long)tris);
    }
}

cudaError_t launch_megakernel_tiled(const RenderArgs& a, uint32_t tile_w, cudaStream_t stream)
{
    const uint32_t th = 128 / tile_w;
    dim3 grid((a.width + tile_w - 1) / tile_w, (a.height + th - 1) / th);
    switch (tile_w) {
    case 8:
        k_megakernel<8><<<grid, 128, 0, stream>>>(a);
        break;
    case 16:
        k_megakernel<16><<<grid, 128, 0, stream>>>(a);
        break;
    case 32:
        k_megakernel<32><<<grid, 128, 0, stream>>>(a);
        break;
    default:
        return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_megakernel(const RenderArgs& a, cudaStream_t stream) { return launch_megakernel_tiled(a, 16, stream); }

} // namespace pt

namespace pt {

cudaError_t render_init_tables(const uint32_t* table128, const float* srgb256, cudaStream_t stream)
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

} // namespace pt
