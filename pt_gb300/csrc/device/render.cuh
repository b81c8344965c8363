// render.cuh — camera rays, path loop and accumulation (pathtrace.rg.hlsl:9-68).
#pragma once
#include <cuda_fp16.h>

#include "shade.cuh"

namespace pt {

struct RenderArgs {
    DevScene s;
    float inv_view[12]; // first three rows, row-major
    float inv_proj[12];
    float near_plane, far_plane, focus_dist, lens_radius, exposure;
    uint32_t width, height, sample_index, samples, max_bounces, rr_start;
    float4* image;          // RGBA32F running mean (the accumulation image)
    double* sum64;          // optional FP64 sums: rgb + sample count per pixel
    float4* snapshot;       // optional: the running mean once it holds snapshot_after samples
    uint32_t snapshot_after;
    float4* feat_a;         // optional first-hit feature means: base colour + hit distance
    float4* feat_n;         //   and shading normal (PT_RENDER_FEATURES)
    uint32_t fp16_features; // feat_a, feat_n and snapshot hold 4 x FP16 per pixel (PT_RENDER_FEATURES_FP16)
    unsigned long long* counters; // [0] segments, [1] shadow rays, [2] paths, [3] node visits, [4] triangle tests
};

// sample_camera_ray (sample.hlsli:258-280)
__device__ __forceinline__ void camera_ray(const RenderArgs& a, uint32_t px, uint32_t py, f2 u_pixel, f2 u_lens, f3& origin, f3& dir)
{
    float fx = __uint2float_rn(px) + u_pixel.x, fy = __uint2float_rn(py) + u_pixel.y;
    float nx = (fx / __uint2float_rn(a.width)) * 2.0f - 1.0f;
    float ny = (fy / __uint2float_rn(a.height)) * 2.0f - 1.0f;
    const float* ip = a.inv_proj;
    f3 target = mk3(((ip[0] * nx + ip[1] * ny) + ip[2] * 1.0f) + ip[3] * 1.0f, ((ip[4] * nx + ip[5] * ny) + ip[6] * 1.0f) + ip[7] * 1.0f,
                    ((ip[8] * nx + ip[9] * ny) + ip[10] * 1.0f) + ip[11] * 1.0f);
    f3 ro = mk3(0.0f, 0.0f, 0.0f), rd = target;
    if (a.lens_radius > 0.0f) {
        f2 d = sample_concentric_disk(u_lens);
        f2 lp = {a.lens_radius * d.x, a.lens_radius * d.y};
        float t = a.focus_dist / -rd.z;
        f3 fp = ro + t * rd;
        ro = mk3(lp.x, lp.y, 0.0f);
        rd = fp - ro;
    }
    const float* iv = a.inv_view;
    origin = mk3(((iv[0] * ro.x + iv[1] * ro.y) + iv[2] * ro.z) + iv[3] * 1.0f, ((iv[4] * ro.x + iv[5] * ro.y) + iv[6] * ro.z) + iv[7] * 1.0f,
                 ((iv[8] * ro.x + iv[9] * ro.y) + iv[10] * ro.z) + iv[11] * 1.0f);
    dir = normalize(mk3(((iv[0] * rd.x + iv[1] * rd.y) + iv[2] * rd.z) + iv[3] * 0.0f,
                        ((iv[4] * rd.x + iv[5] * rd.y) + iv[6] * rd.z) + iv[7] * 0.0f,
                        ((iv[8] * rd.x + iv[9] * rd.y) + iv[10] * rd.z) + iv[11] * 0.0f));
}

// Feature and snapshot buffers: float4 per pixel, or 4 x FP16 (8 bytes) per
// pixel when `h` is set (values rounded to nearest on store).
__device__ __forceinline__ float4 feat_load(const float4* p, size_t i, uint32_t h)
{
    if (h) {
        const __half2* q = reinterpret_cast<const __half2*>(p) + 2 * i;
        const float2 a = __half22float2(q[0]), b = __half22float2(q[1]);
        return make_float4(a.x, a.y, b.x, b.y);
    }
    return p[i];
}

__device__ __forceinline__ void feat_store(float4* p, size_t i, float4 v, uint32_t h)
{
    if (h) {
        __half2* q = reinterpret_cast<__half2*>(p) + 2 * i;
        q[0] = __floats2half2_rn(v.x, v.y);
        q[1] = __floats2half2_rn(v.z, v.w);
        return;
    }
    p[i] = v;
}

// Running mean of pathtrace.rg.hlsl:62-67 with one sample per update (the
// reference dispatches one sample per submission in headless mode,
// ptdispatch.cpp:101).
__device__ __forceinline__ void accumulate(float4& acc, f3 r, uint32_t si)
{
    if (si == 0) {
        acc.x = r.x / 1.0f;
        acc.y = r.y / 1.0f;
        acc.z = r.z / 1.0f;
        acc.w = 1.0f;
    } else {
        float n = __uint2float_rn(si + 1u);
        acc.x = acc.x + (r.x - 1.0f * acc.x) / n;
        acc.y = acc.y + (r.y - 1.0f * acc.y) / n;
        acc.z = acc.z + (r.z - 1.0f * acc.z) / n;
    }
}

} // namespace pt
