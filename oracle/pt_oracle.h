/*
 * pt_oracle.h — CPU oracle of pt's headless path-tracing path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (libptgpu.so, the `pt`
 * CLI, the Python package) links, loads or calls this code.  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg use it, as the
 * checker of the CUDA path and as the timed CPU baseline ("port").
 *
 * What it restates (reference file:line in anveba/pt):
 *   - Sobol'/Owen sampler: shaders/pathtrace/sample.hlsli:94-166, util.hlsli:8-27
 *   - camera ray: sample.hlsli:258-280
 *   - ray generation / accumulation: pathtrace.rg.hlsl:9-68, pathtrace.hlsli:118-139
 *   - closest hit, BSDF, NEE: pathtrace.ch.hlsl:32-360, lightsample.hlsli:13-143,
 *     geometry.hlsli:38-69, material.hlsli:93-172, sample.hlsli:193-246
 *   - miss / shadow: pathtrace.ms.hlsl:6-11, shadowray.ah.hlsl:12-40, shadowray.ms.hlsl:3-7
 *   - host RNG: src/rng.cpp:24-60; alias tables: src/aliastable.h:21-67
 *   - scene packing: src/scene/scenebuffer.cpp:65-168, src/scene/lightsample.cpp:5-221
 *   - camera matrices: src/scene/camera.h:16, camera.cpp:21-26, scenebuild.cpp:184-191,
 *     pathtrace.cpp:381-396
 *   - MSE: util/meansq/meansq.cpp:34-43
 * The reference's ray traversal is the Vulkan driver's (closed); here it is a
 * binned-SAH BVH2 with a watertight ray/triangle test (Woop, Benthin & Wald
 * 2013), conservative box tests and a (t, instance, primitive) tie-break, so
 * the closest hit is the exact argmin over all triangles, independent of the
 * BVH.  Parity of the shader restatement is pinned by source semantics only
 * (the HLSL cannot run on this machine); the host pieces (RNG, alias tables,
 * light stream, camera matrices, sRGB decode, MSE) are pinned against the
 * reference's own C++ compiled from its sources (oracle/build_ref.sh).
 */
#ifndef PT_ORACLE_H_INCLUDED
#define PT_ORACLE_H_INCLUDED

#include <stddef.h>
#include <stdint.h>

#include "../include/pt_gpu.h"
#include "../include/pt_scene.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- integer sampler pieces (sample.hlsli, util.hlsli) ---- */
uint32_t or_hash(uint32_t x);
uint32_t or_hash_combine(uint32_t seed, uint32_t x);
uint32_t or_sobol(uint32_t index, uint32_t dimension);
uint32_t or_scramble(uint32_t x, uint32_t seed);
/* Draw a sequence from the per-pixel sampler: kinds[i] = 1 (sample_1d) or
 * 2 (sample_2d); writes 1 or 2 floats per draw into out. Returns floats written. */
uint32_t or_sampler_sequence(uint32_t px, uint32_t py, uint32_t sample_index, uint32_t seed,
                             const uint8_t* kinds, uint32_t n, float* out);

/* ---- float functions shared by oracle and device (same method, same bits) ---- */
float or_sin(float x);
float or_cos(float x);

/* ---- host RNG (src/rng.cpp) ---- */
void or_xshiro128_stream(const uint32_t seed4[4], uint32_t n, uint32_t* out_u32, float* out_f32);
void or_splitmix32_stream(uint32_t state, uint32_t n, uint32_t* out);

/* ---- alias table (src/aliastable.h:21-67) ---- */
void or_alias_build(const float* weights, uint32_t n, float* p, float* q, uint32_t* alias);

/* ---- colour / camera ---- */
float or_from_srgb(float x);
void or_camera_params(const pt_camera_desc* cam, uint32_t width, uint32_t height, pt_render_params* out);

/* ---- scene packing (scenebuffer.cpp + lightsample.cpp) ---- */
typedef struct or_packed or_packed;
or_packed* or_pack(const pt_raw_scene* raw);
void or_packed_view(const or_packed* p, pt_scene_view* out);
void or_packed_free(or_packed* p);

/* ---- rendering ---- */
typedef struct or_stats {
    uint64_t segments;      /* traced primary + extension rays      */
    uint64_t shadow_rays;   /* traced shadow rays                    */
    uint64_t paths;
    uint64_t node_visits;   /* interior BVH2 nodes visited (TLAS+BLAS), all rays */
    uint64_t tri_tests;     /* ray/triangle tests, all rays          */
    uint64_t inst_visits;   /* instance (BLAS) entries               */
    uint64_t ray_count;     /* rays traversed (segments + shadow)    */
} or_stats;

typedef struct or_scene or_scene;
/* brute_force != 0: test every triangle of every instance (no BVH). */
or_scene* or_scene_create(const pt_scene_view* view, int brute_force);
void or_scene_destroy(or_scene* s);
/* One texture lookup of the scene's texture `index` at (u, v): bilinear,
 * REPEAT, level 0, sRGB decode for sRGB textures (material.hlsli
 * SampleLevel with the sampler of src/graphics/sampler.cpp:8-22). */
void or_texture_sample(const or_scene* s, uint32_t index, float u, float v, float out[4]);

/* Render rows [row_begin, row_end) of params->samples samples starting at
 * params->sample_index.  rgba (width*height*4 floats) holds the running mean
 * as the reference keeps it; sum64 (may be NULL) accumulates the corrected
 * radiance of each sample in FP64 (rgb + count in alpha).  threads <= 0 uses
 * all OpenMP threads. */
int or_render(or_scene* s, const pt_render_params* params, uint32_t row_begin, uint32_t row_end,
              float* rgba, double* sum64, or_stats* stats, int threads);

/* Trace one path and report its hit sequence (instance<<32 | primitive per
 * segment, ~0 for a miss); returns the number of entries written. */
uint32_t or_path_signature(or_scene* s, const pt_render_params* params, uint32_t px, uint32_t py,
                           uint32_t sample_index, uint64_t* out, uint32_t cap);

/* Closest hit of one world-space ray: returns 1 on hit and fills t, b1, b2,
 * instance, primitive. */
int or_intersect(or_scene* s, const float o[3], const float d[3], float tmin, float tmax,
                 float* t, float* b1, float* b2, uint32_t* instance, uint32_t* primitive);

/* util/meansq semantics: SSE over RGB / (w*h*3 - 1), FP64. */
double or_meansq(const float* reference_rgba, const float* image_rgba, uint32_t width, uint32_t height);
double or_meansq64(const double* reference_rgb_mean, const float* image_rgba, uint32_t width, uint32_t height);

int or_max_threads(void);

/* ACES tone map of tonemap.cs.hlsl:17-77 in place (src linear, dst sRGB). */
void or_tonemap(float* rgba, uint64_t pixels);

#ifdef __cplusplus
}
#endif

#endif
