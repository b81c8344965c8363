/*
 * pt_gpu.h — C ABI of the GB300 path-tracing library (libptgpu.so).
 *
 * This header is the drop-in boundary for pt's headless path-tracing path.
 * Each entry point names the interface of the reference (anveba/pt) that it
 * replaces, as file:line within that project.  No C++ or torch types cross
 * this boundary: plain pointers, sizes and status codes only.
 *
 * Ownership: the caller owns every host array passed in (borrowed for the
 * duration of the call only); a pt_ctx owns all device memory it allocates;
 * results are copied into caller buffers.  A pt_ctx is thread-compatible
 * (one thread at a time), not thread-safe.  No exception crosses the ABI:
 * every call returns a pt_status and pt_last_error() explains the last one.
 */
#ifndef PT_GPU_H_INCLUDED
#define PT_GPU_H_INCLUDED

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PT_ABI_VERSION 2

/* Status codes (0 = ok, < 0 = error class).  The reference throws
 * std::runtime_error instead (e.g. src/pathtrace/ptdispatch.cpp:44-47,127-128). */
typedef enum pt_status {
    PT_OK = 0,
    PT_ERR_INVALID = -1,     /* bad argument or malformed scene data            */
    PT_ERR_CUDA = -2,        /* CUDA runtime error                              */
    PT_ERR_OOM = -3,         /* device or host allocation failed                */
    PT_ERR_STATE = -4,       /* call out of order (e.g. render before upload)   */
    PT_ERR_TIMEOUT = -5,     /* a device loop hit its iteration cap            */
    PT_ERR_DEVICE = -6,      /* a kernel reported an error word (bounds etc.)   */
    PT_ERR_IO = -7,          /* file could not be read or written               */
    PT_ERR_UNSUPPORTED = -8  /* feature outside what this build implements      */
} pt_status;

/* ---- Constants shared with the reference's device contract (share/constants.h:3-28) ---- */
#define PT_BASE_COLOUR_MAP_BIT (1u << 0)
#define PT_EMISSION_MAP_BIT (1u << 1)
#define PT_ROUGHNESS_MAP_BIT (1u << 2)
#define PT_METALNESS_MAP_BIT (1u << 3)
#define PT_ROUGHNESS_METALNESS_MAP_BIT (1u << 4)
#define PT_SPECULAR_MAP_BIT (1u << 5)
#define PT_SPECULAR_TINT_MAP_BIT (1u << 6)
#define PT_SHEEN_MAP_BIT (1u << 7)
#define PT_SHEEN_TINT_MAP_BIT (1u << 8)
#define PT_CLEARCOAT_MAP_BIT (1u << 9)
#define PT_CLEARCOAT_ROUGHNESS_MAP_BIT (1u << 10)
#define PT_ANISOTROPY_MAP_BIT (1u << 11)
#define PT_NORMAL_MAP_BIT (1u << 12)
#define PT_MATERIAL_IS_TRANSPARENT_BIT (1u << 13)
#define PT_ANY_MAP_BITS 0x1FFFu

#define PT_LIGHT_TYPE_POINT 1u
#define PT_LIGHT_TYPE_DIRECTIONAL 2u
#define PT_LIGHT_TYPE_EMITTER 3u
#define PT_NO_EMITTER_INDEX 0xFFFFFFFFu
#define PT_LIGHT_BIN_SIZE 10u   /* u32 words per light alias-table bin   */
#define PT_EMITTER_BIN_SIZE 6u  /* u32 words per emitter-triangle bin    */

/* ---- Scene data contract (the reference's SceneBuffer regions) ---- */

/* Vertex: 32 B = position xyz, normal xyz, uv (src/scene/mesh.h:10-18;
 * read on the device as two float4, shaders/pathtrace/geometry.hlsli:27-36). */
#define PT_VERTEX_FLOATS 8

/* Per-mesh ranges into the flat vertex/index arrays (the reference's
 * SceneBuffer::start_indices, src/scene/scenebuffer.cpp:116-132). */
typedef struct pt_mesh_range {
    uint32_t vertex_offset; /* first vertex of the mesh in the vertex array  */
    uint32_t index_offset;  /* first index (3 per triangle) in index array   */
    uint32_t tri_count;
    uint32_t vertex_count;
} pt_mesh_range;

/* InstanceData, 128 B (src/scene/scenebuffer.h:13-24): transform is the
 * object-to-world matrix stored row-major (world = transform * p); normal
 * holds the rows of the normal matrix (inverse-transpose), each padded to
 * 16 B, as the shaders read it (shaders/pathtrace/geometry.hlsli:4-11). */
typedef struct pt_instance_data {
    uint32_t vertex_index;
    uint32_t index_index;
    uint32_t emitter_index;  /* PT_NO_EMITTER_INDEX if not emissive */
    uint32_t material_index;
    float transform[4][4];
    float normal[3][4];
} pt_instance_data;

/* PbrMaterial, 96 B (src/scene/material.h:24-29). rough_metal_normal_map_bits[3]
 * carries the map bits as raw u32 bits. */
typedef struct pt_material {
    float base_colour[4];
    float emission[4]; /* rgb, a = strength */
    float rough_metal_normal_map_bits[4];
    float specular[4];
    float sheen[4];
    float cc_ccrgh_aniso[4];
} pt_material;

/* A borrowed view of a packed scene.  Mirrors the descriptor bindings 3-6 and
 * 9 of the reference (src/pathtrace/pathtrace.cpp:36-69) plus the per-instance
 * data the reference hands to the driver's acceleration-structure build
 * (src/pathtrace/accstruct.cpp:186-218). */
/* One texture (TextureData, src/scene/texturedata.cpp:30-60): 8-bit texels,
 * 1, 2 or 4 channels (3-channel images are stored as 4 with alpha 255),
 * rows from the top of the image; srgb = 1 when the colour channels are
 * sRGB-encoded (VK_FORMAT_R8G8B8A8_SRGB: base colour and emission maps,
 * scene.cpp:42-48).  Sampled bilinearly with REPEAT addressing at level 0
 * (src/graphics/sampler.cpp:8-22). */
typedef struct pt_texture {
    uint64_t offset; /* byte offset of texel (0, 0) in the texel array */
    uint32_t width;
    uint32_t height;
    uint32_t channels; /* 1, 2 or 4 */
    uint32_t srgb;     /* 0 or 1 */
} pt_texture;

typedef struct pt_scene_view {
    const float* vertices;   /* vertex_count * PT_VERTEX_FLOATS */
    uint32_t vertex_count;
    const uint32_t* indices; /* mesh-local vertex indices, 3 per triangle */
    uint32_t index_count;
    const pt_mesh_range* meshes;
    uint32_t mesh_count;
    const pt_instance_data* instances;
    const uint32_t* instance_mesh; /* mesh (BLAS) of each instance */
    /* Optional: world-to-object affine transform per instance, 12 floats
     * row-major (3x4).  NULL lets the library derive it from transform. */
    const float* instance_world_to_object;
    const uint8_t* instance_opaque; /* optional; NULL = all opaque (accstruct.cpp:212-214) */
    uint32_t instance_count;
    const pt_material* materials;
    uint32_t material_count;
    const uint32_t* light_words; /* light-sampler stream (lightsample.cpp:89-221) */
    uint32_t light_word_count;
    uint32_t light_count;        /* bins of the top-level light alias table */
    float environment_colour[3]; /* linear (already sRGB-decoded) */
    /* Textures referenced by materials' map bits (may be empty). */
    const uint8_t* texels;
    uint64_t texel_bytes;
    const pt_texture* textures;
    uint32_t texture_count;
    /* Optional (NULL = none), material_count entries.  An extension of this
     * library (the reference's materials have no refraction): a material
     * whose entry is > 0 is a smooth dielectric of that index of refraction
     * against vacuum.  It reflects or refracts by the exact Fresnel
     * reflectance, tints refracted light by its base colour, takes no light
     * samples (a delta BSDF, so emission reached through it counts in full),
     * and is opaque to shadow rays.  Entries must be 0 or finite and >= 1. */
    const float* material_ior;
} pt_scene_view;

/* Accumulation modes. */
#define PT_ACCUM_FP32 0u      /* running mean in FP32, as the reference       */
#define PT_ACCUM_FP32_FP64 1u /* additionally sum radiance in FP64 (oracle)   */

/* Kernel strategy (chosen by the autotuner when PT_KERNEL_AUTO). */
#define PT_KERNEL_AUTO 0u
#define PT_KERNEL_MEGA 1u
#define PT_KERNEL_WAVEFRONT 2u

/* Render parameters: the reference's UniformBufferObject
 * (src/pathtrace/pathtrace.h:21-41, shaders/pathtrace/pathtrace.hlsli:8-29). */
typedef struct pt_render_params {
    float inv_view[16]; /* row-major, as uploaded (pathtrace.cpp:387-388) */
    float inv_proj[16];
    float near_plane;
    float far_plane;
    float focus_dist;
    float lens_radius;
    float exposure;
    uint32_t width;
    uint32_t height;
    uint32_t sample_index; /* first sample of this call; 0 resets the image */
    uint32_t samples;      /* samples per pixel rendered by this call      */
    uint32_t max_bounces;
    uint32_t accum_mode;   /* PT_ACCUM_*  */
    uint32_t kernel;       /* PT_KERNEL_* */
    uint32_t rr_start;     /* first segment with Russian roulette; 1 = reference */
    uint32_t flags;        /* PT_RENDER_* (0 = the reference's behaviour)        */
    uint32_t reserved[2];
} pt_render_params;

/* pt_render_params.flags: also accumulate, over every sample of the image, the
 * first-hit features the denoiser reads (base colour, shading normal facing
 * the camera, hit distance; zero where the camera ray escapes), as running
 * means like the image.  The rendered image is unchanged. */
#define PT_RENDER_FEATURES 1u
/* pt_render_params.flags: time the wavefront's stages with CUDA events
 * recorded between its launches (pt_render_stats.stage_ms). */
#define PT_RENDER_TIME_STAGES 2u
/* pt_render_params.flags (with PT_RENDER_FEATURES or an armed snapshot, and
 * for pt_render_features): store the denoiser's feature buffers and the
 * half-sample snapshot as 4 x FP16 per pixel instead of 4 x FP32 (running
 * means are updated in FP32 and rounded to nearest on every store).  The
 * image itself stays FP32. */
#define PT_RENDER_FEATURES_FP16 4u
/* pt_render_params.flags: clear the image and the FP64 sums before this call
 * even when sample_index > 0.  For replicas rendering a sample range
 * [sample_index, sample_index + samples) of a larger render on another GPU:
 * their FP64 sums (PT_IMAGE_SUMS64) are that range's contribution; the FP32
 * image of such a call is not a mean of anything and is not meant to be read. */
#define PT_RENDER_RESTART 8u

/* Counters of the last pt_render call. */
typedef struct pt_render_stats {
    uint64_t segments;        /* traced primary + extension rays           */
    uint64_t shadow_rays;     /* traced NEE shadow rays                    */
    uint64_t paths;           /* pixel samples                             */
    uint64_t node_visits;     /* BVH interior nodes whose children were tested */
    uint64_t tri_tests;       /* ray/triangle tests                        */
    float milliseconds;       /* device time of the render (CUDA events)   */
    uint32_t kernel_launches; /* kernels launched by the call              */
    uint32_t kernel_used;     /* PT_KERNEL_MEGA or PT_KERNEL_WAVEFRONT     */
    uint32_t error_word;      /* device error word (0 = none)              */
    /* With PT_RENDER_TIME_STAGES (wavefront): device time of the raygen,
     * extend (closest hit), shade (hit shading and the escaped rays' miss
     * shading), shadow (any hit), queue-reset and accumulate launches, in ms,
     * summed over the call; `stage_launches` counts the extend launches.
     * Zero otherwise. */
    float stage_ms[6];
    uint32_t stage_launches;
} pt_render_stats;

/* Accelerating-structure summary. */
typedef struct pt_accel_info {
    uint32_t blas_count;
    uint32_t tlas_nodes;
    uint64_t blas_nodes;
    uint64_t triangles;
    uint64_t device_bytes;
    float build_ms;
} pt_accel_info;

typedef struct pt_ctx pt_ctx;

/* Library ABI version (PT_ABI_VERSION of the build). */
int pt_abi_version(void);

/* Create a context on CUDA device `device`.  Replaces the Vulkan context and
 * device set-up of PathTraceDispatcher's constructor (ptdispatch.cpp:18-35). */
pt_ctx* pt_create(int device);

/* Destroy a context and free its device memory (~PathTraceDispatcher,
 * ptdispatch.cpp:37-40). */
void pt_destroy(pt_ctx* ctx);

/* Message for the last failing call on this context (or of pt_create when ctx
 * is NULL).  Valid until the next call on the context. */
const char* pt_last_error(const pt_ctx* ctx);

/* Upload a packed scene (SceneBuffer::build, scenebuffer.cpp:65-168).  The
 * view is copied; the caller may free its arrays after the call returns. */
int pt_upload_scene(pt_ctx* ctx, const pt_scene_view* scene);

/* Build the two-level acceleration structure on the device: one BLAS per mesh
 * and one TLAS over all instances (AccelerationStructure ctor,
 * accstruct.cpp:288-319, create_blas :69-164, create_tlas :186-286). */
int pt_build_accel(pt_ctx* ctx, pt_accel_info* info_out /* may be NULL */);

/* Render params->samples samples per pixel starting at params->sample_index.
 * Replaces PathTraceDispatcher::render (ptdispatch.cpp:97-134) with
 * PathTracer::set_camera/set_samples/set_max_bounces/update_uniforms
 * (pathtrace.cpp:381-516).  Asynchronous unless stats_out is non-NULL. */
int pt_render(pt_ctx* ctx, const pt_render_params* params, pt_render_stats* stats_out);

/* Progressive rendering without a window (the reference's interactive loop,
 * headless): pt_set_camera keeps params (camera, image size, bounces, mode,
 * kernel) in the context and restarts accumulation at sample 0, as
 * PathTracer::set_camera resets sample_index (pathtrace.cpp:381-396);
 * pt_render_next then adds `samples` samples to the running mean and advances
 * the sample index (PathTracer::update_uniforms, pathtrace.cpp:511-516;
 * PathTraceDispatcher::render's per-frame submission, ptdispatch.cpp:97-134).
 * params->sample_index and params->samples are ignored by pt_set_camera. */
int pt_set_camera(pt_ctx* ctx, const pt_render_params* params);
int pt_render_next(pt_ctx* ctx, uint32_t samples, pt_render_stats* stats_out);

/* Copy the accumulated image to host memory as RGBA rows of `pitch_bytes`
 * bytes (float when fp64 == 0, double when fp64 == 1).  Replaces the copy
 * into the host-visible image and vkMapMemory of ptdispatch.cpp:77-94.
 * fp64 == PT_IMAGE_SUMS64 copies the raw FP64 sums instead (rgb radiance
 * sums and the sample count per pixel, 4 doubles): the form in which
 * replicas rendering disjoint sample ranges on several GPUs are merged (an
 * element-wise sum). */
#define PT_IMAGE_SUMS64 3
int pt_read_image(pt_ctx* ctx, void* rgba, size_t pitch_bytes, int fp64);

/* Checkpoint / resume of long progressive renders (no reference
 * counterpart: the reference keeps its running mean only in device memory).
 * A checkpoint is pt_read_image (the FP32 running mean, and PT_IMAGE_SUMS64
 * for renders with FP64 sums) after `samples_done` samples; pt_restore_image
 * puts both back into a context (same or new), after which pt_render with
 * sample_index = samples_done continues the image exactly as if it had
 * never stopped (the per-sample values depend only on pixel and sample
 * index).  sums64 may be NULL for FP32-only renders; pitch is the rgba rows'
 * byte stride; sums64 rows are packed (4 doubles per pixel). */
int pt_restore_image(pt_ctx* ctx, const float* rgba, size_t pitch_bytes, const double* sums64, uint32_t width,
                     uint32_t height, uint32_t samples_done);

/* Wait for all work of the context. */
int pt_synchronize(pt_ctx* ctx);

/* ACES tone map of the accumulation image in place, as the reference does
 * before writing PNG (tonemap.cs.hlsl:17-77, ptdispatch.cpp:175-179). */
int pt_tonemap(pt_ctx* ctx);

/* Mean squared error between the FP32 image of `ctx` and a reference RGBA
 * image in device-visible host memory, with util/meansq semantics
 * (meansq.cpp:34-43): SSE over RGB / (w*h*3 - 1), reduced in FP64. */
int pt_mse_host(pt_ctx* ctx, const float* reference_rgba, double* mse_out);

/* Mean squared error for callers that cannot allocate device memory: host
 * applications that reserve the GPU's memory for their own pool and forbid
 * allocations inside plug-ins, processes under a hard device-memory cap, and
 * real-time loops that cannot risk the implicit device synchronisation of
 * cudaMalloc/cudaFree.  This entry point has no counterpart in the reference.
 *
 * Same value as pt_mse_host (util/meansq semantics) for two caller-owned
 * device images (RGBA float rows, 16-byte aligned, width * height pixels);
 * the result is written to the caller-owned device double *mse_out,
 * asynchronously on `stream` (a cudaStream_t, NULL = default stream).  It
 * allocates nothing: its scratch is a fixed device array of
 * PT_MSE_NOALLOC_SCRATCH_BYTES bytes inside the library, present on every GPU
 * that loads it until the process exits.  The first call on a device (with
 * that device current) looks up the array's address; make that first call
 * before any stream capture.  All calls share the array: calls that overlap on
 * the GPU race.  Images above PT_MSE_NOALLOC_MAX_PIXELS pixels are rejected
 * with PT_ERR_UNSUPPORTED; null pointers, images not 16-byte aligned and an
 * output not 8-byte aligned with PT_ERR_INVALID. */
#define PT_MSE_NOALLOC_SCRATCH_BYTES 9728u
#define PT_MSE_NOALLOC_MAX_PIXELS 2147483648ull
int pt_mse_noalloc(const float* image_rgba, const float* reference_rgba, uint32_t width, uint32_t height, double* mse_out,
                   void* stream);

/* ---- Batched rendering ----------------------------------------------------
 * Many render jobs, each with its own scene, camera, image size, sample count
 * and bounce limit, rendered by one call.  The jobs' paths share the waves of
 * one wavefront launch sequence (a wave holds consecutive samples of several
 * jobs, so small jobs fill the GPU together), the sequence is captured into a
 * CUDA graph and launched as one unit, and small jobs may instead run as
 * megakernel launches on a parallel branch of the same graph.  Jobs with less
 * work go into the first waves, so small jobs finish early.  An autotuner
 * times short trial batches (every job at 1/32 of its samples, at least one)
 * and picks the wave capacity (2^21, 2^23, 2^25 or 2^26 paths in flight, within a
 * quarter of the free device memory), the megakernel tile and the
 * work size below which a job runs on the megakernel; its choice is cached
 * per batch.  Every job's image equals, bit for bit, rendering that job alone
 * with pt_render.  The reference renders one scene per process and has no
 * counterpart; the call exists to keep the GPU full with many small jobs. */
typedef struct pt_batch_job {
    const pt_ctx* scene;     /* context holding the job's scene (uploaded, acceleration structure built);
                                same device; may be the batch context itself */
    pt_render_params params; /* sample_index 0, flags 0; kernel PT_KERNEL_AUTO lets the tuner decide,
                                PT_KERNEL_MEGA / PT_KERNEL_WAVEFRONT force one */
} pt_batch_job;

#define PT_BATCH_NO_TUNE 1u  /* skip the tuner: every AUTO job on the wavefront, 2^23 paths per wave */
#define PT_BATCH_NO_GRAPH 2u /* issue the launch sequence directly instead of through a CUDA graph */
#define PT_BATCH_RETUNE 4u   /* ignore the tuning cache */
/* Fixes the wave capacity at 2^n paths (10 <= n <= 25) instead of tuning it. */
#define PT_BATCH_CAPACITY_LOG2(n) ((uint32_t)(n) << 8)

typedef struct pt_batch_stats {
    uint64_t segments, shadow_rays, paths; /* over all jobs */
    float milliseconds;       /* device time of the batch render (CUDA events around the graph launch) */
    float tune_milliseconds;  /* host time of the tuner's trial batches (0 on a cache hit or NO_TUNE) */
    float build_milliseconds; /* host time of planning, graph capture and instantiation (0 when reused) */
    uint32_t waves;           /* wavefront waves */
    uint32_t kernel_launches; /* kernels in the launch sequence */
    uint32_t mega_jobs;       /* jobs rendered by the megakernel */
    uint32_t wave_capacity;   /* paths per wave */
    uint32_t tile_w;          /* megakernel tile: tile_w x (128 / tile_w) pixels */
    uint32_t graph_reused;    /* 1: the graph of an identical earlier batch was launched again */
    uint64_t mega_threshold;  /* AUTO jobs whose trial work, pixels x max(1, samples / 32) x (bounces + 1),
                                 is below this ran on the megakernel */
    uint32_t error_word;      /* device error word (0 = none) */
    uint32_t reserved;
} pt_batch_stats;

/* Render `count` jobs; synchronous (returns when every image is final). */
int pt_render_batch(pt_ctx* ctx, const pt_batch_job* jobs, uint32_t count, uint32_t flags, pt_batch_stats* stats_out);
/* Copy job `job`'s image of the last pt_render_batch to host memory, as
 * pt_read_image does (fp64 = 1 needs PT_ACCUM_FP32_FP64 for that job). */
int pt_read_batch_image(pt_ctx* ctx, uint32_t job, void* rgba, size_t pitch_bytes, int fp64);
/* Per-job latency of the last pt_render_batch: ms[j] = device time from the
 * batch's start until job j's image was final (the wave holding its last
 * samples, or its last megakernel launch, completed).  Waves take the jobs
 * with the least work (pixels x samples) first.  `count` must be the last
 * batch's job count. */
int pt_batch_job_times(pt_ctx* ctx, float* ms, uint32_t count);

#ifdef __cplusplus
}
#endif

#endif /* PT_GPU_H_INCLUDED */
