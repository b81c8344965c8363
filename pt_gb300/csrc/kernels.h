// kernels.h — host-side declarations of the device kernels' launchers.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace pt {

struct RenderArgs;
struct BvhNode;
struct Bvh4Node;
struct TriRec;
struct DevInstance;
struct DevInstanceData;

cudaError_t launch_megakernel(const RenderArgs& a, cudaStream_t stream);
// The megakernel with a tile of tile_w x (128 / tile_w) pixels per block
// (tile_w 8, 16 or 32).
cudaError_t launch_megakernel_tiled(const RenderArgs& a, uint32_t tile_w, cudaStream_t stream);

// Per-stage device time of the wavefront: an event is recorded before every
// launch and after the last one; the interval after event i belongs to
// stage[i].  Stages: 0 raygen, 1 extend, 2 shade, 3 shadow, 4 reset,
// 5 accumulate, 6 end marker.
struct StageTimer {
    cudaEvent_t* events = nullptr;
    uint8_t* stage = nullptr;
    uint32_t capacity = 0;
    uint32_t count = 0;
    void mark(cudaStream_t st, uint8_t s)
    {
        if (count < capacity) {
            cudaEventRecord(events[count], st);
            stage[count] = s;
            count++;
        }
    }
};
constexpr int STAGE_COUNT = 6;

// Wavefront path tracer (render_wave.cu).  `state` holds wave_state_bytes(n)
// bytes of path state for up to n_paths_max paths (a multiple of the pixel
// count); r.samples samples are rendered in waves of n_paths_max / pixels.
size_t wave_state_bytes(uint32_t n_paths_max);
// Several sub-waves in flight: `ways` path states of the same size, each
// with its own stream (state[0] / stream[0] are the launch's own).  Waves go
// round-robin over them, so the ragged end of one wave's launches overlaps
// the others' work; the accumulation kernels run in wave order (events
// acc[]), which keeps the running mean, FP64 sums, feature means and
// snapshot exactly those of one stream.  fork / join[] tie the extra streams
// to the launch's stream before and after.
constexpr int MAX_WAVE_WAYS = 4;
struct WaveMulti {
    int ways;
    void* state[MAX_WAVE_WAYS];
    size_t state_bytes[MAX_WAVE_WAYS];
    cudaStream_t stream[MAX_WAVE_WAYS];
    cudaEvent_t fork, join[MAX_WAVE_WAYS], acc[MAX_WAVE_WAYS];
};
cudaError_t launch_wavefront(const RenderArgs& r, void* state, size_t state_bytes, uint32_t n_paths_max, int sm_count,
                             uint32_t* launches, cudaStream_t stream, StageTimer* timer = nullptr,
                             const WaveMulti* multi = nullptr);
cudaError_t wave_init_tables(const uint32_t* table128, const float* srgb256, cudaStream_t stream);

// Batched wavefront: waves hold shares of several jobs (RenderArgs in device
// memory, one per job).  A share is `samples` consecutive samples from
// `first_sample` of all `pixels` pixels of job `job`: path ids [path_base,
// path_base + samples * pixels) in sample-major order and accumulation
// threads [pixel_base, pixel_base + pixels).  Shares of a wave are sorted by
// path_base and pixel_base.
struct WaveShare {
    uint32_t job, path_base, pixel_base, first_sample, samples, pixels;
};
struct BatchWave {
    uint32_t share_offset, share_count; // into the device share array
    uint32_t n_paths, n_pixels;         // totals of the wave's shares
    uint32_t max_bounces;               // largest of the wave's jobs
};
// `path_share` holds n_paths_max u32; `waves` is host memory (the launch
// sequence is fixed by it, so the whole call can be captured in a graph).
// w4: every job's scene has 4-wide nodes (the 4-wide traversal kernels run).
// multi (optional, ways <= 2 used): a second path state with its own
// path_share2 array and stream; waves alternate over the two as in
// launch_wavefront, accumulation in wave order.
// Occupancy queries of the batched kernels; call before capturing a batch.
cudaError_t wave_batch_prepare();
cudaError_t launch_wavefront_batch(const RenderArgs* jobs, const WaveShare* shares, const BatchWave* waves, uint32_t wave_count,
                                   uint32_t* path_share, unsigned long long* counters, void* state, size_t state_bytes,
                                   uint32_t n_paths_max, bool w4, int sm_count, uint32_t* launches, cudaStream_t stream,
                                   const WaveMulti* multi = nullptr, uint32_t* path_share2 = nullptr,
                                   cudaEvent_t* wave_done = nullptr);
// Records `ev` on `st` so that its time can be read later: inside a stream
// capture as an external event (an event-record node of the graph; a plain
// record there only orders streams), otherwise as a plain record (the
// external flag is refused outside a capture).
inline cudaError_t record_timed(cudaEvent_t ev, cudaStream_t st)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaError_t e = cudaStreamIsCapturing(st, &cs);
    if (e != cudaSuccess)
        return e;
    return cs == cudaStreamCaptureStatusActive ? cudaEventRecordWithFlags(ev, st, cudaEventRecordExternal)
                                               : cudaEventRecord(ev, st);
}

cudaError_t features_init_tables(const uint32_t* table128, const float* srgb256, cudaStream_t stream);

// Denoiser features and packing (features.cu).
cudaError_t launch_features(const RenderArgs& a, float4* feat_a, float4* feat_n, cudaStream_t stream);
// fa/fn (and half) hold 4 x FP16 per pixel when feat_fp16 (half_fp16) is set.
cudaError_t launch_denoise_input(const float4* img, const float4* half, const float4* fa, const float4* fn, uint32_t pixels,
                                 float spp_feature, uint16_t* out, float* base, uint32_t feat_fp16, uint32_t half_fp16,
                                 cudaStream_t stream);
cudaError_t launch_denoise_output(const float* out32, uint32_t pixels, float4* img, cudaStream_t stream);

// Output stage (post.cu).
constexpr uint32_t MSE_MAX_BLOCKS = 152 * 8; // partial sums: one per block
cudaError_t launch_tonemap(float4* img, uint32_t n, cudaStream_t stream);
uint32_t mse_blocks(uint32_t pixels);
// meansq of RGB: writes SSE / (w*h*3 - 1) to *out (device); `partial` holds
// mse_blocks(w*h) doubles of scratch.
cudaError_t launch_mse(const float4* img, const float4* ref, uint32_t width, uint32_t height, double* partial, double* out,
                       cudaStream_t stream);

// Two-level LBVH build on the device (Karras 2012 radix tree per segment).
struct BvhBuildInput {
    // BLAS: all meshes at once, one key segment per mesh.
    const float4* vertices;     // 2 float4 per vertex
    const uint32_t* indices;    // mesh-local
    const uint32_t* mesh_vertex_offset;
    const uint32_t* mesh_index_offset;
    const uint32_t* mesh_tri_base; // prefix sum of tri counts (mesh_count + 1 entries)
    uint32_t mesh_count;
    uint32_t tri_count;
    // TLAS
    const DevInstanceData* inst_data;
    const uint32_t* inst_mesh;
    uint32_t instance_count;
};

struct BvhBuildOutput {
    BvhNode* nodes;      // (tri_count - 1) BLAS nodes followed by TLAS nodes
    TriRec* tris;        // tri_count records in leaf order
    DevInstance* dinst;  // blas_root and the world box are filled in
    int* mesh_root;      // mesh_count
    int tlas_root;       // host value after the build
};

// 4-wide nodes derived from the n BVH2 nodes (same indices), and whether the
// tracer uses them (PT_BVH_WIDTH=2 keeps the BVH2 traversal).
cudaError_t build_bvh4(const BvhNode* nodes, uint32_t n, Bvh4Node* out, uint32_t* overflow, cudaStream_t stream);
bool use_bvh4();

// Scratch sizing for bvh_build (bytes).
size_t bvh_scratch_bytes(uint32_t mesh_count, uint32_t tri_count, uint32_t instance_count);
size_t bvh_node_count(uint32_t tri_count, uint32_t instance_count);

// Builds everything on `stream`; `scratch` must hold bvh_scratch_bytes().
// dinst must already hold the world-to-object rows and flags.
cudaError_t bvh_build(const BvhBuildInput& in, BvhBuildOutput& out, void* scratch, size_t scratch_bytes, cudaStream_t stream);

} // namespace pt
