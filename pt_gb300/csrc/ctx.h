// ctx.h — the context behind the C ABI (pt_ctx of include/pt_gpu.h): device
// buffers of one scene and its acceleration structure, the accumulation image,
// wavefront path state, denoiser buffers and the batch renderer's state.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "../../include/pt_gpu.h"
#include "device/render.cuh"
#include "kernels.h"

namespace pt {
struct BatchState; // batch.cu
void batch_free(BatchState* b);
} // namespace pt

using pt::Bvh4Node;
using pt::BvhNode;
using pt::DevInstance;
using pt::DevInstanceData;
using pt::DevMaterial;
using pt::DevTexture;
using pt::REF_EMPTY;
using pt::TriRec;

// One device allocation; released explicitly or by the owning context.
template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    cudaError_t alloc(size_t count)
    {
        release();
        if (count == 0)
            count = 1;
        cudaError_t e = cudaMalloc((void**)&p, count * sizeof(T));
        if (e != cudaSuccess) {
            p = nullptr;
            return e;
        }
        n = count;
        return cudaSuccess;
    }
    void release()
    {
        if (p)
            cudaFree(p);
        p = nullptr;
        n = 0;
    }
};

struct pt_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    bool tables = false;
    // scene
    bool scene_ok = false;
    DevBuf<float4> vertices;
    DevBuf<uint32_t> indices;
    DevBuf<DevInstanceData> inst_data;
    DevBuf<DevMaterial> materials;
    DevBuf<float> material_ior; // refractive extension; meaningful only when has_ior
    bool has_ior = false;
    DevBuf<uint8_t> texels;
    DevBuf<DevTexture> textures;
    uint32_t texture_count = 0;
    DevBuf<uint32_t> light;
    DevBuf<uint32_t> mesh_vertex_offset, mesh_index_offset, mesh_tri_base, inst_mesh;
    DevBuf<DevInstance> dinst;
    uint32_t vertex_count = 0, index_count = 0, mesh_count = 0, tri_count = 0, instance_count = 0, material_count = 0;
    uint32_t light_words = 0, light_count = 0;
    float env[3] = {0, 0, 0};
    std::vector<DevInstance> h_dinst;
    // acceleration structure
    bool accel_ok = false;
    DevBuf<BvhNode> nodes;
    DevBuf<Bvh4Node> nodes4; // empty when the BVH2 is traversed (PT_BVH_WIDTH=2)
    DevBuf<TriRec> tris;
    DevBuf<int> mesh_root;
    int tlas_root = REF_EMPTY;
    pt_accel_info accel{};
    // image
    DevBuf<float4> image;
    DevBuf<double> sum64;
    uint32_t width = 0, height = 0;
    uint32_t samples_done = 0;
    bool have_fp64 = false;
    DevBuf<unsigned long long> counters;
    DevBuf<uint32_t> error_word;
    DevBuf<char> wave_state;    // wavefront path state
    // further sub-waves in flight (index 0 unused: wave_state and stream);
    // streams and events are created on first use
    DevBuf<char> wave_state_x[pt::MAX_WAVE_WAYS];
    uint32_t wave_paths_x[pt::MAX_WAVE_WAYS] = {};
    cudaStream_t side[pt::MAX_WAVE_WAYS] = {};
    cudaEvent_t wave_fork = nullptr, wave_join[pt::MAX_WAVE_WAYS] = {}, wave_acc[pt::MAX_WAVE_WAYS] = {};
    uint32_t wave_paths = 0;    // paths the wave state holds
    int sm_count = 0;
    pt_render_params camera{};  // pt_set_camera state
    bool camera_set = false;
    uint32_t next_sample = 0;
    DevBuf<float4> feat_a, feat_n; // denoiser features: albedo + depth, normal
    uint32_t feat_w = 0, feat_h = 0;
    bool feat_fp16 = false, half_fp16 = false; // storage of feat_a/feat_n and of the snapshot
    DevBuf<float4> denoised;    // last pt_denoise result
    DevBuf<float4> half;        // pt_denoise_snapshot: mean image of the first samples
    uint32_t half_w = 0, half_h = 0, half_spp = 0, half_epoch = 0;
    uint32_t snapshot_armed = 0; // pt_denoise_snapshot_at: take it at this many samples (0 = off)
    uint32_t image_epoch = 0;   // counts fresh renders (sample_index 0)
    DevBuf<float4> mse_ref;     // reference image for pt_mse_host
    DevBuf<double> mse_partial; // [0] result, [1..] per-block partial sums
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::vector<cudaEvent_t> stage_events; // PT_RENDER_TIME_STAGES event pool
    std::vector<uint8_t> stage_of;
    uint64_t scene_generation = 0;   // bumped by every scene upload and acceleration build
    pt::BatchState* batch = nullptr; // pt_render_batch state (images, job tables, graph, tuning cache)

    int fail(int code, const std::string& msg)
    {
        err = msg;
        return code;
    }
    int cuda_fail(cudaError_t e, const char* what)
    {
        err = std::string(what) + ": " + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? PT_ERR_OOM : PT_ERR_CUDA;
    }
};

// Device view of the context's scene and the camera/image of `p` (api.cu).
pt::RenderArgs render_args(const pt_ctx* c, const pt_render_params* p, bool fp64);
