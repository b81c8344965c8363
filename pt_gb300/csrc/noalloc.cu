// noalloc.cu — pt_mse_noalloc: the meansq reduction without any allocation.
//
// Some callers of this library cannot allocate device memory: host
// applications (renderers, game engines, simulation frameworks) that reserve
// the GPU's memory for their own pool up front and forbid allocations inside
// plug-ins, processes started under a hard device-memory cap, and real-time
// loops that cannot afford the implicit device synchronisation that
// cudaMalloc/cudaFree may cause.  This entry point computes the same value as
// pt_mse_host from caller-owned device buffers, with its only scratch (the
// per-block partial sums) in a fixed file-scope device array.
//
// The array lives in every GPU that loads the library until the process
// exits.  Its device address is looked up once per device, by the first call
// on that device (made with that device current); make that first call before
// any stream capture.  Every call shares the one array: calls that overlap on
// the GPU (different streams, or different host threads, without ordering
// between them) race on it.  Each block overwrites its own partial sum before
// the final pass reads it, so no clearing is needed between calls.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/pt_gpu.h"
#include "kernels.h"

namespace {

// One result slot is not needed (the caller passes the output); the array
// holds one partial sum per block of the reduction grid.
constexpr uint32_t NOALLOC_PARTIALS = pt::MSE_MAX_BLOCKS;
static_assert(NOALLOC_PARTIALS * sizeof(double) == PT_MSE_NOALLOC_SCRATCH_BYTES, "scratch size in pt_gpu.h");

static __device__ __align__(256) double g_mse_scratch[NOALLOC_PARTIALS];

constexpr int MAX_DEVICES = 64;
std::mutex g_lock;
double* g_scratch_ptr[MAX_DEVICES] = {};

} // namespace

extern "C" {

int pt_mse_noalloc(const float* image, const float* reference, uint32_t width, uint32_t height, double* mse_out, void* stream)
{
    if (!image || !reference || !mse_out) {
        return PT_ERR_INVALID;
    }
    if (width == 0 || height == 0) {
        return PT_ERR_INVALID;
    }
    if ((uint64_t)width * height > PT_MSE_NOALLOC_MAX_PIXELS) {
        return PT_ERR_UNSUPPORTED;
    }
    if ((((uintptr_t)image | (uintptr_t)reference) & 15u) || ((uintptr_t)mse_out & 7u)) {
        return PT_ERR_INVALID;
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) {
        return PT_ERR_CUDA;
    }
    double* scratch;
    {
        std::lock_guard<std::mutex> lock(g_lock);
        if (!g_scratch_ptr[dev]) {
            void* p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_mse_scratch);
            if (e != cudaSuccess || !p) {
                return PT_ERR_CUDA;
            }
            g_scratch_ptr[dev] = (double*)p;
        }
        scratch = g_scratch_ptr[dev];
    }
    cudaError_t e = pt::launch_mse((const float4*)image, (const float4*)reference, width, height, scratch, mse_out,
                                   (cudaStream_t)stream);
    if (e != cudaSuccess) {
        return PT_ERR_CUDA;
    }
    return PT_OK;
}

} // extern "C"
