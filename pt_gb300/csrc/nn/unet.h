// unet.h — the denoiser network: a 4-level U-Net of 3x3 convolutions
// (channels 32 / 64 / 96 / 128, two convolutions per level, 2x2 average
// pooling down, nearest upsampling up, skip connections by concatenation)
// mapping 16 input feature channels to 16 output channels of which the first
// three are log(1 + radiance).  The output layer adds an FP32 residual base
// (the caller's log(1 + noisy radiance)) so that pixels the network leaves
// alone keep full precision.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "nn.h"

namespace pt {
namespace nn {

struct LayerSpec {
    int cin, cout;
    bool relu;
};

constexpr int N_LAYERS = 15;
constexpr int IN_CHANNELS = 16;
constexpr int OUT_CHANNELS = 16;
extern const LayerSpec LAYERS[N_LAYERS];

// Parameters of all layers in order; layer l holds w[9][cin][cout] then b[cout].
size_t param_count();
size_t weight_offset(int layer);
size_t bias_offset(int layer);

// Loss on the first three output channels (log radiance) against a linear
// RGB target t: mean over pixels and channels of (1 + min(t, 16))^2 *
// (out - log(1 + t))^2.  The weight makes the loss track the squared error of
// expm1(out) in linear radiance.
constexpr float LOSS_CLAMP = 16.0f;

class UNet {
  public:
    ~UNet();
    // Fixed batch and image size (multiples of 8); allocates every buffer.
    bool init(int device, int n, int h, int w, std::string& err);
    int n() const { return n_; }
    int h() const { return h_; }
    int w() const { return w_; }

    bool set_params(const float* host, size_t count, std::string& err);
    bool get_params(float* host, size_t count, std::string& err);
    bool get_grads(float* host, size_t count, std::string& err);
    // Adam moments (fp32, parameter order) and the number of steps taken.
    bool get_adam_state(float* m, float* v, size_t count, uint32_t* step, std::string& err);
    bool set_adam_state(const float* m, const float* v, size_t count, uint32_t step, std::string& err);

    // Input: bf16 [n][h][w][16] (device).  Output fp32 [n][h][w][16] in output().
    uint16_t* input() { return x0_.a.p; }
    // fp32 [n][h][w][4] added to output channels 0-3 (zero unless set).
    float* base() { return base32_; }
    const float* output() const { return out32_; }
    cudaError_t forward(cudaStream_t st);
    // Gradients of the loss against `target` (fp32 linear RGBA [n][h][w][4],
    // device) after forward(); *loss (host) receives the loss when non-null.
    cudaError_t backward(const float* target, double* loss, cudaStream_t st);
    cudaError_t adam(float lr, cudaStream_t st);
    uint32_t device_error();
    int launches_per_forward() const { return 2 * N_LAYERS + 6; }

    struct Buf {
        Act a;
        CUtensorMap tile, chunk;
        CUtensorMap halo[4]; // halo boxes for 1, 2, 4 and 8 rows per tile
    };

  private:
    bool make(Buf& b, int level, int channels, std::string& err);
    cudaError_t conv(int layer, Buf& in, int c0, Buf& out, int out_c0, cudaStream_t st);
    cudaError_t run_conv(ConvCall& c, Buf& in, const uint16_t* rows_wpk, cudaStream_t st);
    cudaError_t dgrad(int layer, Buf& g, Buf& out, const Buf* mask, int mask_c0, cudaStream_t st);
    cudaError_t wgrad(int layer, Buf& x, int x_c0, Buf& g, cudaStream_t st);
    cudaError_t repack(cudaStream_t st);

    int device_ = 0, n_ = 0, h_ = 0, w_ = 0, sm_count_ = 0;
    std::vector<void*> allocs_;
    void* alloc(size_t bytes);
    // activations
    Buf x0_, e0a_, cat0_, p1_, e1a_, cat1_, p2_, e2a_, cat2_, p3_, b3a_, b3b_, d2a_, d2b_, d1a_, d1b_, d0a_, d0b_;
    float* out32_ = nullptr;
    float* base32_ = nullptr;
    // gradients
    Buf g_out_, g_d0b_, g_d0a_, g_cat0_, g_d1b_, g_d1a_, g_cat1_, g_d2b_, g_d2a_, g_cat2_, g_b3b_, g_b3a_, g_p3_, g_e2b_, g_e2a_,
        g_p2_, g_e1b_, g_e1a_, g_p1_, g_e0b_, g_e0a_;
    // parameters
    float *params_ = nullptr, *grads_ = nullptr, *adam_m_ = nullptr, *adam_v_ = nullptr;
    uint16_t *wfwd_ = nullptr, *wbwd_ = nullptr;   // per-tap kernel layouts
    uint16_t *wrfwd_ = nullptr, *wrbwd_ = nullptr; // halo kernel layouts
    bool rows_ = true;
    size_t packed_off_[N_LAYERS] = {};
    bool packed_ok_ = false;
    int adam_t_ = 0;
    double* loss_acc_ = nullptr;
    uint32_t* error_ = nullptr;
};

// Loss and output-gradient kernel (unet.cu).
cudaError_t loss_backward(const float* out32, const float* target, size_t pixels, uint16_t* g_out, double* loss_acc,
                          cudaStream_t st);

} // namespace nn
} // namespace pt
