// nn.h — host-side interface of the denoiser's device kernels.
//
// Activations are NHWC bf16 buffers whose pixel pitch (channels per pixel)
// is a multiple of 16; a layer may read or write a channel range [c0, c0 + C)
// of a wider buffer, which is how the U-Net's skip concatenations are built
// without copies.  Weights are kept in FP32 as [tap][c_in][c_out] (tap =
// 3*ky + kx) and packed to BF16 tensor-core layouts before use.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>

namespace pt {
namespace nn {

struct Act {
    uint16_t* p = nullptr; // bf16 bits
    int n = 0, h = 0, w = 0, pitch = 0;
    __host__ __device__ size_t pixels() const { return (size_t)n * h * w; }
};

// Tensor map over an activation buffer with a box of 8 channels x tx x ty
// pixels of one image.  False (and a message in *why) on failure.
bool encode_act_map(CUtensorMap* map, const Act& a, int tx, int ty, const char** why);

// Tile shapes: conv tiles hold 128 pixels, weight-gradient chunks 64.
void conv_tile_shape(int w, int& tx, int& ty);
void wgrad_chunk_shape(int w, int& tx, int& ty);

// Packed weight sizes (elements) of one layer.
inline size_t packed_elems(int cin, int cout) { return (size_t)9 * cin * cout; }

// out = act(conv3x3(in[c0 : c0 + cin]) + bias) written to out[out_c0 : +nout]
// (bf16) or, when out_f32 is set, to out_f32 with pitch out.pitch.  With
// `mask` the result is multiplied by (mask[mask_c0 + c] > 0).  `wpk` holds the
// weights packed by pack_weights (forward layout for a forward pass, the
// data-gradient layout for a backward pass; nout is then the layer's c_in).
// `in_map` must cover `in` with the conv tile box.  With out_f32, `residual`
// (fp32, 4 per pixel, may be null) is added to output channels 0-3.
struct ConvCall {
    const CUtensorMap* in_map;
    Act in;
    int c0, cin;
    const uint16_t* wpk;
    int nout;
    const float* bias;
    bool relu;
    Act out;
    int out_c0;
    float* out_f32;
    const Act* mask;
    int mask_c0;
    const float* residual; // fp32 [pixel][4] added to output channels 0-3 (with out_f32 only)
};
cudaError_t conv3x3(const ConvCall& c, uint32_t* error, cudaStream_t st);

// The same convolution with halo reuse (conv_rows.cu): persistent CTAs over
// tiles of rows_per_tile(nout) rows x 128 pixels; `halo_map` must cover `in`
// with a box of 8 channels x 130 x (rows_per_tile + 2) pixels
// (encode_act_map(map, in, 130, rows + 2)), `c.wpk` the weights packed by
// pack_weights_rows.
int rows_per_tile(int nout);
cudaError_t pack_weights_rows(const float* w, int cin, int cout, uint16_t* fwd, uint16_t* bwd, cudaStream_t st);
cudaError_t conv3x3_rows(const ConvCall& c, const CUtensorMap* halo_map, int sm_count, uint32_t* error, cudaStream_t st);
// True unless PT_CONV_KERNEL=tap selects the one-tile-per-CTA kernel.
bool use_rows_kernel();

// dw[tap][ci][co] += sum_p x[p + offset(tap)][x_c0 + ci] * g[p][g_c0 + co]
// over all pixels (dw must be zeroed by the caller).  Maps use the wgrad box.
struct WgradCall {
    const CUtensorMap* x_map;
    int x_c0, cin;
    const CUtensorMap* g_map;
    int g_c0, cout;
    int n, h, w;
    float* dw;
};
cudaError_t conv3x3_wgrad(const WgradCall& c, int sm_count, uint32_t* error, cudaStream_t st);

// Element-wise and reduction kernels (ops.cu).
cudaError_t pool2(const Act& in, int in_c0, int c, const Act& out, int out_c0, cudaStream_t st);
cudaError_t upsample2(const Act& in, int in_c0, int c, const Act& out, int out_c0, cudaStream_t st);
// g_low[c] = (sum of the 2x2 block of g_high[gc0 + c]) * (z[zc0 + c] > 0)
cudaError_t upsample2_backward(const Act& g_high, int g_c0, int c, const Act& z, int z_c0, const Act& g_low, cudaStream_t st);
// g[c] = (g_skip[s_c0 + c] + g_pool[c] / 4 at (y/2, x/2)) * (z[z_c0 + c] > 0)
cudaError_t pool2_backward(const Act& g_skip, int s_c0, const Act& g_pool, int c, const Act& z, int z_c0, const Act& g,
                           cudaStream_t st);
// db[c] += sum over pixels of g[c0 + c]
cudaError_t bias_grad(const Act& g, int c0, int c, float* db, cudaStream_t st);
// Packs fp32 [9][cin][cout] weights to the forward layout [9][cin/8][cout][8]
// and the data-gradient layout [9][cout/8][cin][8] (taps mirrored).
cudaError_t pack_weights(const float* w, int cin, int cout, uint16_t* fwd, uint16_t* bwd, cudaStream_t st);
cudaError_t adam_step(float* p, const float* g, float* m, float* v, size_t n, float lr, float beta1, float beta2, float eps,
                      float bc1, float bc2, cudaStream_t st);

} // namespace nn
} // namespace pt
