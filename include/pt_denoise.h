/* pt_denoise.h — learned denoiser of libptgpu.
 *
 * The reference renders plain progressive Monte-Carlo images and has no
 * denoiser: nothing here replaces a reference interface.  These entry points
 * add a small convolutional U-Net that maps a low-sample image plus first-hit
 * features to an estimate of the converged image, trained on the GPU by the
 * library's own BF16 tensor-core kernels (FP32 accumulation).
 *
 * Conventions: device pointers are plain CUDA device addresses of the
 * library's device; activations are NHWC with bf16 elements (uint16_t bit
 * patterns); `stream` is a cudaStream_t or NULL for the legacy stream.  All
 * functions return PT_OK (0) or a negative pt_status from pt_gpu.h.
 */
#ifndef PT_DENOISE_H
#define PT_DENOISE_H

#include <stddef.h>
#include <stdint.h>

#include "pt_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Network input: 16 bf16 channels per pixel.
 *   0-2   log(1 + radiance) of the noisy mean image
 *   3-5   first-hit base colour      6-8  first-hit world normal
 *   9     log(1 + hit distance) / 4  10   log2(samples per pixel) / 8
 *   11-13 noise estimate: sign(d) log(1 + |d|), d = snapshot mean - mean
 *         (see pt_denoise_snapshot), zero without a snapshot
 *   14    1 when a snapshot was used, else 0
 *   15    zero
 * Network output: 16 fp32 channels, 0-2 = log(1 + radiance), computed as the
 * residual base plus the network's correction. */
#define PT_UNET_IN_CHANNELS 16u
#define PT_UNET_OUT_CHANNELS 16u

typedef struct pt_unet pt_unet;

/* Number of fp32 parameters; layer l stores w[9][c_in][c_out] (tap = 3*ky+kx)
 * then b[c_out], layers in the order of pt_unet_layer_shape. */
size_t pt_unet_param_count(void);
/* Input/output channels of layer l (0..14); returns 0 for a bad index. */
int pt_unet_layer_shape(int layer, uint32_t* c_in, uint32_t* c_out);

/* A network for a fixed batch and image size (sides multiples of 8).  NULL on
 * failure; pt_unet_last_error(NULL) then says why. */
pt_unet* pt_unet_create(int device, uint32_t batch, uint32_t height, uint32_t width);
void pt_unet_destroy(pt_unet* u);
const char* pt_unet_last_error(const pt_unet* u);

int pt_unet_set_params(pt_unet* u, const float* host_params, size_t count);
int pt_unet_get_params(pt_unet* u, float* host_params, size_t count);
/* Gradients of the last pt_unet_backward (fp32, parameter order). */
int pt_unet_get_grads(pt_unet* u, float* host_grads, size_t count);

/* Batch, height and width the network was created for. */
void pt_unet_shape(const pt_unet* u, uint32_t* batch, uint32_t* height, uint32_t* width);
/* Device buffer the next forward pass reads: bf16 [batch][h][w][16]. */
uint16_t* pt_unet_input(pt_unet* u);
/* Device buffer holding the last forward pass's fp32 [batch][h][w][16]. */
const float* pt_unet_output(const pt_unet* u);
/* Residual base, fp32 [batch][h][w][4] (device, zero after creation): added to
 * output channels 0-3, so the network predicts a correction of
 * log(1 + noisy radiance) that pt_denoise_input writes here in full FP32. */
float* pt_unet_base(pt_unet* u);
/* Forward pass; writes fp32 [batch][h][w][16] to `output` (device, may be
 * NULL to keep it internal). */
int pt_unet_forward(pt_unet* u, float* output, void* stream);
/* Loss and gradients after a forward pass.  `target` = fp32 linear RGBA
 * [batch][h][w][4] (device).  Loss: mean over pixels and RGB of
 * (1 + min(t, 16))^2 * (out - log(1 + t))^2.  *loss (host) may be NULL. */
int pt_unet_backward(pt_unet* u, const float* target, double* loss, void* stream);
/* One Adam step (beta 0.9 / 0.999, eps 1e-8) with learning rate lr. */
int pt_unet_adam(pt_unet* u, float lr, void* stream);
/* Optimizer state for training checkpoints: the first and second Adam
 * moments (fp32, parameter order, `count` = pt_unet_param_count()) and the
 * number of Adam steps taken (bias correction).  pt_unet_set_params clears
 * the state, so a resume sets the parameters first and the state second. */
int pt_unet_get_adam_state(pt_unet* u, float* m, float* v, size_t count, uint32_t* step);
int pt_unet_set_adam_state(pt_unet* u, const float* m, const float* v, size_t count, uint32_t step);

/* Single layers, for tests.  `in` is bf16 [n][h][w][in_pitch] read at
 * channels [c0, c0 + c_in); `weights` fp32 [9][c_in][c_out] (device).
 * conv:  out[n][h][w][c_out] (bf16) = act(conv3x3(in) + bias), relu 0/1.
 * dgrad: grad_in[..][c_in] = conv3x3^T(grad_out[..][c_out]) * (mask > 0)
 *        (mask bf16 [..][c_in] or NULL).
 * wgrad: dw[9][c_in][c_out] (fp32) += correlation of in and grad_out. */
int pt_nn_conv3x3(const uint16_t* in, uint32_t n, uint32_t h, uint32_t w, uint32_t in_pitch, uint32_t c0, uint32_t c_in,
                  const float* weights, const float* bias, uint32_t c_out, int relu, uint16_t* out, void* stream);
int pt_nn_conv3x3_dgrad(const uint16_t* grad_out, uint32_t n, uint32_t h, uint32_t w, uint32_t c_out, const float* weights,
                        uint32_t c_in, const uint16_t* mask, uint16_t* grad_in, void* stream);
int pt_nn_conv3x3_wgrad(const uint16_t* in, uint32_t n, uint32_t h, uint32_t w, uint32_t in_pitch, uint32_t c0, uint32_t c_in,
                        const uint16_t* grad_out, uint32_t c_out, float* dw, void* stream);

/* Renderer side (pt_gpu.h context).
 * First-hit features for the current image size: for each pixel, the mean
 * over the camera rays of samples [sample_index, sample_index + samples) of
 * base colour, world shading normal (facing the camera) and hit distance
 * (zero where the ray escapes).  Kept in the context. */
int pt_render_features(pt_ctx* ctx, const pt_render_params* params);
/* Copies the feature image (width x height of the last features) to host:
 * albedo_depth gets base colour + hit distance, normal the shading normal,
 * 4 floats per pixel each (either may be NULL). */
int pt_read_features(pt_ctx* ctx, float* albedo_depth, float* normal);
/* Keeps a copy of the context's current mean image (the first samples of the
 * image being accumulated).  pt_denoise_input then derives a per-pixel noise
 * estimate from it, as long as the image was continued (not restarted)
 * since. */
int pt_denoise_snapshot(pt_ctx* ctx);
/* Arms the same snapshot for the moment the image holds `samples` samples:
 * the next pt_render whose sample range reaches that count writes the running
 * mean at that sample into the snapshot (bitwise what pt_denoise_snapshot
 * would copy after stopping there), so a whole denoiser input takes one
 * render call.  0 disarms. */
int pt_denoise_snapshot_at(pt_ctx* ctx, uint32_t samples);
/* Packs the context's current mean image and features into a denoiser input
 * (bf16 [h][w][16], device) for an image of `spp` samples per pixel, and when
 * `base` is not NULL its residual base (fp32 [h][w][4]: log(1 + radiance),
 * 0). */
int pt_denoise_input(pt_ctx* ctx, uint32_t spp, uint16_t* input, float* base, void* stream);
/* Packs, runs the network (batch 1, same size as the image) and stores
 * expm1(max(out, 0)) as the context's denoised RGBA image, read back with
 * pt_read_image(ctx, rgba, pitch, PT_IMAGE_DENOISED). */
int pt_denoise(pt_ctx* ctx, pt_unet* u, uint32_t spp);
#define PT_IMAGE_DENOISED 2

#ifdef __cplusplus
}
#endif

#endif
