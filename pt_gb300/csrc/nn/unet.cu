// unet.cu — forward, backward and Adam for the denoiser U-Net.
//
// Layer order (encoder, bottleneck, decoder):
//   0 e0a 16->32   1 e0b 32->32   (level 0, full resolution)
//   2 e1a 32->64   3 e1b 64->64   (level 1)
//   4 e2a 64->96   5 e2b 96->96   (level 2)
//   6 b3a 96->128  7 b3b 128->128 (level 3)
//   8 d2a 224->96  9 d2b 96->96   (level 2: upsampled b3b ++ e2b)
//  10 d1a 160->64 11 d1b 64->64   (level 1: upsampled d2b ++ e1b)
//  12 d0a 96->32  13 d0b 32->32   (level 0: upsampled d1b ++ e0b)
//  14 out 32->16 (linear)
// The skip outputs e0b / e1b / e2b are written straight into the upper
// channel range of the decoder's concatenation buffer.
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>

#include "unet.h"

namespace pt {
namespace nn {

const LayerSpec LAYERS[N_LAYERS] = {
    {16, 32, true},   {32, 32, true},   {32, 64, true},  {64, 64, true},  {64, 96, true},
    {96, 96, true},   {96, 128, true},  {128, 128, true}, {224, 96, true}, {96, 96, true},
    {160, 64, true},  {64, 64, true},   {96, 32, true},  {32, 32, true},  {32, 16, false},
};

size_t weight_offset(int layer)
{
    size_t off = 0;
    for (int l = 0; l < layer; l++)
        off += (size_t)9 * LAYERS[l].cin * LAYERS[l].cout + LAYERS[l].cout;
    return off;
}

size_t bias_offset(int layer)
{
    return weight_offset(layer) + (size_t)9 * LAYERS[layer].cin * LAYERS[layer].cout;
}

size_t param_count()
{
    return weight_offset(N_LAYERS);
}

namespace {

__global__ void k_loss(const float* out32, const float4* target, size_t pixels, uint16_t* g_out, double* loss_acc)
{
    double local = 0.0;
    const float scale = 2.0f / (3.0f * (float)pixels);
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < pixels; p += (size_t)gridDim.x * blockDim.x) {
        const float4 t4 = target[p];
        const float t[3] = {t4.x, t4.y, t4.z};
        uint32_t g2[2];
        float gv[4] = {0, 0, 0, 0};
        for (int c = 0; c < 3; c++) {
            const float tc = fmaxf(t[c], 0.0f);
            const float y = log1pf(tc);
            const float wgt = (1.0f + fminf(tc, LOSS_CLAMP)) * (1.0f + fminf(tc, LOSS_CLAMP));
            const float d = out32[p * OUT_CHANNELS + c] - y;
            local += (double)(wgt * d * d);
            gv[c] = scale * wgt * d;
        }
        __nv_bfloat162 a = __floats2bfloat162_rn(gv[0], gv[1]);
        __nv_bfloat162 b = __floats2bfloat162_rn(gv[2], gv[3]);
        g2[0] = *reinterpret_cast<uint32_t*>(&a);
        g2[1] = *reinterpret_cast<uint32_t*>(&b);
        *reinterpret_cast<uint2*>(g_out + p * OUT_CHANNELS) = make_uint2(g2[0], g2[1]);
    }
    for (int o = 16; o > 0; o >>= 1)
        local += __shfl_down_sync(0xffffffffu, local, o);
    if ((threadIdx.x & 31) == 0)
        atomicAdd(loss_acc, local);
}

} // namespace

cudaError_t loss_backward(const float* out32, const float* target, size_t pixels, uint16_t* g_out, double* loss_acc,
                          cudaStream_t st)
{
    size_t blocks = (pixels + 255) / 256;
    if (blocks > 152 * 8)
        blocks = 152 * 8;
    k_loss<<<(unsigned)(blocks ? blocks : 1), 256, 0, st>>>(out32, reinterpret_cast<const float4*>(target), pixels, g_out,
                                                             loss_acc);
    return cudaGetLastError();
}

UNet::~UNet()
{
    if (!allocs_.empty()) {
        cudaSetDevice(device_);
        for (void* p : allocs_)
            cudaFree(p);
    }
}

void* UNet::alloc(size_t bytes)
{
    void* p = nullptr;
    if (cudaMalloc(&p, (bytes + 255) & ~(size_t)255) != cudaSuccess)
        return nullptr;
    allocs_.push_back(p);
    return p;
}

bool UNet::make(Buf& b, int level, int channels, std::string& err)
{
    b.a.n = n_;
    b.a.h = h_ >> level;
    b.a.w = w_ >> level;
    b.a.pitch = channels;
    b.a.p = static_cast<uint16_t*>(alloc(b.a.pixels() * channels * 2));
    if (!b.a.p) {
        err = "device allocation of a denoiser activation failed";
        return false;
    }
    cudaMemset(b.a.p, 0, b.a.pixels() * channels * 2);
    int tx, ty;
    const char* why = nullptr;
    conv_tile_shape(b.a.w, tx, ty);
    if (!encode_act_map(&b.tile, b.a, tx, ty, &why)) {
        err = why;
        return false;
    }
    wgrad_chunk_shape(b.a.w, tx, ty);
    if (!encode_act_map(&b.chunk, b.a, tx, ty, &why)) {
        err = why;
        return false;
    }
    for (int k = 0; k < 4; k++)
        if (!encode_act_map(&b.halo[k], b.a, 130, (1 << k) + 2, &why)) {
            err = why;
            return false;
        }
    return true;
}

static int halo_index(int rows)
{
    return rows >= 8 ? 3 : rows >= 4 ? 2 : rows >= 2 ? 1 : 0;
}

bool UNet::init(int device, int n, int h, int w, std::string& err)
{
    if (n < 1 || h < 8 || w < 8 || h % 8 || w % 8) {
        err = "denoiser batch must be >= 1 and image sides multiples of 8";
        return false;
    }
    device_ = device;
    n_ = n;
    h_ = h;
    w_ = w;
    if (cudaSetDevice(device) != cudaSuccess) {
        err = "cudaSetDevice failed";
        return false;
    }
    cudaDeviceGetAttribute(&sm_count_, cudaDevAttrMultiProcessorCount, device);
    struct {
        Buf* b;
        int level, c;
    } acts[] = {
        {&x0_, 0, 16},     {&e0a_, 0, 32},    {&cat0_, 0, 96},   {&p1_, 1, 32},     {&e1a_, 1, 64},    {&cat1_, 1, 160},
        {&p2_, 2, 64},     {&e2a_, 2, 96},    {&cat2_, 2, 224},  {&p3_, 3, 96},     {&b3a_, 3, 128},   {&b3b_, 3, 128},
        {&d2a_, 2, 96},    {&d2b_, 2, 96},    {&d1a_, 1, 64},    {&d1b_, 1, 64},    {&d0a_, 0, 32},    {&d0b_, 0, 32},
        {&g_out_, 0, 16},  {&g_d0b_, 0, 32},  {&g_d0a_, 0, 32},  {&g_cat0_, 0, 96}, {&g_d1b_, 1, 64},  {&g_d1a_, 1, 64},
        {&g_cat1_, 1, 160}, {&g_d2b_, 2, 96}, {&g_d2a_, 2, 96},  {&g_cat2_, 2, 224}, {&g_b3b_, 3, 128}, {&g_b3a_, 3, 128},
        {&g_p3_, 3, 96},   {&g_e2b_, 2, 96},  {&g_e2a_, 2, 96},  {&g_p2_, 2, 64},   {&g_e1b_, 1, 64},  {&g_e1a_, 1, 64},
        {&g_p1_, 1, 32},   {&g_e0b_, 0, 32},  {&g_e0a_, 0, 32},
    };
    for (auto& a : acts)
        if (!make(*a.b, a.level, a.c, err))
            return false;
    const size_t P = param_count();
    out32_ = static_cast<float*>(alloc((size_t)n * h * w * OUT_CHANNELS * sizeof(float)));
    base32_ = static_cast<float*>(alloc((size_t)n * h * w * 4 * sizeof(float)));
    params_ = static_cast<float*>(alloc(P * sizeof(float)));
    grads_ = static_cast<float*>(alloc(P * sizeof(float)));
    adam_m_ = static_cast<float*>(alloc(P * sizeof(float)));
    adam_v_ = static_cast<float*>(alloc(P * sizeof(float)));
    size_t packed = 0;
    for (int l = 0; l < N_LAYERS; l++) {
        packed_off_[l] = packed;
        packed += packed_elems(LAYERS[l].cin, LAYERS[l].cout);
    }
    wfwd_ = static_cast<uint16_t*>(alloc(packed * 2));
    wbwd_ = static_cast<uint16_t*>(alloc(packed * 2));
    wrfwd_ = static_cast<uint16_t*>(alloc(packed * 2));
    wrbwd_ = static_cast<uint16_t*>(alloc(packed * 2));
    rows_ = use_rows_kernel();
    loss_acc_ = static_cast<double*>(alloc(sizeof(double)));
    error_ = static_cast<uint32_t*>(alloc(sizeof(uint32_t)));
    if (!out32_ || !base32_ || !params_ || !grads_ || !adam_m_ || !adam_v_ || !wfwd_ || !wbwd_ || !wrfwd_ || !wrbwd_ ||
        !loss_acc_ || !error_) {
        err = "device allocation of denoiser parameters failed";
        return false;
    }
    cudaMemset(params_, 0, P * sizeof(float));
    cudaMemset(adam_m_, 0, P * sizeof(float));
    cudaMemset(adam_v_, 0, P * sizeof(float));
    cudaMemset(error_, 0, sizeof(uint32_t));
    cudaMemset(base32_, 0, (size_t)n * h * w * 4 * sizeof(float));
    if (cudaDeviceSynchronize() != cudaSuccess) {
        err = "denoiser initialisation failed";
        return false;
    }
    return true;
}

bool UNet::set_params(const float* host, size_t count, std::string& err)
{
    if (count != param_count()) {
        err = "parameter count mismatch";
        return false;
    }
    cudaSetDevice(device_);
    if (cudaMemcpy(params_, host, count * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) {
        err = "parameter upload failed";
        return false;
    }
    cudaMemset(adam_m_, 0, count * sizeof(float));
    cudaMemset(adam_v_, 0, count * sizeof(float));
    adam_t_ = 0;
    packed_ok_ = false;
    return true;
}

bool UNet::get_params(float* host, size_t count, std::string& err)
{
    if (count != param_count()) {
        err = "parameter count mismatch";
        return false;
    }
    cudaSetDevice(device_);
    return cudaMemcpy(host, params_, count * sizeof(float), cudaMemcpyDeviceToHost) == cudaSuccess;
}

bool UNet::get_grads(float* host, size_t count, std::string& err)
{
    if (count != param_count()) {
        err = "parameter count mismatch";
        return false;
    }
    cudaSetDevice(device_);
    return cudaMemcpy(host, grads_, count * sizeof(float), cudaMemcpyDeviceToHost) == cudaSuccess;
}

bool UNet::get_adam_state(float* m, float* v, size_t count, uint32_t* step, std::string& err)
{
    if (count != param_count()) {
        err = "parameter count mismatch";
        return false;
    }
    cudaSetDevice(device_);
    if (cudaMemcpy(m, adam_m_, count * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(v, adam_v_, count * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess) {
        err = "optimizer state download failed";
        return false;
    }
    *step = (uint32_t)adam_t_;
    return true;
}

bool UNet::set_adam_state(const float* m, const float* v, size_t count, uint32_t step, std::string& err)
{
    if (count != param_count()) {
        err = "parameter count mismatch";
        return false;
    }
    if (step > (uint32_t)INT32_MAX) {
        err = "optimizer step out of range";
        return false;
    }
    cudaSetDevice(device_);
    if (cudaMemcpy(adam_m_, m, count * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(adam_v_, v, count * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) {
        err = "optimizer state upload failed";
        return false;
    }
    adam_t_ = (int)step;
    return true;
}

uint32_t UNet::device_error()
{
    uint32_t e = 0;
    cudaMemcpy(&e, error_, sizeof(e), cudaMemcpyDeviceToHost);
    return e;
}

cudaError_t UNet::repack(cudaStream_t st)
{
    for (int l = 0; l < N_LAYERS; l++) {
        cudaError_t e = rows_ ? pack_weights_rows(params_ + weight_offset(l), LAYERS[l].cin, LAYERS[l].cout,
                                                  wrfwd_ + packed_off_[l], wrbwd_ + packed_off_[l], st)
                              : pack_weights(params_ + weight_offset(l), LAYERS[l].cin, LAYERS[l].cout,
                                             wfwd_ + packed_off_[l], wbwd_ + packed_off_[l], st);
        if (e != cudaSuccess)
            return e;
    }
    packed_ok_ = true;
    return cudaSuccess;
}

cudaError_t UNet::run_conv(ConvCall& c, Buf& in, const uint16_t* rows_wpk, cudaStream_t st)
{
    if (!rows_)
        return conv3x3(c, error_, st);
    c.wpk = rows_wpk;
    return conv3x3_rows(c, &in.halo[halo_index(rows_per_tile(c.nout))], sm_count_, error_, st);
}

cudaError_t UNet::conv(int l, Buf& in, int c0, Buf& out, int out_c0, cudaStream_t st)
{
    ConvCall c{};
    c.in_map = &in.tile;
    c.in = in.a;
    c.c0 = c0;
    c.cin = LAYERS[l].cin;
    c.wpk = wfwd_ + packed_off_[l];
    c.nout = LAYERS[l].cout;
    c.bias = params_ + bias_offset(l);
    c.relu = LAYERS[l].relu;
    c.out = out.a;
    c.out_c0 = out_c0;
    return run_conv(c, in, wrfwd_ + packed_off_[l], st);
}

cudaError_t UNet::dgrad(int l, Buf& g, Buf& out, const Buf* mask, int mask_c0, cudaStream_t st)
{
    ConvCall c{};
    c.in_map = &g.tile;
    c.in = g.a;
    c.c0 = 0;
    c.cin = LAYERS[l].cout;
    c.wpk = wbwd_ + packed_off_[l];
    c.nout = LAYERS[l].cin;
    c.bias = nullptr;
    c.relu = false;
    c.out = out.a;
    c.out_c0 = 0;
    c.mask = mask ? &mask->a : nullptr;
    c.mask_c0 = mask_c0;
    return run_conv(c, g, wrbwd_ + packed_off_[l], st);
}

cudaError_t UNet::wgrad(int l, Buf& x, int x_c0, Buf& g, cudaStream_t st)
{
    WgradCall c{};
    c.x_map = &x.chunk;
    c.x_c0 = x_c0;
    c.cin = LAYERS[l].cin;
    c.g_map = &g.chunk;
    c.g_c0 = 0;
    c.cout = LAYERS[l].cout;
    c.n = g.a.n;
    c.h = g.a.h;
    c.w = g.a.w;
    c.dw = grads_ + weight_offset(l);
    cudaError_t e = conv3x3_wgrad(c, sm_count_, error_, st);
    if (e != cudaSuccess)
        return e;
    return bias_grad(g.a, 0, LAYERS[l].cout, grads_ + bias_offset(l), st);
}

#define PT_TRY(x)                                                                                                                 \
    do {                                                                                                                          \
        cudaError_t e_ = (x);                                                                                                     \
        if (e_ != cudaSuccess)                                                                                                    \
            return e_;                                                                                                            \
    } while (0)

cudaError_t UNet::forward(cudaStream_t st)
{
    cudaSetDevice(device_);
    if (!packed_ok_)
        PT_TRY(repack(st));
    PT_TRY(conv(0, x0_, 0, e0a_, 0, st));
    PT_TRY(conv(1, e0a_, 0, cat0_, 64, st));
    PT_TRY(pool2(cat0_.a, 64, 32, p1_.a, 0, st));
    PT_TRY(conv(2, p1_, 0, e1a_, 0, st));
    PT_TRY(conv(3, e1a_, 0, cat1_, 96, st));
    PT_TRY(pool2(cat1_.a, 96, 64, p2_.a, 0, st));
    PT_TRY(conv(4, p2_, 0, e2a_, 0, st));
    PT_TRY(conv(5, e2a_, 0, cat2_, 128, st));
    PT_TRY(pool2(cat2_.a, 128, 96, p3_.a, 0, st));
    PT_TRY(conv(6, p3_, 0, b3a_, 0, st));
    PT_TRY(conv(7, b3a_, 0, b3b_, 0, st));
    PT_TRY(upsample2(b3b_.a, 0, 128, cat2_.a, 0, st));
    PT_TRY(conv(8, cat2_, 0, d2a_, 0, st));
    PT_TRY(conv(9, d2a_, 0, d2b_, 0, st));
    PT_TRY(upsample2(d2b_.a, 0, 96, cat1_.a, 0, st));
    PT_TRY(conv(10, cat1_, 0, d1a_, 0, st));
    PT_TRY(conv(11, d1a_, 0, d1b_, 0, st));
    PT_TRY(upsample2(d1b_.a, 0, 64, cat0_.a, 0, st));
    PT_TRY(conv(12, cat0_, 0, d0a_, 0, st));
    PT_TRY(conv(13, d0a_, 0, d0b_, 0, st));
    // output layer in fp32
    ConvCall c{};
    c.in_map = &d0b_.tile;
    c.in = d0b_.a;
    c.cin = LAYERS[14].cin;
    c.wpk = wfwd_ + packed_off_[14];
    c.nout = LAYERS[14].cout;
    c.bias = params_ + bias_offset(14);
    c.relu = false;
    c.out = d0b_.a;
    c.out.pitch = OUT_CHANNELS;
    c.out_f32 = out32_;
    c.residual = base32_;
    return run_conv(c, d0b_, wrfwd_ + packed_off_[14], st);
}

cudaError_t UNet::backward(const float* target, double* loss, cudaStream_t st)
{
    cudaSetDevice(device_);
    PT_TRY(cudaMemsetAsync(grads_, 0, param_count() * sizeof(float), st));
    PT_TRY(cudaMemsetAsync(loss_acc_, 0, sizeof(double), st));
    PT_TRY(loss_backward(out32_, target, x0_.a.pixels(), g_out_.a.p, loss_acc_, st));
    // output layer and level-0 decoder
    PT_TRY(wgrad(14, d0b_, 0, g_out_, st));
    PT_TRY(dgrad(14, g_out_, g_d0b_, &d0b_, 0, st));
    PT_TRY(wgrad(13, d0a_, 0, g_d0b_, st));
    PT_TRY(dgrad(13, g_d0b_, g_d0a_, &d0a_, 0, st));
    PT_TRY(wgrad(12, cat0_, 0, g_d0a_, st));
    PT_TRY(dgrad(12, g_d0a_, g_cat0_, nullptr, 0, st));
    PT_TRY(upsample2_backward(g_cat0_.a, 0, 64, d1b_.a, 0, g_d1b_.a, st));
    // level 1 decoder
    PT_TRY(wgrad(11, d1a_, 0, g_d1b_, st));
    PT_TRY(dgrad(11, g_d1b_, g_d1a_, &d1a_, 0, st));
    PT_TRY(wgrad(10, cat1_, 0, g_d1a_, st));
    PT_TRY(dgrad(10, g_d1a_, g_cat1_, nullptr, 0, st));
    PT_TRY(upsample2_backward(g_cat1_.a, 0, 96, d2b_.a, 0, g_d2b_.a, st));
    // level 2 decoder
    PT_TRY(wgrad(9, d2a_, 0, g_d2b_, st));
    PT_TRY(dgrad(9, g_d2b_, g_d2a_, &d2a_, 0, st));
    PT_TRY(wgrad(8, cat2_, 0, g_d2a_, st));
    PT_TRY(dgrad(8, g_d2a_, g_cat2_, nullptr, 0, st));
    PT_TRY(upsample2_backward(g_cat2_.a, 0, 128, b3b_.a, 0, g_b3b_.a, st));
    // bottleneck
    PT_TRY(wgrad(7, b3a_, 0, g_b3b_, st));
    PT_TRY(dgrad(7, g_b3b_, g_b3a_, &b3a_, 0, st));
    PT_TRY(wgrad(6, p3_, 0, g_b3a_, st));
    PT_TRY(dgrad(6, g_b3a_, g_p3_, nullptr, 0, st));
    PT_TRY(pool2_backward(g_cat2_.a, 128, g_p3_.a, 96, cat2_.a, 128, g_e2b_.a, st));
    // level 2 encoder
    PT_TRY(wgrad(5, e2a_, 0, g_e2b_, st));
    PT_TRY(dgrad(5, g_e2b_, g_e2a_, &e2a_, 0, st));
    PT_TRY(wgrad(4, p2_, 0, g_e2a_, st));
    PT_TRY(dgrad(4, g_e2a_, g_p2_, nullptr, 0, st));
    PT_TRY(pool2_backward(g_cat1_.a, 96, g_p2_.a, 64, cat1_.a, 96, g_e1b_.a, st));
    // level 1 encoder
    PT_TRY(wgrad(3, e1a_, 0, g_e1b_, st));
    PT_TRY(dgrad(3, g_e1b_, g_e1a_, &e1a_, 0, st));
    PT_TRY(wgrad(2, p1_, 0, g_e1a_, st));
    PT_TRY(dgrad(2, g_e1a_, g_p1_, nullptr, 0, st));
    PT_TRY(pool2_backward(g_cat0_.a, 64, g_p1_.a, 32, cat0_.a, 64, g_e0b_.a, st));
    // level 0 encoder
    PT_TRY(wgrad(1, e0a_, 0, g_e0b_, st));
    PT_TRY(dgrad(1, g_e0b_, g_e0a_, &e0a_, 0, st));
    PT_TRY(wgrad(0, x0_, 0, g_e0a_, st));
    if (loss) {
        PT_TRY(cudaMemcpyAsync(loss, loss_acc_, sizeof(double), cudaMemcpyDeviceToHost, st));
        PT_TRY(cudaStreamSynchronize(st));
        *loss /= 3.0 * (double)x0_.a.pixels();
    }
    return cudaSuccess;
}

cudaError_t UNet::adam(float lr, cudaStream_t st)
{
    cudaSetDevice(device_);
    adam_t_++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float bc1 = 1.0f - powf(b1, (float)adam_t_), bc2 = 1.0f - powf(b2, (float)adam_t_);
    PT_TRY(adam_step(params_, grads_, adam_m_, adam_v_, param_count(), lr, b1, b2, 1e-8f, bc1, bc2, st));
    return repack(st);
}

} // namespace nn
} // namespace pt
