// api_nn.cu — C ABI of the denoiser network (include/pt_denoise.h).
#include <cstring>
#include <new>
#include <string>

#include "../../../include/pt_denoise.h"
#include "unet.h"

struct pt_unet {
    pt::nn::UNet net;
    std::string err;
    int fail(int code, const std::string& m)
    {
        err = m;
        return code;
    }
    int cuda_fail(cudaError_t e, const char* what)
    {
        err = std::string(what) + ": " + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? PT_ERR_OOM : PT_ERR_CUDA;
    }
};

static thread_local std::string g_unet_create_error;

namespace {

using pt::nn::Act;

// Per-call tensor maps for the single-layer entry points.
bool map_for(CUtensorMap* tile, CUtensorMap* chunk, const Act& a, std::string& err)
{
    int tx, ty;
    const char* why = nullptr;
    pt::nn::conv_tile_shape(a.w, tx, ty);
    if (tile && !pt::nn::encode_act_map(tile, a, tx, ty, &why)) {
        err = why;
        return false;
    }
    pt::nn::wgrad_chunk_shape(a.w, tx, ty);
    if (chunk && !pt::nn::encode_act_map(chunk, a, tx, ty, &why)) {
        err = why;
        return false;
    }
    return true;
}

thread_local std::string g_layer_error;

struct Scratch {
    uint16_t* fwd = nullptr;
    uint16_t* bwd = nullptr;
    uint32_t* err = nullptr;
    ~Scratch()
    {
        cudaFree(fwd);
        cudaFree(bwd);
        cudaFree(err);
    }
    bool init(uint32_t cin, uint32_t cout)
    {
        size_t n = pt::nn::packed_elems(cin, cout) * 2;
        return cudaMalloc(&fwd, n) == cudaSuccess && cudaMalloc(&bwd, n) == cudaSuccess &&
               cudaMalloc(&err, 4) == cudaSuccess && cudaMemset(err, 0, 4) == cudaSuccess;
    }
    int finish(cudaStream_t st)
    {
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            g_layer_error = cudaGetErrorString(e);
            return PT_ERR_CUDA;
        }
        uint32_t w = 0;
        cudaMemcpy(&w, err, 4, cudaMemcpyDeviceToHost);
        if (w) {
            g_layer_error = "tensor-core kernel timed out waiting on a barrier";
            return PT_ERR_DEVICE;
        }
        return PT_OK;
    }
};

int sm_count()
{
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms;
}

// One convolution through the selected kernel; the halo map is made per call.
cudaError_t run(pt::nn::ConvCall& c, const Act& in, bool rows, cudaStream_t st, uint32_t* err)
{
    if (!rows)
        return pt::nn::conv3x3(c, err, st);
    CUtensorMap halo;
    const char* why = nullptr;
    const int mt = pt::nn::rows_per_tile(c.nout);
    if (!pt::nn::encode_act_map(&halo, in, 130, mt + 2, &why)) {
        g_layer_error = why;
        return cudaErrorInvalidValue;
    }
    return pt::nn::conv3x3_rows(c, &halo, sm_count(), err, st);
}

bool shape_ok(uint32_t n, uint32_t h, uint32_t w, uint32_t pitch, uint32_t c0, uint32_t c)
{
    return n && h && w && pitch % 16 == 0 && c0 % 8 == 0 && c % 16 == 0 && c0 + c <= pitch && c > 0;
}

} // namespace

extern "C" {

size_t pt_unet_param_count(void)
{
    return pt::nn::param_count();
}

int pt_unet_layer_shape(int layer, uint32_t* c_in, uint32_t* c_out)
{
    if (layer < 0 || layer >= pt::nn::N_LAYERS)
        return 0;
    if (c_in)
        *c_in = (uint32_t)pt::nn::LAYERS[layer].cin;
    if (c_out)
        *c_out = (uint32_t)pt::nn::LAYERS[layer].cout;
    return 1;
}

pt_unet* pt_unet_create(int device, uint32_t batch, uint32_t height, uint32_t width)
{
    pt_unet* u = new (std::nothrow) pt_unet();
    if (!u) {
        g_unet_create_error = "out of host memory";
        return nullptr;
    }
    std::string err;
    if (!u->net.init(device, (int)batch, (int)height, (int)width, err)) {
        g_unet_create_error = err;
        delete u;
        return nullptr;
    }
    return u;
}

void pt_unet_destroy(pt_unet* u)
{
    delete u;
}

const char* pt_unet_last_error(const pt_unet* u)
{
    if (!u)
        return g_unet_create_error.empty() ? g_layer_error.c_str() : g_unet_create_error.c_str();
    return u->err.c_str();
}

int pt_unet_set_params(pt_unet* u, const float* p, size_t count)
{
    if (!u || !p)
        return PT_ERR_INVALID;
    return u->net.set_params(p, count, u->err) ? PT_OK : PT_ERR_INVALID;
}

int pt_unet_get_params(pt_unet* u, float* p, size_t count)
{
    if (!u || !p)
        return PT_ERR_INVALID;
    return u->net.get_params(p, count, u->err) ? PT_OK : PT_ERR_INVALID;
}

int pt_unet_get_grads(pt_unet* u, float* g, size_t count)
{
    if (!u || !g)
        return PT_ERR_INVALID;
    return u->net.get_grads(g, count, u->err) ? PT_OK : PT_ERR_INVALID;
}

int pt_unet_get_adam_state(pt_unet* u, float* m, float* v, size_t count, uint32_t* step)
{
    if (!u || !m || !v || !step)
        return PT_ERR_INVALID;
    return u->net.get_adam_state(m, v, count, step, u->err) ? PT_OK : PT_ERR_INVALID;
}

int pt_unet_set_adam_state(pt_unet* u, const float* m, const float* v, size_t count, uint32_t step)
{
    if (!u || !m || !v)
        return PT_ERR_INVALID;
    return u->net.set_adam_state(m, v, count, step, u->err) ? PT_OK : PT_ERR_INVALID;
}

void pt_unet_shape(const pt_unet* u, uint32_t* batch, uint32_t* height, uint32_t* width)
{
    if (batch)
        *batch = u ? (uint32_t)u->net.n() : 0;
    if (height)
        *height = u ? (uint32_t)u->net.h() : 0;
    if (width)
        *width = u ? (uint32_t)u->net.w() : 0;
}

uint16_t* pt_unet_input(pt_unet* u)
{
    return u ? u->net.input() : nullptr;
}

const float* pt_unet_output(const pt_unet* u)
{
    return u ? u->net.output() : nullptr;
}

float* pt_unet_base(pt_unet* u)
{
    return u ? u->net.base() : nullptr;
}

int pt_unet_forward(pt_unet* u, float* output, void* stream)
{
    if (!u)
        return PT_ERR_INVALID;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = u->net.forward(st);
    if (e == cudaSuccess && output)
        e = cudaMemcpyAsync(output, u->net.output(),
                            (size_t)u->net.n() * u->net.h() * u->net.w() * pt::nn::OUT_CHANNELS * sizeof(float),
                            cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(st);
    if (e != cudaSuccess)
        return u->cuda_fail(e, "denoiser forward");
    if (u->net.device_error())
        return u->fail(PT_ERR_DEVICE, "tensor-core kernel timed out waiting on a barrier");
    return PT_OK;
}

int pt_unet_backward(pt_unet* u, const float* target, double* loss, void* stream)
{
    if (!u || !target)
        return PT_ERR_INVALID;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    double l = 0.0;
    cudaError_t e = u->net.backward(target, &l, st);
    if (e != cudaSuccess)
        return u->cuda_fail(e, "denoiser backward");
    if (u->net.device_error())
        return u->fail(PT_ERR_DEVICE, "tensor-core kernel timed out waiting on a barrier");
    if (loss)
        *loss = l;
    return PT_OK;
}

int pt_unet_adam(pt_unet* u, float lr, void* stream)
{
    if (!u || !(lr > 0.0f))
        return PT_ERR_INVALID;
    cudaError_t e = u->net.adam(lr, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess)
        return u->cuda_fail(e, "denoiser Adam step");
    return PT_OK;
}

int pt_nn_conv3x3(const uint16_t* in, uint32_t n, uint32_t h, uint32_t w, uint32_t in_pitch, uint32_t c0, uint32_t c_in,
                  const float* weights, const float* bias, uint32_t c_out, int relu, uint16_t* out, void* stream)
{
    if (!in || !weights || !out || !shape_ok(n, h, w, in_pitch, c0, c_in) || c_out % 16 || c_out == 0 || c_out > 256)
        return PT_ERR_INVALID;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    Scratch s;
    if (!s.init(c_in, c_out))
        return PT_ERR_OOM;
    Act a;
    a.p = const_cast<uint16_t*>(in);
    a.n = (int)n;
    a.h = (int)h;
    a.w = (int)w;
    a.pitch = (int)in_pitch;
    CUtensorMap tile;
    if (!map_for(&tile, nullptr, a, g_layer_error))
        return PT_ERR_INVALID;
    const bool rows = pt::nn::use_rows_kernel();
    if ((rows ? pt::nn::pack_weights_rows(weights, (int)c_in, (int)c_out, s.fwd, s.bwd, st)
              : pt::nn::pack_weights(weights, (int)c_in, (int)c_out, s.fwd, s.bwd, st)) != cudaSuccess)
        return PT_ERR_CUDA;
    pt::nn::ConvCall c{};
    c.in_map = &tile;
    c.in = a;
    c.c0 = (int)c0;
    c.cin = (int)c_in;
    c.wpk = s.fwd;
    c.nout = (int)c_out;
    c.bias = bias;
    c.relu = relu != 0;
    c.out = a;
    c.out.p = out;
    c.out.pitch = (int)c_out;
    if (run(c, a, rows, st, s.err) != cudaSuccess)
        return PT_ERR_CUDA;
    return s.finish(st);
}

int pt_nn_conv3x3_dgrad(const uint16_t* grad_out, uint32_t n, uint32_t h, uint32_t w, uint32_t c_out, const float* weights,
                        uint32_t c_in, const uint16_t* mask, uint16_t* grad_in, void* stream)
{
    if (!grad_out || !weights || !grad_in || !shape_ok(n, h, w, c_out, 0, c_out) || c_in % 16 || c_in == 0 || c_in > 256)
        return PT_ERR_INVALID;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    Scratch s;
    if (!s.init(c_in, c_out))
        return PT_ERR_OOM;
    Act g;
    g.p = const_cast<uint16_t*>(grad_out);
    g.n = (int)n;
    g.h = (int)h;
    g.w = (int)w;
    g.pitch = (int)c_out;
    CUtensorMap tile;
    if (!map_for(&tile, nullptr, g, g_layer_error))
        return PT_ERR_INVALID;
    const bool rows = pt::nn::use_rows_kernel();
    if ((rows ? pt::nn::pack_weights_rows(weights, (int)c_in, (int)c_out, s.fwd, s.bwd, st)
              : pt::nn::pack_weights(weights, (int)c_in, (int)c_out, s.fwd, s.bwd, st)) != cudaSuccess)
        return PT_ERR_CUDA;
    Act m = g;
    m.p = const_cast<uint16_t*>(mask);
    m.pitch = (int)c_in;
    pt::nn::ConvCall c{};
    c.in_map = &tile;
    c.in = g;
    c.cin = (int)c_out;
    c.wpk = s.bwd;
    c.nout = (int)c_in;
    c.out = g;
    c.out.p = grad_in;
    c.out.pitch = (int)c_in;
    c.mask = mask ? &m : nullptr;
    if (run(c, g, rows, st, s.err) != cudaSuccess)
        return PT_ERR_CUDA;
    return s.finish(st);
}

int pt_nn_conv3x3_wgrad(const uint16_t* in, uint32_t n, uint32_t h, uint32_t w, uint32_t in_pitch, uint32_t c0, uint32_t c_in,
                        const uint16_t* grad_out, uint32_t c_out, float* dw, void* stream)
{
    if (!in || !grad_out || !dw || !shape_ok(n, h, w, in_pitch, c0, c_in) || c_out % 16 || c_out == 0 || c_out > 128)
        return PT_ERR_INVALID;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    Scratch s;
    if (cudaMalloc(&s.err, 4) != cudaSuccess || cudaMemset(s.err, 0, 4) != cudaSuccess)
        return PT_ERR_OOM;
    Act x;
    x.p = const_cast<uint16_t*>(in);
    x.n = (int)n;
    x.h = (int)h;
    x.w = (int)w;
    x.pitch = (int)in_pitch;
    Act g = x;
    g.p = const_cast<uint16_t*>(grad_out);
    g.pitch = (int)c_out;
    CUtensorMap xc, gc;
    if (!map_for(nullptr, &xc, x, g_layer_error) || !map_for(nullptr, &gc, g, g_layer_error))
        return PT_ERR_INVALID;
    const int sms = sm_count();
    pt::nn::WgradCall c{};
    c.x_map = &xc;
    c.x_c0 = (int)c0;
    c.cin = (int)c_in;
    c.g_map = &gc;
    c.cout = (int)c_out;
    c.n = (int)n;
    c.h = (int)h;
    c.w = (int)w;
    c.dw = dw;
    if (pt::nn::conv3x3_wgrad(c, sms, s.err, st) != cudaSuccess)
        return PT_ERR_CUDA;
    return s.finish(st);
}

} // extern "C"
