// api.cu — the C ABI of libptgpu.so (include/pt_gpu.h): context, scene upload,
// acceleration-structure build, rendering and read-back.
//
// Replaces the reference's PathTraceDispatcher / PathTracer host code
// (src/pathtrace/ptdispatch.cpp:18-204, pathtrace.cpp:81-516) with one CUDA
// stream per context and explicit device buffers.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/pt_checked.h"
#include "../../include/pt_denoise.h"
#include "../../include/pt_gpu.h"
#include "ctx.h"
#include "device/render.cuh"
#include "kernels.h"

namespace pt {
cudaError_t render_init_tables(const uint32_t* table128, const float* srgb256, cudaStream_t stream);
}

using namespace pt;

namespace {


// Sobol' direction numbers for 4 dimensions: van der Corput, then the
// primitive polynomials / initial numbers (s, a, m) = (1, 0, {1}),
// (2, 1, {1, 3}), (3, 1, {1, 3, 1}) of Joe & Kuo (2008) — the table of
// shaders/pathtrace/sample.hlsli:31-67.
void sobol_table(uint32_t v[4][32])
{
    for (int b = 0; b < 32; b++)
        v[0][b] = 1u << (31 - b);
    const int s_[3] = {1, 2, 3};
    const uint32_t a_[3] = {0, 1, 1};
    const uint32_t m_[3][3] = {{1, 0, 0}, {1, 3, 0}, {1, 3, 1}};
    for (int d = 1; d < 4; d++) {
        int s = s_[d - 1];
        for (int k = 0; k < s; k++)
            v[d][k] = m_[d - 1][k] << (31 - k);
        for (int k = s; k < 32; k++) {
            uint32_t x = v[d][k - s] ^ (v[d][k - s] >> s);
            for (int j = 1; j < s; j++)
                if ((a_[d - 1] >> (s - 1 - j)) & 1u)
                    x ^= v[d][k - j];
            v[d][k] = x;
        }
    }
}

// 4x4 inverse by cofactors in FP64 (row-major), for world-to-object rows
// when the caller does not supply them.
void inverse4(const double m[16], double out[16])
{
    const double* a = m;
    double inv[16];
    inv[0] = a[5] * a[10] * a[15] - a[5] * a[11] * a[14] - a[9] * a[6] * a[15] + a[9] * a[7] * a[14] + a[13] * a[6] * a[11] - a[13] * a[7] * a[10];
    inv[4] = -a[4] * a[10] * a[15] + a[4] * a[11] * a[14] + a[8] * a[6] * a[15] - a[8] * a[7] * a[14] - a[12] * a[6] * a[11] + a[12] * a[7] * a[10];
    inv[8] = a[4] * a[9] * a[15] - a[4] * a[11] * a[13] - a[8] * a[5] * a[15] + a[8] * a[7] * a[13] + a[12] * a[5] * a[11] - a[12] * a[7] * a[9];
    inv[12] = -a[4] * a[9] * a[14] + a[4] * a[10] * a[13] + a[8] * a[5] * a[14] - a[8] * a[6] * a[13] - a[12] * a[5] * a[10] + a[12] * a[6] * a[9];
    inv[1] = -a[1] * a[10] * a[15] + a[1] * a[11] * a[14] + a[9] * a[2] * a[15] - a[9] * a[3] * a[14] - a[13] * a[2] * a[11] + a[13] * a[3] * a[10];
    inv[5] = a[0] * a[10] * a[15] - a[0] * a[11] * a[14] - a[8] * a[2] * a[15] + a[8] * a[3] * a[14] + a[12] * a[2] * a[11] - a[12] * a[3] * a[10];
    inv[9] = -a[0] * a[9] * a[15] + a[0] * a[11] * a[13] + a[8] * a[1] * a[15] - a[8] * a[3] * a[13] - a[12] * a[1] * a[11] + a[12] * a[3] * a[9];
    inv[13] = a[0] * a[9] * a[14] - a[0] * a[10] * a[13] - a[8] * a[1] * a[14] + a[8] * a[2] * a[13] + a[12] * a[1] * a[10] - a[12] * a[2] * a[9];
    inv[2] = a[1] * a[6] * a[15] - a[1] * a[7] * a[14] - a[5] * a[2] * a[15] + a[5] * a[3] * a[14] + a[13] * a[2] * a[7] - a[13] * a[3] * a[6];
    inv[6] = -a[0] * a[6] * a[15] + a[0] * a[7] * a[14] + a[4] * a[2] * a[15] - a[4] * a[3] * a[14] - a[12] * a[2] * a[7] + a[12] * a[3] * a[6];
    inv[10] = a[0] * a[5] * a[15] - a[0] * a[7] * a[13] - a[4] * a[1] * a[15] + a[4] * a[3] * a[13] + a[12] * a[1] * a[7] - a[12] * a[3] * a[5];
    inv[14] = -a[0] * a[5] * a[14] + a[0] * a[6] * a[13] + a[4] * a[1] * a[14] - a[4] * a[2] * a[13] - a[12] * a[1] * a[6] + a[12] * a[2] * a[5];
    inv[3] = -a[1] * a[6] * a[11] + a[1] * a[7] * a[10] + a[5] * a[2] * a[11] - a[5] * a[3] * a[10] - a[9] * a[2] * a[7] + a[9] * a[3] * a[6];
    inv[7] = a[0] * a[6] * a[11] - a[0] * a[7] * a[10] - a[4] * a[2] * a[11] + a[4] * a[3] * a[10] + a[8] * a[2] * a[7] - a[8] * a[3] * a[6];
    inv[11] = -a[0] * a[5] * a[11] + a[0] * a[7] * a[9] + a[4] * a[1] * a[11] - a[4] * a[3] * a[9] - a[8] * a[1] * a[7] + a[8] * a[3] * a[5];
    inv[15] = a[0] * a[5] * a[10] - a[0] * a[6] * a[9] - a[4] * a[1] * a[10] + a[4] * a[2] * a[9] + a[8] * a[1] * a[6] - a[8] * a[2] * a[5];
    double det = a[0] * inv[0] + a[1] * inv[4] + a[2] * inv[8] + a[3] * inv[12];
    double id = 1.0 / det;
    for (int i = 0; i < 16; i++)
        out[i] = inv[i] * id;
}

} // namespace


static thread_local std::string g_create_error;

// The 4-wide node a reachable BVH2 node must have (k_make_bvh4 restated):
// its grandchildren's links, and their boxes rounded outwards to half precision.
// The node's children are in range (checked by the caller); its
// grandchildren are read only when in range.
static bool bvh4_matches(const std::vector<BvhNode>& nodes, size_t i, const Bvh4Node& got)
{
    const BvhNode& nd = nodes[i];
    float b[6][4] = {};
    int ref[4] = {REF_EMPTY, REF_EMPTY, REF_EMPTY, REF_EMPTY};
    int k = 0;
    auto put = [&](float4 xy, float zlo, float zhi, int r) {
        b[0][k] = xy.x, b[1][k] = xy.y, b[2][k] = xy.z, b[3][k] = xy.w, b[4][k] = zlo, b[5][k] = zhi;
        ref[k++] = r;
    };
    for (int c = 0; c < 2; c++) {
        const int cr = c == 0 ? nd.link.x : nd.link.y;
        if (cr >= 0 && (size_t)cr < nodes.size()) {
            const BvhNode& g = nodes[cr];
            put(g.c0xy, g.c01z.x, g.c01z.y, g.link.x);
            put(g.c1xy, g.c01z.z, g.c01z.w, g.link.y);
        } else if (c == 0) {
            put(nd.c0xy, nd.c01z.x, nd.c01z.y, cr);
        } else {
            put(nd.c1xy, nd.c01z.z, nd.c01z.w, cr);
        }
    }
    // each half-precision plane is the BVH2's plane rounded outwards
    const uint4* axes[3] = {&got.x, &got.y, &got.z};
    for (int a = 0; a < 3; a++) {
        const uint32_t w[4] = {axes[a]->x, axes[a]->y, axes[a]->z, axes[a]->w};
        for (int j = 0; j < k; j++) {
            const uint32_t lo_w = w[j / 2], hi_w = w[2 + j / 2];
            const unsigned short lo_bits = (unsigned short)(j & 1 ? lo_w >> 16 : lo_w & 0xFFFFu);
            const unsigned short hi_bits = (unsigned short)(j & 1 ? hi_w >> 16 : hi_w & 0xFFFFu);
            const __half lo = __ushort_as_half(lo_bits), hi = __ushort_as_half(hi_bits);
            if (!(lo_bits == __half_as_ushort(__float2half_rd(b[2 * a][j])) && __half2float(lo) <= b[2 * a][j]))
                return false;
            if (!(hi_bits == __half_as_ushort(__float2half_ru(b[2 * a + 1][j])) && __half2float(hi) >= b[2 * a + 1][j]))
                return false;
        }
    }
    const int gl[4] = {got.link.x, got.link.y, got.link.z, got.link.w};
    return std::memcmp(gl, ref, sizeof(gl)) == 0;
}

// Host-side structural check of a freshly built acceleration structure
// (enabled by PT_VALIDATE_BVH=1): every reference in range, every BLAS
// covering each of its mesh's triangles exactly once, the TLAS covering each
// instance exactly once, no cycles, and each reachable node's 4-wide copy
// holding its grandchildren.  Returns an empty string when valid.
static std::string validate_accel(pt_ctx* c, const std::vector<uint32_t>& tri_base)
{
    const uint32_t T = c->tri_count, I = c->instance_count, M = c->mesh_count;
    const size_t blas_nodes = T > 1 ? T - 1 : 0;
    std::vector<BvhNode> nodes(c->nodes.n);
    std::vector<Bvh4Node> nodes4(c->nodes4.p ? c->nodes4.n : 0);
    std::vector<TriRec> tris(T);
    std::vector<int> roots(M);
    std::vector<DevInstance> dinst(I);
    if (cudaMemcpy(nodes.data(), c->nodes.p, nodes.size() * sizeof(BvhNode), cudaMemcpyDeviceToHost) != cudaSuccess ||
        (!nodes4.empty() &&
         cudaMemcpy(nodes4.data(), c->nodes4.p, nodes4.size() * sizeof(Bvh4Node), cudaMemcpyDeviceToHost) != cudaSuccess) ||
        (T && cudaMemcpy(tris.data(), c->tris.p, T * sizeof(TriRec), cudaMemcpyDeviceToHost) != cudaSuccess) ||
        (M && cudaMemcpy(roots.data(), c->mesh_root.p, M * sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) ||
        (I && cudaMemcpy(dinst.data(), c->dinst.p, I * sizeof(DevInstance), cudaMemcpyDeviceToHost) != cudaSuccess))
        return "copy-back failed";
    std::vector<uint8_t> seen(std::max<size_t>(T, I), 0);
    auto walk = [&](int root, size_t node_lo, size_t node_hi, uint32_t leaf_lo, uint32_t leaf_hi, uint32_t expect) -> std::string {
        std::vector<int> st{root};
        size_t internal = 0;
        uint32_t leaves = 0;
        while (!st.empty()) {
            int r = st.back();
            st.pop_back();
            if (r >= 0) {
                if ((size_t)r < node_lo || (size_t)r >= node_hi)
                    return "node reference " + std::to_string(r) + " out of range";
                if (++internal > (size_t)expect)
                    return "cycle or duplicate nodes";
                for (int ch : {nodes[r].link.x, nodes[r].link.y})
                    if (ch >= 0 && ((size_t)ch < node_lo || (size_t)ch >= node_hi))
                        return "node reference " + std::to_string(ch) + " out of range";
                if (!nodes4.empty() && !bvh4_matches(nodes, (size_t)r, nodes4[r]))
                    return "4-wide node " + std::to_string(r) + " differs from its BVH2 grandchildren";
                st.push_back(nodes[r].link.x);
                st.push_back(nodes[r].link.y);
            } else if (ref_is_leaf(r)) {
                uint32_t f = leaf_first(r), n = leaf_count(r);
                if (f < leaf_lo || f + n > leaf_hi)
                    return "leaf range out of bounds";
                for (uint32_t k = f; k < f + n; k++) {
                    if (seen[k]++)
                        return "primitive referenced twice";
                }
                leaves += n;
            } else {
                return "sentinel inside the tree";
            }
        }
        return leaves == expect ? "" : "tree covers " + std::to_string(leaves) + " of " + std::to_string(expect) + " primitives";
    };
    for (uint32_t m = 0; m < M; m++) {
        uint32_t n = tri_base[m + 1] - tri_base[m];
        if (n == 0) {
            if (roots[m] != REF_EMPTY)
                return "empty mesh with a root";
            continue;
        }
        std::string e = walk(roots[m], 0, blas_nodes, tri_base[m], tri_base[m + 1], n);
        if (!e.empty())
            return "mesh " + std::to_string(m) + ": " + e;
        for (uint32_t k = tri_base[m]; k < tri_base[m + 1]; k++) {
            uint32_t prim;
            std::memcpy(&prim, &tris[k].v0.w, 4);
            if (prim >= n)
                return "mesh " + std::to_string(m) + ": primitive index out of range";
        }
    }
    std::fill(seen.begin(), seen.end(), 0);
    if (I > 0) {
        std::string e = walk(c->tlas_root, blas_nodes, blas_nodes + (I > 1 ? I - 1 : 0), 0, I, I);
        if (!e.empty())
            return "TLAS: " + e;
        std::vector<uint32_t> im(I);
        cudaMemcpy(im.data(), c->inst_mesh.p, I * sizeof(uint32_t), cudaMemcpyDeviceToHost);
        for (uint32_t i = 0; i < I; i++)
            if (dinst[i].blas_root != roots[im[i]])
                return "instance " + std::to_string(i) + " has the wrong BLAS root";
    }
    return "";
}

template <typename T>
static cudaError_t upload(pt_ctx* c, DevBuf<T>& b, const T* src, size_t n)
{
    cudaError_t e = b.alloc(n);
    if (e != cudaSuccess || n == 0)
        return e;
    return cudaMemcpyAsync(b.p, src, n * sizeof(T), cudaMemcpyHostToDevice, c->stream);
}


extern "C" {

int pt_abi_version(void) { return PT_ABI_VERSION; }

pt_ctx* pt_create(int device)
{
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        g_create_error = std::string("no CUDA device: ") + cudaGetErrorString(e);
        return nullptr;
    }
    if (device < 0 || device >= count) {
        g_create_error = "device index out of range";
        return nullptr;
    }
    e = cudaSetDevice(device);
    if (e != cudaSuccess) {
        g_create_error = std::string("cudaSetDevice: ") + cudaGetErrorString(e);
        return nullptr;
    }
    pt_ctx* c = new (std::nothrow) pt_ctx();
    if (!c) {
        g_create_error = "out of host memory";
        return nullptr;
    }
    c->device = device;
    if ((e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreate(&c->ev0)) != cudaSuccess || (e = cudaEventCreate(&c->ev1)) != cudaSuccess ||
        (e = c->counters.alloc(8)) != cudaSuccess || (e = c->error_word.alloc(1)) != cudaSuccess) {
        g_create_error = std::string("context set-up: ") + cudaGetErrorString(e);
        delete c;
        return nullptr;
    }
    uint32_t table[4][32];
    sobol_table(table);
    cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
    // sRGB decode of 8-bit texels (the _SRGB formats), evaluated in FP64 and rounded once
    float srgb[256];
    for (int i = 0; i < 256; i++) {
        const double v = i / 255.0;
        srgb[i] = (float)(v <= 0.04045 ? v / 12.92 : std::pow((v + 0.055) / 1.055, 2.4));
    }
    if ((e = render_init_tables(&table[0][0], srgb, c->stream)) != cudaSuccess ||
        (e = wave_init_tables(&table[0][0], srgb, c->stream)) != cudaSuccess ||
        (e = features_init_tables(&table[0][0], srgb, c->stream)) != cudaSuccess) {
        g_create_error = std::string("sampler tables: ") + cudaGetErrorString(e);
        delete c;
        return nullptr;
    }
    cudaMemsetAsync(c->error_word.p, 0, sizeof(uint32_t), c->stream);
    cudaStreamSynchronize(c->stream);
    return c;
}

void pt_destroy(pt_ctx* c)
{
    if (!c)
        return;
    cudaSetDevice(c->device);
    if (c->stream)
        cudaStreamSynchronize(c->stream);
    c->vertices.release();
    c->indices.release();
    c->inst_data.release();
    c->materials.release();
    c->material_ior.release();
    c->has_ior = false;
    c->light.release();
    c->mesh_vertex_offset.release();
    c->mesh_index_offset.release();
    c->mesh_tri_base.release();
    c->inst_mesh.release();
    c->dinst.release();
    c->nodes.release();
    c->nodes4.release();
    c->tris.release();
    c->mesh_root.release();
    c->image.release();
    c->sum64.release();
    c->counters.release();
    c->error_word.release();
    c->mse_ref.release();
    c->mse_partial.release();
    c->wave_state.release();
    for (int k = 0; k < pt::MAX_WAVE_WAYS; k++) {
        c->wave_state_x[k].release();
        if (c->side[k])
            cudaStreamDestroy(c->side[k]);
        if (c->wave_join[k])
            cudaEventDestroy(c->wave_join[k]);
        if (c->wave_acc[k])
            cudaEventDestroy(c->wave_acc[k]);
    }
    if (c->wave_fork)
        cudaEventDestroy(c->wave_fork);
    c->texels.release();
    c->textures.release();
    c->feat_a.release();
    c->feat_n.release();
    c->denoised.release();
    c->half.release();
    pt::batch_free(c->batch);
    c->batch = nullptr;
    for (cudaEvent_t ev : c->stage_events)
        cudaEventDestroy(ev);
    c->stage_events.clear();
    if (c->ev0)
        cudaEventDestroy(c->ev0);
    if (c->ev1)
        cudaEventDestroy(c->ev1);
    if (c->stream)
        cudaStreamDestroy(c->stream);
    delete c;
}

const char* pt_last_error(const pt_ctx* c)
{
    if (!c)
        return g_create_error.c_str();
    return c->err.c_str();
}

int pt_synchronize(pt_ctx* c)
{
    if (!c)
        return PT_ERR_INVALID;
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess)
        return c->cuda_fail(e, "synchronize");
    return PT_OK;
}

int pt_upload_scene(pt_ctx* c, const pt_scene_view* v)
{
    if (!c || !v)
        return PT_ERR_INVALID;
    cudaSetDevice(c->device);
    c->scene_ok = false;
    c->accel_ok = false;
    c->scene_generation++;
    if ((v->vertex_count && !v->vertices) || (v->index_count && !v->indices) || (v->mesh_count && !v->meshes) ||
        (v->instance_count && (!v->instances || !v->instance_mesh)) || (v->material_count && !v->materials) ||
        (v->light_word_count && !v->light_words))
        return c->fail(PT_ERR_INVALID, "scene view has a null array with a non-zero count");
    if (v->index_count % 3 != 0)
        return c->fail(PT_ERR_INVALID, "index count is not a multiple of 3");
    if (v->mesh_count >= 65536)
        return c->fail(PT_ERR_UNSUPPORTED, "more than 65535 meshes");
    if (v->light_count > 0 && v->light_word_count < v->light_count * PT_LIGHT_BIN_SIZE)
        return c->fail(PT_ERR_INVALID, "light stream shorter than its top-level table");
    // meshes
    // non-finite positions would give the BVH build NaN boxes (no consistent
    // merge order) and the light tables NaN weights: rejected up front
    for (uint64_t i = 0; i < v->vertex_count; i++) {
        const float* f = v->vertices + i * PT_VERTEX_FLOATS;
        if (!std::isfinite(f[0]) || !std::isfinite(f[1]) || !std::isfinite(f[2]))
            return c->fail(PT_ERR_INVALID, "vertex " + std::to_string(i) + " has a non-finite position");
    }
    std::vector<uint32_t> vo(v->mesh_count), io(v->mesh_count), tb(v->mesh_count + 1);
    uint64_t tris = 0;
    for (uint32_t m = 0; m < v->mesh_count; m++) {
        const pt_mesh_range& r = v->meshes[m];
        if ((uint64_t)r.vertex_offset + r.vertex_count > v->vertex_count || (uint64_t)r.index_offset + 3ull * r.tri_count > v->index_count)
            return c->fail(PT_ERR_INVALID, "mesh " + std::to_string(m) + " range outside the vertex/index arrays");
        for (uint64_t k = 0; k < 3ull * r.tri_count; k++)
            if (v->indices[r.index_offset + k] >= r.vertex_count)
                return c->fail(PT_ERR_INVALID, "mesh " + std::to_string(m) + " has an index outside its vertices");
        vo[m] = r.vertex_offset;
        io[m] = r.index_offset;
        tb[m] = (uint32_t)tris;
        tris += r.tri_count;
    }
    if (tris >= (1u << 28))
        return c->fail(PT_ERR_UNSUPPORTED, "more than 2^28 triangles");
    tb[v->mesh_count] = (uint32_t)tris;
    if (v->instance_count >= (1u << 28))
        return c->fail(PT_ERR_UNSUPPORTED, "more than 2^28 instances");
    // textures: every texel of every texture inside the texel array
    if (v->texture_count && (!v->textures || !v->texels))
        return c->fail(PT_ERR_INVALID, "textures without texel data");
    for (uint32_t i = 0; i < v->texture_count; i++) {
        const pt_texture& t = v->textures[i];
        if (t.width == 0 || t.height == 0 || t.width > (1u << 16) || t.height > (1u << 16) ||
            !(t.channels == 1 || t.channels == 2 || t.channels == 4) ||
            t.offset + (uint64_t)t.width * t.height * t.channels > v->texel_bytes)
            return c->fail(PT_ERR_INVALID, "texture " + std::to_string(i) + " is malformed");
    }
    if (v->material_ior)
        for (uint32_t i = 0; i < v->material_count; i++) {
            const float n = v->material_ior[i];
            if (!(n == 0.0f || (n >= 1.0f && std::isfinite(n))))
                return c->fail(PT_ERR_INVALID, "material " + std::to_string(i) + ": index of refraction must be 0 or >= 1");
        }
    // instances
    c->h_dinst.assign(v->instance_count, DevInstance{});
    for (uint32_t i = 0; i < v->instance_count; i++) {
        const pt_instance_data& d = v->instances[i];
        uint32_t m = v->instance_mesh[i];
        if (m >= v->mesh_count)
            return c->fail(PT_ERR_INVALID, "instance " + std::to_string(i) + " names a missing mesh");
        if (d.material_index >= v->material_count)
            return c->fail(PT_ERR_INVALID, "instance " + std::to_string(i) + " names a missing material");
        if (d.vertex_index != v->meshes[m].vertex_offset || d.index_index != v->meshes[m].index_offset)
            return c->fail(PT_ERR_INVALID, "instance " + std::to_string(i) + " offsets disagree with its mesh");
        DevInstance& di = c->h_dinst[i];
        float w[12];
        if (v->instance_world_to_object) {
            std::memcpy(w, v->instance_world_to_object + 12 * (size_t)i, sizeof(w));
        } else {
            double M[16], inv[16];
            for (int r = 0; r < 4; r++)
                for (int k = 0; k < 4; k++)
                    M[r * 4 + k] = d.transform[r][k];
            inverse4(M, inv);
            for (int k = 0; k < 12; k++)
                w[k] = (float)inv[k];
        }
        for (int r = 0; r < 3; r++)
            di.w2o[r] = make_float4(w[4 * r + 0], w[4 * r + 1], w[4 * r + 2], w[4 * r + 3]);
        di.blas_root = REF_EMPTY;
        di.flags = (v->instance_opaque == nullptr || v->instance_opaque[i]) ? 1u : 0u;
        di.mesh = m;
    }
    cudaError_t e;
    static_assert(sizeof(DevInstanceData) == sizeof(pt_instance_data), "InstanceData layout");
    static_assert(sizeof(DevMaterial) == sizeof(pt_material), "PbrMaterial layout");
    static_assert(sizeof(DevTexture) == sizeof(pt_texture), "texture descriptor layout");
    if ((e = upload(c, c->vertices, (const float4*)v->vertices, 2 * (size_t)v->vertex_count)) != cudaSuccess ||
        (e = upload(c, c->indices, v->indices, v->index_count)) != cudaSuccess ||
        (e = upload(c, c->inst_data, (const DevInstanceData*)v->instances, v->instance_count)) != cudaSuccess ||
        (e = upload(c, c->materials, (const DevMaterial*)v->materials, v->material_count)) != cudaSuccess ||
        (e = upload(c, c->material_ior, v->material_ior, v->material_ior ? v->material_count : 0)) != cudaSuccess ||
        (e = upload(c, c->light, v->light_words, v->light_word_count)) != cudaSuccess ||
        (e = upload(c, c->mesh_vertex_offset, vo.data(), vo.size())) != cudaSuccess ||
        (e = upload(c, c->mesh_index_offset, io.data(), io.size())) != cudaSuccess ||
        (e = upload(c, c->mesh_tri_base, tb.data(), tb.size())) != cudaSuccess ||
        (e = upload(c, c->inst_mesh, v->instance_mesh, v->instance_count)) != cudaSuccess ||
        (e = upload(c, c->dinst, c->h_dinst.data(), c->h_dinst.size())) != cudaSuccess ||
        (e = upload(c, c->texels, v->texels, (size_t)v->texel_bytes)) != cudaSuccess ||
        (e = upload(c, c->textures, (const DevTexture*)v->textures, v->texture_count)) != cudaSuccess)
        return c->cuda_fail(e, "scene upload");
    if ((e = cudaStreamSynchronize(c->stream)) != cudaSuccess)
        return c->cuda_fail(e, "scene upload");
    c->vertex_count = v->vertex_count;
    c->index_count = v->index_count;
    c->mesh_count = v->mesh_count;
    c->tri_count = (uint32_t)tris;
    c->instance_count = v->instance_count;
    c->material_count = v->material_count;
    c->has_ior = v->material_ior != nullptr && v->material_count != 0;
    c->texture_count = v->texture_count;
    c->light_words = v->light_word_count;
    c->light_count = v->light_count;
    std::memcpy(c->env, v->environment_colour, sizeof(c->env));
    c->scene_ok = true;
    return PT_OK;
}

int pt_build_accel(pt_ctx* c, pt_accel_info* info)
{
    if (!c)
        return PT_ERR_INVALID;
    if (!c->scene_ok)
        return c->fail(PT_ERR_STATE, "no scene uploaded");
    cudaSetDevice(c->device);
    cudaError_t e;
    size_t n_nodes = bvh_node_count(c->tri_count, c->instance_count);
    const bool wide = use_bvh4();
    if (!wide)
        c->nodes4.release();
    if ((e = c->nodes.alloc(n_nodes)) != cudaSuccess || (e = c->tris.alloc(c->tri_count)) != cudaSuccess ||
        (e = c->mesh_root.alloc(c->mesh_count)) != cudaSuccess || (wide && (e = c->nodes4.alloc(n_nodes)) != cudaSuccess))
        return c->cuda_fail(e, "acceleration structure allocation");
    size_t scratch_bytes = bvh_scratch_bytes(c->mesh_count, c->tri_count, c->instance_count);
    scratch_bytes = (scratch_bytes + 15) & ~(size_t)15;
    void* scratch = nullptr;
    // the scratch plus one word: set when a 4-wide node's half planes overflow
    if ((e = cudaMalloc(&scratch, scratch_bytes + 16)) != cudaSuccess)
        return c->cuda_fail(e, "BVH scratch allocation");
    uint32_t* overflow = reinterpret_cast<uint32_t*>(static_cast<char*>(scratch) + scratch_bytes);
    BvhBuildInput in{};
    in.vertices = c->vertices.p;
    in.indices = c->indices.p;
    in.mesh_vertex_offset = c->mesh_vertex_offset.p;
    in.mesh_index_offset = c->mesh_index_offset.p;
    in.mesh_tri_base = c->mesh_tri_base.p;
    in.mesh_count = c->mesh_count;
    in.tri_count = c->tri_count;
    in.inst_data = c->inst_data.p;
    in.inst_mesh = c->inst_mesh.p;
    in.instance_count = c->instance_count;
    BvhBuildOutput out{};
    out.nodes = c->nodes.p;
    out.tris = c->tris.p;
    out.dinst = c->dinst.p;
    out.mesh_root = c->mesh_root.p;
    cudaEventRecord(c->ev0, c->stream);
    // node slots no tree uses stay zero (finite boxes for the 4-wide view)
    e = cudaMemsetAsync(c->nodes.p, 0, n_nodes * sizeof(BvhNode), c->stream);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(overflow, 0, sizeof(uint32_t), c->stream);
    if (e == cudaSuccess)
        e = bvh_build(in, out, scratch, scratch_bytes, c->stream);
    if (e == cudaSuccess && wide)
        e = build_bvh4(c->nodes.p, (uint32_t)n_nodes, c->nodes4.p, overflow, c->stream);
    cudaEventRecord(c->ev1, c->stream);
    cudaError_t e2 = cudaStreamSynchronize(c->stream);
    uint32_t overflowed = 0;
    if (e == cudaSuccess && e2 == cudaSuccess && wide)
        e2 = cudaMemcpy(&overflowed, overflow, sizeof(uint32_t), cudaMemcpyDeviceToHost);
    cudaFree(scratch);
    if (e != cudaSuccess)
        return c->cuda_fail(e, "BVH build");
    if (e2 != cudaSuccess)
        return c->cuda_fail(e2, "BVH build");
    // coordinates beyond the half range: traverse the full-precision BVH2
    if (overflowed)
        c->nodes4.release();
    const bool wide_used = wide && !overflowed;
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    c->tlas_root = out.tlas_root;
    const char* validate = std::getenv("PT_VALIDATE_BVH");
    if (validate && validate[0] == '1') {
        std::vector<uint32_t> tb(c->mesh_count + 1);
        cudaMemcpy(tb.data(), c->mesh_tri_base.p, tb.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost);
        std::string problem = validate_accel(c, tb);
        if (!problem.empty())
            return c->fail(PT_ERR_DEVICE, "BVH validation: " + problem);
    }
    c->accel_ok = true;
    c->scene_generation++;
    c->accel.blas_count = c->mesh_count;
    c->accel.tlas_nodes = c->instance_count > 1 ? c->instance_count - 1 : 0;
    c->accel.blas_nodes = c->tri_count > 1 ? c->tri_count - 1 : 0;
    c->accel.triangles = c->tri_count;
    c->accel.device_bytes = n_nodes * sizeof(BvhNode) + (wide_used ? n_nodes * sizeof(Bvh4Node) : 0) +
                            (size_t)c->tri_count * sizeof(TriRec) + (size_t)c->instance_count * sizeof(DevInstance);
    c->accel.build_ms = ms;
    if (info)
        *info = c->accel;
    return PT_OK;
}

static int ensure_image(pt_ctx* c, uint32_t w, uint32_t h, bool fp64, bool reset)
{
    cudaError_t e;
    size_t n = (size_t)w * h;
    if (c->width != w || c->height != h || !c->image.p) {
        if ((e = c->image.alloc(n)) != cudaSuccess)
            return c->cuda_fail(e, "image allocation");
        c->width = w;
        c->height = h;
        c->sum64.release();
        reset = true;
    }
    if (fp64 && !c->sum64.p) {
        if ((e = c->sum64.alloc(4 * n)) != cudaSuccess)
            return c->cuda_fail(e, "FP64 image allocation");
        cudaMemsetAsync(c->sum64.p, 0, 4 * n * sizeof(double), c->stream);
    }
    if (reset) {
        cudaMemsetAsync(c->image.p, 0, n * sizeof(float4), c->stream);
        if (c->sum64.p)
            cudaMemsetAsync(c->sum64.p, 0, 4 * n * sizeof(double), c->stream);
        c->samples_done = 0;
    }
    return PT_OK;
}

} // extern "C"

// Device view of the context's scene and the camera/image of `p`.
RenderArgs render_args(const pt_ctx* c, const pt_render_params* p, bool fp64)
{
    RenderArgs a{};
    a.s.vertices = c->vertices.p;
    a.s.indices = c->indices.p;
    a.s.inst_data = c->inst_data.p;
    a.s.materials = c->materials.p;
    a.s.material_ior = c->has_ior ? c->material_ior.p : nullptr;
    a.s.light = c->light.p;
    a.s.light_words = c->light_words;
    a.s.light_count = c->light_count;
    a.s.instance_count = c->instance_count;
    a.s.vertex_count = c->vertex_count;
    a.s.texels = c->texels.p;
    a.s.textures = c->textures.p;
    a.s.texture_count = c->texture_count;
    // A traversal of a valid BVH visits each node at most once; the cap only
    // stops a malformed tree from spinning.
    a.s.max_iterations = 4u * (uint32_t)std::min<size_t>(c->nodes.n + c->tri_count + c->instance_count, 1u << 28) + 4096u;
    // PT_TRAVERSAL_CAP lowers the cap (tests make the watchdog fire with it: a
    // traversal that reaches the cap stops and reports PT_ERR_TIMEOUT)
    static const uint32_t cap = [] {
        const char* e = std::getenv("PT_TRAVERSAL_CAP");
        return e ? (uint32_t)std::max(1, std::atoi(e)) : 0u;
    }();
    if (cap)
        a.s.max_iterations = std::min(a.s.max_iterations, cap);
    a.s.nodes = c->nodes.p;
    a.s.nodes4 = c->nodes4.p;
    a.s.tris = c->tris.p;
    a.s.node_count = (uint32_t)c->nodes.n;
    a.s.tri_count = c->tri_count;
    a.s.index_count = c->index_count;
    a.s.dinst = c->dinst.p;
    a.s.tlas_root = c->tlas_root;
    a.s.env = mk3(c->env[0], c->env[1], c->env[2]);
    a.s.error_word = c->error_word.p;
    std::memcpy(a.inv_view, p->inv_view, sizeof(a.inv_view));
    std::memcpy(a.inv_proj, p->inv_proj, sizeof(a.inv_proj));
    a.near_plane = p->near_plane;
    a.far_plane = p->far_plane;
    a.focus_dist = p->focus_dist;
    a.lens_radius = p->lens_radius;
    a.exposure = p->exposure;
    a.width = p->width;
    a.height = p->height;
    a.max_bounces = p->max_bounces;
    a.rr_start = p->rr_start == 0 ? 1 : p->rr_start;
    a.image = c->image.p;
    a.sum64 = fp64 ? c->sum64.p : nullptr;
    a.counters = c->counters.p;
    return a;
}

extern "C" {

int pt_render(pt_ctx* c, const pt_render_params* p, pt_render_stats* stats)
{
    if (!c || !p)
        return PT_ERR_INVALID;
    if (!c->accel_ok)
        return c->fail(PT_ERR_STATE, "acceleration structure not built");
    if (p->width == 0 || p->height == 0 || p->samples == 0)
        return c->fail(PT_ERR_INVALID, "zero width, height or sample count");
    if ((uint64_t)p->width * p->height > (1ull << 31))
        return c->fail(PT_ERR_UNSUPPORTED, "image larger than 2^31 pixels");
    if ((uint64_t)p->sample_index + p->samples > 0xFFFFFFFFull)
        return c->fail(PT_ERR_INVALID, "sample index overflows 32 bits");
    if (p->accum_mode > PT_ACCUM_FP32_FP64 || p->kernel > PT_KERNEL_WAVEFRONT)
        return c->fail(PT_ERR_INVALID, "unknown accumulation mode or kernel");
    cudaSetDevice(c->device);
    bool fp64 = p->accum_mode == PT_ACCUM_FP32_FP64;
    if (p->flags & ~(PT_RENDER_FEATURES | PT_RENDER_TIME_STAGES | PT_RENDER_FEATURES_FP16 | PT_RENDER_RESTART))
        return c->fail(PT_ERR_INVALID, "unknown render flags");
    const bool restart = p->sample_index == 0 || (p->flags & PT_RENDER_RESTART) != 0;
    // FP64 sums that continue a progression must hold every earlier sample:
    // after an FP32-only chunk (or a restore without sums) they do not.
    const bool continues = !restart && c->image.p && c->width == p->width && c->height == p->height;
    if (fp64 && continues && !c->have_fp64)
        return c->fail(PT_ERR_STATE, "FP64 sums requested for a continued render whose earlier samples have none "
                                     "(restart it, or keep FP64 sums from its first sample)");
    int rc = ensure_image(c, p->width, p->height, fp64, restart);
    if (rc != PT_OK)
        return rc;
    if (restart)
        c->image_epoch++;
    RenderArgs a = render_args(c, p, fp64);
    const bool features = (p->flags & PT_RENDER_FEATURES) != 0;
    a.fp16_features = (p->flags & PT_RENDER_FEATURES_FP16) ? 1u : 0u;
    if (features) {
        const size_t px = (size_t)p->width * p->height;
        if (c->feat_a.n < px) {
            cudaError_t e = c->feat_a.alloc(px);
            if (e == cudaSuccess)
                e = c->feat_n.alloc(px);
            if (e != cudaSuccess)
                return c->cuda_fail(e, "feature buffers");
        }
        a.feat_a = c->feat_a.p;
        a.feat_n = c->feat_n.p;
    }
    // an armed snapshot is taken inside this render when its sample range reaches it
    const bool snap = c->snapshot_armed > p->sample_index && c->snapshot_armed <= p->sample_index + p->samples;
    if (snap) {
        const size_t px = (size_t)p->width * p->height;
        if (c->half.n < px) {
            cudaError_t e = c->half.alloc(px);
            if (e != cudaSuccess)
                return c->cuda_fail(e, "snapshot buffer");
        }
        a.snapshot = c->half.p;
        a.snapshot_after = c->snapshot_armed;
    }
    cudaMemsetAsync(c->counters.p, 0, 8 * sizeof(unsigned long long), c->stream);
    cudaMemsetAsync(c->error_word.p, 0, sizeof(uint32_t), c->stream); // errors belong to this render
    const bool timing = (p->flags & PT_RENDER_TIME_STAGES) != 0;
    uint32_t stage_marks = 0;
    uint64_t pixels = (uint64_t)p->width * p->height;
    uint32_t kernel = p->kernel == PT_KERNEL_MEGA ? PT_KERNEL_MEGA : PT_KERNEL_WAVEFRONT;
    uint32_t launches = 0;
    int ways = 1;        // sub-waves in flight
    uint64_t wave_k = 1; // samples per wave
    if (kernel == PT_KERNEL_WAVEFRONT) {
        // Waves of k samples, k * pixels paths (at least one sample), at most
        // 2^n paths, n = PT_WAVE_PATHS_LOG2 (20..27, default 26: up to 15.6 GB
        // of path state), and at most a quarter of the device memory free now
        // (counting this context's current state), so that many contexts
        // shrink their waves instead of running out of memory.  Bigger waves
        // keep the late segments' queues large: on the mid scene at 1024² x
        // 128 spp, 2^23 / 2^25 / 2^26 / 2^27 paths gave 1,075 / 1,276 /
        // 1,320 / 1,344 Mpath-segs/s.
        static const int wave_log2 = [] {
            const char* e = std::getenv("PT_WAVE_PATHS_LOG2");
            const int v = e ? std::atoi(e) : 26;
            return v < 20 ? 20 : (v > 27 ? 27 : v);
        }();
        // Sub-waves in flight (PT_WAVE_STREAMS, 1-4, default 2): the samples
        // are split over that many path states, each at most 1/(4 x ways) of
        // the free memory, run on as many streams.  Not with stage timing
        // (one stream of events), nor with FP16 features: their running means
        // are stored rounded after every wave, and one wave keeps them the
        // FP32 means rounded once.
        static const int ways_env = [] {
            const char* e = std::getenv("PT_WAVE_STREAMS");
            const int v = e ? std::atoi(e) : 2;
            return v < 1 ? 1 : (v > pt::MAX_WAVE_WAYS ? pt::MAX_WAVE_WAYS : v);
        }();
        ways = (timing || (p->flags & PT_RENDER_FEATURES_FP16)) ? 1 : (int)std::min<uint64_t>(ways_env, p->samples);
        uint64_t cap = 1ull << wave_log2;
        size_t free_b = 0, total_b = 0;
        if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess) {
            const uint64_t per_path = wave_state_bytes(1u << 20) >> 20;
            uint64_t avail = (uint64_t)free_b + (uint64_t)c->wave_state.n;
            for (int k = 1; k < pt::MAX_WAVE_WAYS; k++)
                avail += (uint64_t)c->wave_state_x[k].n;
            cap = std::min<uint64_t>(cap, std::max<uint64_t>(avail / (4 * (uint64_t)ways) / per_path, 1));
        }
        const uint64_t per_state = (p->samples + ways - 1) / ways;
        uint64_t k = std::max<uint64_t>(1, std::min<uint64_t>(per_state, cap / pixels));
        uint64_t n = k * pixels;
        if (c->wave_paths < n) {
            c->wave_state.release();
            cudaError_t e = c->wave_state.alloc(wave_state_bytes((uint32_t)n));
            if (e != cudaSuccess) {
                c->wave_paths = 0;
                return c->cuda_fail(e, "wavefront state allocation");
            }
            c->wave_paths = (uint32_t)n;
        }
        for (int k = 1; k < ways; k++) {
            if (c->wave_paths_x[k] < n) {
                c->wave_state_x[k].release();
                cudaError_t e = c->wave_state_x[k].alloc(wave_state_bytes((uint32_t)n));
                if (e != cudaSuccess) {
                    c->wave_paths_x[k] = 0;
                    return c->cuda_fail(e, "wavefront state allocation");
                }
                c->wave_paths_x[k] = (uint32_t)n;
            }
            cudaError_t e = cudaSuccess;
            if (!c->side[k])
                e = cudaStreamCreateWithFlags(&c->side[k], cudaStreamNonBlocking);
            if (e == cudaSuccess && !c->wave_join[k])
                e = cudaEventCreateWithFlags(&c->wave_join[k], cudaEventDisableTiming);
            if (e != cudaSuccess)
                return c->cuda_fail(e, "sub-wave stream");
        }
        if (ways > 1) {
            cudaError_t e = cudaSuccess;
            if (!c->wave_fork)
                e = cudaEventCreateWithFlags(&c->wave_fork, cudaEventDisableTiming);
            for (int k = 0; k < ways && e == cudaSuccess; k++)
                if (!c->wave_acc[k])
                    e = cudaEventCreateWithFlags(&c->wave_acc[k], cudaEventDisableTiming);
            if (e != cudaSuccess)
                return c->cuda_fail(e, "sub-wave events");
        }
        wave_k = k;
    }
    cudaEventRecord(c->ev0, c->stream);
    if (kernel == PT_KERNEL_MEGA) {
        // Split long renders so no single launch covers more than 2^26 path samples.
        uint32_t per_launch = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(p->samples, (1ull << 26) / pixels));
        for (uint32_t done = 0; done < p->samples; done += per_launch) {
            a.sample_index = p->sample_index + done;
            a.samples = std::min(per_launch, p->samples - done);
            cudaError_t e = launch_megakernel(a, c->stream);
            if (e != cudaSuccess)
                return c->cuda_fail(e, "render launch");
            launches++;
        }
    } else {
        a.sample_index = p->sample_index;
        a.samples = p->samples;
        uint32_t n_paths = (uint32_t)(wave_k * pixels);
        StageTimer timer;
        if (timing) {
            // waves x ((bounces + 1) x 4 + 2) launches, one event before each and one at the end
            const uint64_t waves = (p->samples + n_paths / pixels - 1) / (n_paths / pixels);
            const uint64_t need = waves * ((uint64_t)(p->max_bounces + 1) * 4 + 3);
            if (need > (1u << 20))
                return c->fail(PT_ERR_UNSUPPORTED, "too many launches to time by stage");
            while (c->stage_events.size() < need) {
                cudaEvent_t ev;
                cudaError_t ee = cudaEventCreate(&ev);
                if (ee != cudaSuccess)
                    return c->cuda_fail(ee, "stage timing events");
                c->stage_events.push_back(ev);
            }
            c->stage_of.resize(c->stage_events.size());
            timer.events = c->stage_events.data();
            timer.stage = c->stage_of.data();
            timer.capacity = (uint32_t)c->stage_events.size();
        }
        WaveMulti wm{};
        wm.ways = ways;
        wm.fork = c->wave_fork;
        for (int k = 0; k < ways; k++) {
            wm.state[k] = k ? c->wave_state_x[k].p : c->wave_state.p;
            wm.state_bytes[k] = k ? c->wave_state_x[k].n : c->wave_state.n;
            wm.stream[k] = k ? c->side[k] : c->stream;
            wm.join[k] = c->wave_join[k];
            wm.acc[k] = c->wave_acc[k];
        }
        cudaError_t e = launch_wavefront(a, c->wave_state.p, c->wave_state.n, n_paths, c->sm_count, &launches, c->stream,
                                         timing ? &timer : nullptr, ways > 1 ? &wm : nullptr);
        if (e != cudaSuccess)
            return c->cuda_fail(e, "wavefront launch");
        stage_marks = timer.count;
    }
    cudaEventRecord(c->ev1, c->stream);
    c->samples_done = p->sample_index + p->samples;
    c->have_fp64 = fp64;
    if (features) {
        c->feat_w = p->width;
        c->feat_h = p->height;
        c->feat_fp16 = a.fp16_features != 0;
    }
    if (snap) {
        c->half_fp16 = a.fp16_features != 0;
        c->half_w = p->width;
        c->half_h = p->height;
        c->half_spp = c->snapshot_armed;
        c->half_epoch = c->image_epoch;
        c->snapshot_armed = 0;
    }
    if (stats) {
        cudaError_t e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess)
            return c->cuda_fail(e, "render");
        unsigned long long cnt[8];
        uint32_t ew = 0;
        cudaMemcpy(cnt, c->counters.p, sizeof(cnt), cudaMemcpyDeviceToHost);
        cudaMemcpy(&ew, c->error_word.p, sizeof(ew), cudaMemcpyDeviceToHost);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, c->ev0, c->ev1);
        stats->segments = cnt[0];
        stats->shadow_rays = cnt[1];
        stats->paths = cnt[2];
        stats->node_visits = cnt[3];
        stats->tri_tests = cnt[4];
        stats->milliseconds = ms;
        stats->kernel_launches = launches;
        stats->kernel_used = kernel;
        stats->error_word = ew;
        for (int k = 0; k < STAGE_COUNT; k++)
            stats->stage_ms[k] = 0.0f;
        stats->stage_launches = 0;
        for (uint32_t i = 0; i + 1 < stage_marks; i++) {
            const uint8_t sg = c->stage_of[i];
            if (sg >= STAGE_COUNT)
                continue;
            float t = 0.0f;
            cudaEventElapsedTime(&t, c->stage_events[i], c->stage_events[i + 1]);
            stats->stage_ms[sg] += t;
            stats->stage_launches += sg == 1 ? 1u : 0u;
        }
        if (ew != 0)
            return c->fail((ew & ERR_WATCHDOG) ? PT_ERR_TIMEOUT : PT_ERR_DEVICE,
                          std::string((ew & ERR_WATCHDOG)      ? "traversal iteration cap hit"
                                      : (ew & ERR_BAD_INDEX) ? "index out of range (checked build)"
                                                              : "device error") +
                              " (error word " + std::to_string(ew) + ")");
    }
    return PT_OK;
}

int pt_debug_poke_tlas_link(pt_ctx* c, int value)
{
    if (!c)
        return PT_ERR_INVALID;
#ifndef PT_CHECKED
    (void)value;
    return c->fail(PT_ERR_UNSUPPORTED, "fault injection needs the bounds-checked build (libptgpu_checked.so)");
#else
    if (!c->accel_ok)
        return c->fail(PT_ERR_STATE, "no acceleration structure");
    if (c->tlas_root < 0)
        return c->fail(PT_ERR_STATE, "the TLAS has no node");
    cudaSetDevice(c->device);
    cudaError_t e;
    if (c->nodes4.p)
        e = cudaMemcpy(&c->nodes4.p[c->tlas_root].link.x, &value, sizeof(int), cudaMemcpyHostToDevice);
    else
        e = cudaMemcpy(&c->nodes.p[c->tlas_root].link.x, &value, sizeof(int), cudaMemcpyHostToDevice);
    return e == cudaSuccess ? PT_OK : c->cuda_fail(e, "fault injection");
#endif
}

int pt_restore_image(pt_ctx* c, const float* rgba, size_t pitch, const double* sums64, uint32_t width, uint32_t height,
                     uint32_t samples_done)
{
    if (!c || !rgba || width == 0 || height == 0 || samples_done == 0)
        return PT_ERR_INVALID;
    if ((uint64_t)width * height > (1ull << 31))
        return c->fail(PT_ERR_UNSUPPORTED, "image larger than 2^31 pixels");
    if (pitch < (size_t)width * 16)
        return c->fail(PT_ERR_INVALID, "pitch smaller than a row");
    cudaSetDevice(c->device);
    if (!sums64)
        c->sum64.release(); // no stale sums behind a restored FP32-only image
    int rc = ensure_image(c, width, height, sums64 != nullptr, false);
    if (rc != PT_OK)
        return rc;
    cudaError_t e = cudaMemcpy2DAsync(c->image.p, (size_t)width * 16, rgba, pitch, (size_t)width * 16, height,
                                      cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess && sums64)
        e = cudaMemcpyAsync(c->sum64.p, sums64, (size_t)width * height * 4 * sizeof(double), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess)
        return c->cuda_fail(e, "image restore");
    c->samples_done = samples_done;
    c->have_fp64 = sums64 != nullptr;
    c->image_epoch++;
    return PT_OK;
}

int pt_set_camera(pt_ctx* c, const pt_render_params* p)
{
    if (!c || !p)
        return PT_ERR_INVALID;
    if (p->width == 0 || p->height == 0)
        return c->fail(PT_ERR_INVALID, "zero width or height");
    c->camera = *p;
    c->camera_set = true;
    c->next_sample = 0;
    return PT_OK;
}

int pt_render_next(pt_ctx* c, uint32_t samples, pt_render_stats* stats)
{
    if (!c)
        return PT_ERR_INVALID;
    if (!c->camera_set)
        return c->fail(PT_ERR_STATE, "no camera set (pt_set_camera)");
    pt_render_params p = c->camera;
    p.sample_index = c->next_sample;
    p.samples = samples;
    int rc = pt_render(c, &p, stats);
    if (rc == PT_OK)
        c->next_sample += samples;
    return rc;
}

int pt_read_image(pt_ctx* c, void* rgba, size_t pitch, int fp64)
{
    if (!c || !rgba)
        return PT_ERR_INVALID;
    if (!c->image.p)
        return c->fail(PT_ERR_STATE, "nothing rendered");
    cudaSetDevice(c->device);
    cudaError_t e;
    if (fp64 == PT_IMAGE_DENOISED) {
        if (!c->denoised.p || c->feat_w != c->width || c->feat_h != c->height)
            return c->fail(PT_ERR_STATE, "no denoised image (call pt_denoise)");
        if (pitch < (size_t)c->width * 16)
            return c->fail(PT_ERR_INVALID, "pitch smaller than a row");
        e = cudaMemcpy2DAsync(rgba, pitch, c->denoised.p, (size_t)c->width * 16, (size_t)c->width * 16, c->height,
                              cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(c->stream);
        return e == cudaSuccess ? PT_OK : c->cuda_fail(e, "denoised read-back");
    }
    if (!fp64) {
        if (pitch < (size_t)c->width * 16)
            return c->fail(PT_ERR_INVALID, "pitch smaller than a row");
        e = cudaMemcpy2DAsync(rgba, pitch, c->image.p, (size_t)c->width * 16, (size_t)c->width * 16, c->height, cudaMemcpyDeviceToHost,
                              c->stream);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess)
            return c->cuda_fail(e, "image read-back");
        return PT_OK;
    }
    if (fp64 != 1 && fp64 != PT_IMAGE_SUMS64)
        return c->fail(PT_ERR_INVALID, "unknown image kind");
    if (!c->sum64.p || !c->have_fp64)
        return c->fail(PT_ERR_STATE, "no FP64 accumulation (render with PT_ACCUM_FP32_FP64)");
    if (pitch < (size_t)c->width * 32)
        return c->fail(PT_ERR_INVALID, "pitch smaller than a row");
    if (fp64 == PT_IMAGE_SUMS64) {
        e = cudaMemcpy2DAsync(rgba, pitch, c->sum64.p, (size_t)c->width * 32, (size_t)c->width * 32, c->height,
                              cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(c->stream);
        return e == cudaSuccess ? PT_OK : c->cuda_fail(e, "FP64 sums read-back");
    }
    size_t n = (size_t)c->width * c->height;
    std::vector<double> sums(4 * n);
    e = cudaMemcpyAsync(sums.data(), c->sum64.p, 4 * n * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess)
        return c->cuda_fail(e, "FP64 read-back");
    for (uint32_t y = 0; y < c->height; y++) {
        double* row = (double*)((char*)rgba + pitch * y);
        for (uint32_t x = 0; x < c->width; x++) {
            const double* s = &sums[4 * ((size_t)y * c->width + x)];
            double cnt = s[3] > 0.0 ? s[3] : 1.0;
            row[4 * x + 0] = s[0] / cnt;
            row[4 * x + 1] = s[1] / cnt;
            row[4 * x + 2] = s[2] / cnt;
            row[4 * x + 3] = 1.0;
        }
    }
    return PT_OK;
}

int pt_render_features(pt_ctx* c, const pt_render_params* p)
{
    if (!c || !p)
        return PT_ERR_INVALID;
    if (!c->accel_ok)
        return c->fail(PT_ERR_STATE, "acceleration structure not built");
    if (p->width == 0 || p->height == 0 || p->samples == 0)
        return c->fail(PT_ERR_INVALID, "zero width, height or sample count");
    if ((uint64_t)p->width * p->height > (1ull << 31) || (uint64_t)p->sample_index + p->samples > 0xFFFFFFFFull)
        return c->fail(PT_ERR_INVALID, "image or sample range too large");
    cudaSetDevice(c->device);
    const size_t pixels = (size_t)p->width * p->height;
    if (c->feat_a.n < pixels) {
        cudaError_t e = c->feat_a.alloc(pixels);
        if (e == cudaSuccess)
            e = c->feat_n.alloc(pixels);
        if (e != cudaSuccess)
            return c->cuda_fail(e, "feature buffers");
    }
    if (p->flags & ~PT_RENDER_FEATURES_FP16)
        return c->fail(PT_ERR_INVALID, "unknown flags for the feature pass");
    RenderArgs a = render_args(c, p, false);
    a.sample_index = p->sample_index;
    a.samples = p->samples;
    a.fp16_features = (p->flags & PT_RENDER_FEATURES_FP16) ? 1u : 0u;
    cudaError_t e = launch_features(a, c->feat_a.p, c->feat_n.p, c->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess)
        return c->cuda_fail(e, "feature pass");
    c->feat_w = p->width;
    c->feat_h = p->height;
    c->feat_fp16 = a.fp16_features != 0;
    return PT_OK;
}

int pt_denoise_snapshot(pt_ctx* c)
{
    if (!c)
        return PT_ERR_INVALID;
    if (!c->image.p || c->samples_done == 0)
        return c->fail(PT_ERR_STATE, "nothing rendered");
    cudaSetDevice(c->device);
    const size_t pixels = (size_t)c->width * c->height;
    if (c->half.n < pixels) {
        cudaError_t e = c->half.alloc(pixels);
        if (e != cudaSuccess)
            return c->cuda_fail(e, "snapshot buffer");
    }
    cudaError_t e = cudaMemcpyAsync(c->half.p, c->image.p, pixels * sizeof(float4), cudaMemcpyDeviceToDevice, c->stream);
    if (e != cudaSuccess)
        return c->cuda_fail(e, "snapshot");
    c->half_fp16 = false;
    c->half_w = c->width;
    c->half_h = c->height;
    c->half_spp = c->samples_done;
    c->half_epoch = c->image_epoch;
    return PT_OK;
}

int pt_read_features(pt_ctx* c, float* albedo_depth, float* normal)
{
    if (!c)
        return PT_ERR_INVALID;
    if (!c->feat_a.p || c->feat_w == 0)
        return c->fail(PT_ERR_STATE, "no features rendered");
    cudaSetDevice(c->device);
    const size_t n = (size_t)c->feat_w * c->feat_h;
    cudaError_t e = cudaSuccess;
    if (!c->feat_fp16) {
        if (albedo_depth)
            e = cudaMemcpyAsync(albedo_depth, c->feat_a.p, n * sizeof(float4), cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess && normal)
            e = cudaMemcpyAsync(normal, c->feat_n.p, n * sizeof(float4), cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(c->stream);
        return e == cudaSuccess ? PT_OK : c->cuda_fail(e, "feature read-back");
    }
    // FP16 storage: 4 halves per pixel, widened here
    std::vector<__half> h(4 * n);
    for (int k = 0; k < 2 && e == cudaSuccess; k++) {
        float* dst = k == 0 ? albedo_depth : normal;
        if (!dst)
            continue;
        e = cudaMemcpyAsync(h.data(), k == 0 ? (const void*)c->feat_a.p : (const void*)c->feat_n.p, 4 * n * sizeof(__half),
                            cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(c->stream);
        for (size_t i = 0; e == cudaSuccess && i < 4 * n; i++)
            dst[i] = __half2float(h[i]);
    }
    return e == cudaSuccess ? PT_OK : c->cuda_fail(e, "feature read-back");
}

int pt_denoise_snapshot_at(pt_ctx* c, uint32_t samples)
{
    if (!c)
        return PT_ERR_INVALID;
    c->snapshot_armed = samples;
    return PT_OK;
}

static int denoise_input(pt_ctx* c, uint32_t spp, uint16_t* input, float* base)
{
    if (!c->image.p || c->feat_w != c->width || c->feat_h != c->height)
        return c->fail(PT_ERR_STATE, "render the image and its features (pt_render_features) first");
    if (spp == 0)
        return c->fail(PT_ERR_INVALID, "zero samples per pixel");
    const float spp_feature = log2f((float)spp) / 8.0f;
    // the snapshot counts only if it holds the first samples of this very image
    const bool have_half = c->half.p && c->half_w == c->width && c->half_h == c->height && c->half_epoch == c->image_epoch &&
                           c->half_spp < c->samples_done;
    cudaError_t e = launch_denoise_input(c->image.p, have_half ? c->half.p : nullptr, c->feat_a.p, c->feat_n.p,
                                         c->width * c->height, spp_feature, input, base, c->feat_fp16 ? 1u : 0u,
                                         c->half_fp16 ? 1u : 0u, c->stream);
    if (e != cudaSuccess)
        return c->cuda_fail(e, "denoiser input");
    return PT_OK;
}

int pt_denoise_input(pt_ctx* c, uint32_t spp, uint16_t* input, float* base, void* stream)
{
    if (!c || !input)
        return PT_ERR_INVALID;
    cudaSetDevice(c->device);
    int rc = denoise_input(c, spp, input, base);
    if (rc != PT_OK)
        return rc;
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e == cudaSuccess && stream)
        e = cudaStreamSynchronize(static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? PT_OK : c->cuda_fail(e, "denoiser input");
}

int pt_denoise(pt_ctx* c, pt_unet* u, uint32_t spp)
{
    if (!c || !u)
        return PT_ERR_INVALID;
    uint32_t n = 0, h = 0, w = 0;
    pt_unet_shape(u, &n, &h, &w);
    if (n != 1 || h != c->height || w != c->width)
        return c->fail(PT_ERR_INVALID, "denoiser shape differs from the image (batch 1, same height and width)");
    cudaSetDevice(c->device);
    int rc = denoise_input(c, spp, pt_unet_input(u), pt_unet_base(u));
    if (rc != PT_OK)
        return rc;
    rc = pt_unet_forward(u, nullptr, c->stream);
    if (rc != PT_OK)
        return c->fail(rc, std::string("denoiser: ") + pt_unet_last_error(u));
    const size_t pixels = (size_t)w * h;
    if (c->denoised.n < pixels) {
        cudaError_t e = c->denoised.alloc(pixels);
        if (e != cudaSuccess)
            return c->cuda_fail(e, "denoised image");
    }
    cudaError_t e = launch_denoise_output(pt_unet_output(u), (uint32_t)pixels, c->denoised.p, c->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(c->stream);
    return e == cudaSuccess ? PT_OK : c->cuda_fail(e, "denoised image");
}

int pt_tonemap(pt_ctx* c)
{
    if (!c)
        return PT_ERR_INVALID;
    if (!c->image.p)
        return c->fail(PT_ERR_STATE, "nothing rendered");
    cudaSetDevice(c->device);
    cudaError_t e = launch_tonemap(c->image.p, c->width * c->height, c->stream);
    if (e != cudaSuccess)
        return c->cuda_fail(e, "tone map");
    return PT_OK;
}

int pt_mse_host(pt_ctx* c, const float* ref, double* mse)
{
    if (!c || !ref || !mse)
        return PT_ERR_INVALID;
    if (!c->image.p)
        return c->fail(PT_ERR_STATE, "nothing rendered");
    cudaSetDevice(c->device);
    size_t n = (size_t)c->width * c->height;
    cudaError_t e;
    if (c->mse_ref.n < n && (e = c->mse_ref.alloc(n)) != cudaSuccess)
        return c->cuda_fail(e, "MSE reference allocation");
    if (!c->mse_partial.p && (e = c->mse_partial.alloc(MSE_MAX_BLOCKS + 1)) != cudaSuccess)
        return c->cuda_fail(e, "MSE scratch allocation");
    if ((e = cudaMemcpyAsync(c->mse_ref.p, ref, n * sizeof(float4), cudaMemcpyHostToDevice, c->stream)) != cudaSuccess ||
        (e = launch_mse(c->image.p, c->mse_ref.p, c->width, c->height, c->mse_partial.p + 1, c->mse_partial.p, c->stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(mse, c->mse_partial.p, sizeof(double), cudaMemcpyDeviceToHost, c->stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(c->stream)) != cudaSuccess)
        return c->cuda_fail(e, "MSE");
    return PT_OK;
}

} // extern "C"
