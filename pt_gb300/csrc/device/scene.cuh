// scene.cuh — device-side scene layout and two-level BVH traversal.
//
// HBM layout (one allocation per array, all 16-byte aligned):
//   vertices   float4 x 2 per vertex: the reference's 32-B Vertex (mesh.h:10-18)
//   indices    u32, mesh-local, 3 per triangle
//   instances  pt_instance_data, 128 B (scenebuffer.h:13-24)
//   materials  pt_material, 96 B (material.h:24-29)
//   light      u32 light-sampler stream (lightsample.cpp:89-221)
//   nodes      BvhNode, 64 B: both child boxes of a BVH2 node (one array for
//              every BLAS and the TLAS)
//   nodes4     Bvh4Node, 64 B (half-precision planes rounded outwards; two
//              nodes per cache line), same indices as `nodes`: node i's
//              grandchildren (a child that is a leaf stands for itself), so
//              the traversal descends two BVH2 levels per dependent fetch
//   tris       TriRec, 48 B: the three object-space vertices of a triangle in
//              BVH leaf order plus its mesh-local primitive index
//   dinst      DevInstance, 64 B: world-to-object rows + BLAS root reference
// Traversal reads nodes/tris/dinst with 16-byte vector loads through the
// read-only path.
#pragma once
#include <cstdint>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "ptmath.cuh"

namespace pt {

// Child / root reference: >= 0 interior node index; < 0 a leaf holding the
// primitives (first, count) encoded as ~((first << 2) | (count - 1)), with
// first < 2^28.  Two sentinels below the leaf range drive the traversal loop.
constexpr int REF_DONE = (int)0x80000000;
constexpr int REF_EXIT_BLAS = (int)0x80000001;
constexpr int REF_EMPTY = (int)0x80000002;
__host__ __device__ __forceinline__ bool ref_is_leaf(int r) { return r < 0 && r > (int)0x8000000F; }
__host__ __device__ __forceinline__ int make_leaf(uint32_t first, uint32_t count) { return ~(int)((first << 2) | (count - 1)); }
__host__ __device__ __forceinline__ uint32_t leaf_first(int r) { return ((uint32_t)~r) >> 2; }
__host__ __device__ __forceinline__ uint32_t leaf_count(int r) { return (((uint32_t)~r) & 3u) + 1u; }

struct __align__(16) BvhNode {
    float4 c0xy; // c0.lo.x, c0.hi.x, c0.lo.y, c0.hi.y
    float4 c1xy; // c1.lo.x, c1.hi.x, c1.lo.y, c1.hi.y
    float4 c01z; // c0.lo.z, c0.hi.z, c1.lo.z, c1.hi.z
    int4 link;   // child0, child1, -, -
};

// Four child boxes as x/y/z planes across the children (lane k = child k)
// and their references; REF_EMPTY marks an unused slot.
// Half-precision planes, rounded outwards from the BVH2's boxes (lower planes
// toward -inf, upper planes toward +inf), so each box contains the box it
// stands for; two nodes share a 128-byte line.  Per axis a uint4 holds
// (lo0, lo1), (lo2, lo3), (hi0, hi1), (hi2, hi3) as half2 pairs.
struct __align__(64) Bvh4Node {
    uint4 x, y, z;
    int4 link;
};

struct __align__(16) TriRec {
    float4 v0; // xyz, w = primitive index (bits)
    float4 v1;
    float4 v2;
};

struct __align__(16) DevInstance {
    float4 w2o[3];   // rows of the world-to-object 3x4 transform
    int blas_root;   // reference into nodes/tris (REF_EMPTY for an empty mesh)
    uint32_t flags;  // bit 0: opaque
    uint32_t mesh;
    uint32_t pad;
};

struct DevMaterial {
    float4 base_colour, emission, rmn, specular, sheen, cc;
};

struct DevInstanceData {
    uint32_t vertex_index, index_index, emitter_index, material_index;
    float4 t0, t1, t2, t3; // transform rows
    float4 n0, n1, n2;     // normal matrix rows
};

// pt_texture (include/pt_gpu.h): 8-bit texels, 1 / 2 / 4 channels.
struct DevTexture {
    unsigned long long offset;
    uint32_t width, height, channels, srgb;
};

struct DevScene {
    const float4* vertices;
    const uint32_t* indices;
    const DevInstanceData* inst_data;
    const DevMaterial* materials;
    const float* material_ior; // null, or per material: > 0 = smooth dielectric of that index
    const uint32_t* light;
    uint32_t light_words;
    uint32_t light_count;
    uint32_t instance_count;
    uint32_t vertex_count;
    uint32_t max_iterations; // traversal watchdog: loop iterations per ray
    const uint8_t* texels;   // textures (may be empty)
    const DevTexture* textures;
    uint32_t texture_count;
    const BvhNode* nodes;
    const Bvh4Node* nodes4; // null: traverse the BVH2 `nodes`
    const TriRec* tris;
    uint32_t node_count;  // entries of nodes (and nodes4)
    uint32_t tri_count;   // entries of tris
    uint32_t index_count; // entries of indices
    const DevInstance* dinst;
    int tlas_root;
    f3 env;
    uint32_t* error_word; // bit 0: traversal stack overflow
};

constexpr uint32_t ERR_STACK_OVERFLOW = 1u;
constexpr uint32_t ERR_BAD_INDEX = 2u;
constexpr uint32_t ERR_WATCHDOG = 4u;

// Checked builds (-DPT_CHECKED, libptgpu_checked.so): every node, triangle,
// instance, vertex-index and queue index is compared with its array's length
// before it is used; a bad one sets ERR_BAD_INDEX and ends that ray or entry
// instead of reading outside the array (the stand-in for a memory checker).
#ifdef PT_CHECKED
#define PT_CHECK_INDEX(cond, s, on_fail)          \
    if (!(cond)) {                                \
        atomicOr((s).error_word, ERR_BAD_INDEX); \
        on_fail;                                  \
    }
#else
#define PT_CHECK_INDEX(cond, s, on_fail)
#endif

__device__ __forceinline__ float4 ldg4(const float4* p) { return __ldg(p); }
__device__ __forceinline__ int4 ldg4i(const int4* p) { return __ldg(p); }

// Material map bits (constants.h of the reference; include/pt_gpu.h).
constexpr uint32_t MAP_BASE_COLOUR = 1u << 0;
constexpr uint32_t MAP_EMISSION = 1u << 1;
constexpr uint32_t MAP_ROUGHNESS = 1u << 2;
constexpr uint32_t MAP_METALNESS = 1u << 3;
constexpr uint32_t MAP_ROUGHNESS_METALNESS = 1u << 4;
constexpr uint32_t MAP_SPECULAR = 1u << 5;
constexpr uint32_t MAP_SHEEN = 1u << 7;
constexpr uint32_t MAP_CLEARCOAT = 1u << 9;
constexpr uint32_t MAP_NORMAL = 1u << 12;

// sRGB-to-linear decode of 8-bit values (the _SRGB texture formats), filled
// from the host's FP64 evaluation of the sRGB curve (one copy per translation
// unit, uploaded by that unit's table initialiser).
static __constant__ float c_srgb[256];

__device__ __forceinline__ float4 texel(const DevScene& s, const DevTexture& t, uint32_t x, uint32_t y)
{
    const uint8_t* p = s.texels + t.offset + ((unsigned long long)y * t.width + x) * t.channels;
    if (t.channels == 4) {
        const uint8_t r = p[0], g = p[1], b = p[2], a = p[3]; // byte loads: texture offsets need no alignment
        if (t.srgb)
            return make_float4(c_srgb[r], c_srgb[g], c_srgb[b], (float)a / 255.0f);
        return make_float4((float)r / 255.0f, (float)g / 255.0f, (float)b / 255.0f, (float)a / 255.0f);
    }
    if (t.channels == 2)
        return make_float4((float)p[0] / 255.0f, (float)p[1] / 255.0f, 0.0f, 1.0f);
    return make_float4((float)p[0] / 255.0f, 0.0f, 0.0f, 1.0f);
}

// SampleLevel(uv, 0) with the reference's sampler (linear filtering, REPEAT,
// level 0; src/graphics/sampler.cpp:8-22): uv is wrapped to [0, 1), texel
// centres sit at (i + 0.5) / size, the four neighbours wrap, and the weights
// combine as (1-a)(1-b) t00 + a(1-b) t10 + (1-a)b t01 + ab t11 in that order.
// Out-of-range texture indices read zero.
__device__ __forceinline__ float4 sample_texture(const DevScene& s, uint32_t index, f2 uv)
{
    if (index >= s.texture_count)
        return make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const DevTexture t = s.textures[index];
    float u = uv.x - floorf(uv.x), v = uv.y - floorf(uv.y);
    if (!(u >= 0.0f && u < 1.0f))
        u = 0.0f;
    if (!(v >= 0.0f && v < 1.0f))
        v = 0.0f;
    const float x = u * (float)t.width - 0.5f, y = v * (float)t.height - 0.5f;
    const float fx = floorf(x), fy = floorf(y);
    const float a = x - fx, b = y - fy;
    int x0 = (int)fx, y0 = (int)fy;
    if (x0 < 0)
        x0 += (int)t.width;
    if (y0 < 0)
        y0 += (int)t.height;
    if (x0 >= (int)t.width)
        x0 = (int)t.width - 1;
    if (y0 >= (int)t.height)
        y0 = (int)t.height - 1;
    const uint32_t x1 = (uint32_t)x0 + 1 == t.width ? 0u : (uint32_t)x0 + 1;
    const uint32_t y1 = (uint32_t)y0 + 1 == t.height ? 0u : (uint32_t)y0 + 1;
    const float4 t00 = texel(s, t, x0, y0), t10 = texel(s, t, x1, y0), t01 = texel(s, t, x0, y1), t11 = texel(s, t, x1, y1);
    const float w00 = (1.0f - a) * (1.0f - b), w10 = a * (1.0f - b), w01 = (1.0f - a) * b, w11 = a * b;
    return make_float4(((w00 * t00.x + w10 * t10.x) + w01 * t01.x) + w11 * t11.x,
                       ((w00 * t00.y + w10 * t10.y) + w01 * t01.y) + w11 * t11.y,
                       ((w00 * t00.z + w10 * t10.z) + w01 * t01.z) + w11 * t11.z,
                       ((w00 * t00.w + w10 * t10.w) + w01 * t01.w) + w11 * t11.w);
}

// Texture coordinate of a point of a triangle (get_vertex_attributes,
// geometry.hlsli:38-47); indices outside the vertex array read zero.
__device__ __forceinline__ f2 vertex_uv(const DevScene& s, unsigned long long i)
{
    if (i >= (unsigned long long)s.vertex_count)
        return f2{0.0f, 0.0f};
    const float4 b = __ldg(s.vertices + 2 * (size_t)i + 1);
    return f2{b.z, b.w};
}

__device__ __forceinline__ f2 hit_uv(const DevScene& s, uint32_t inst, uint32_t prim, float b1, float b2)
{
    const DevInstanceData* id = s.inst_data + inst;
    const uint32_t vbase = __ldg(&id->vertex_index), ibase = __ldg(&id->index_index);
    const f2 ua = vertex_uv(s, (unsigned long long)vbase + __ldg(s.indices + ibase + prim * 3 + 0));
    const f2 ub = vertex_uv(s, (unsigned long long)vbase + __ldg(s.indices + ibase + prim * 3 + 1));
    const f2 uc = vertex_uv(s, (unsigned long long)vbase + __ldg(s.indices + ibase + prim * 3 + 2));
    const float ba = (1.0f - b1) - b2;
    return f2{(ba * ua.x + b1 * ub.x) + b2 * uc.x, (ba * ua.y + b1 * ub.y) + b2 * uc.y};
}

// Light-stream word with robust-buffer-access semantics (out of range reads 0).
__device__ __forceinline__ uint32_t lw(const DevScene& s, uint32_t i) { return i < s.light_words ? __ldg(s.light + i) : 0u; }

struct Ray {
    f3 o, d;
};

struct ObjRay {
    f3 o, d;
    f3 inv_d, o_inv; // 1/d and o/d for the slab test
    int kx, ky, kz;
    float sx, sy, sz;
};

__device__ __forceinline__ void setup_slab(ObjRay& r)
{
    r.inv_d = mk3(1.0f / r.d.x, 1.0f / r.d.y, 1.0f / r.d.z);
    r.o_inv = mk3(r.o.x * r.inv_d.x, r.o.y * r.inv_d.y, r.o.z * r.inv_d.z);
}

__device__ __forceinline__ void setup_watertight(ObjRay& r)
{
    float ax = fabsf(r.d.x), ay = fabsf(r.d.y), az = fabsf(r.d.z);
    int kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
    int kx = kz + 1;
    if (kx == 3)
        kx = 0;
    int ky = kx + 1;
    if (ky == 3)
        ky = 0;
    float dz = comp(r.d, kz);
    if (dz < 0.0f) {
        int t = kx;
        kx = ky;
        ky = t;
    }
    r.kx = kx;
    r.ky = ky;
    r.kz = kz;
    r.sx = comp(r.d, kx) / dz;
    r.sy = comp(r.d, ky) / dz;
    r.sz = 1.0f / dz;
}

// Robust slab test (Ize 2013): far distances are scaled by 1 + 2*gamma(3).
// Box planes are padded at build time, so NaNs from 0*inf (a ray on a slab
// plane of a zero direction component) are ignored by fminf/fmaxf safely.
constexpr float SLAB_SCALE = 1.0f + 2.0f * (3.0f * 0x1p-24f) / (1.0f - 3.0f * 0x1p-24f);

__device__ __forceinline__ float slab_enter(float lo, float hi, float inv, float oinv, float& tfar)
{
    float t0 = fmaf(lo, inv, -oinv);
    float t1 = fmaf(hi, inv, -oinv);
    tfar = fmaxf(t0, t1) * SLAB_SCALE;
    return fminf(t0, t1);
}

// Intersect both children of a node; returns a bitmask (1 = c0, 2 = c1) and
// the entry distances.
__device__ __forceinline__ int node_children(const BvhNode* node, const ObjRay& r, float tmin, float tmax, float& e0, float& e1,
                                             int& c0, int& c1)
{
    float4 a = ldg4(&node->c0xy);
    float4 b = ldg4(&node->c1xy);
    float4 z = ldg4(&node->c01z);
    int4 l = ldg4i(&node->link);
    float f0x, f0y, f0z, f1x, f1y, f1z;
    float n0x = slab_enter(a.x, a.y, r.inv_d.x, r.o_inv.x, f0x);
    float n0y = slab_enter(a.z, a.w, r.inv_d.y, r.o_inv.y, f0y);
    float n0z = slab_enter(z.x, z.y, r.inv_d.z, r.o_inv.z, f0z);
    float n1x = slab_enter(b.x, b.y, r.inv_d.x, r.o_inv.x, f1x);
    float n1y = slab_enter(b.z, b.w, r.inv_d.y, r.o_inv.y, f1y);
    float n1z = slab_enter(z.z, z.w, r.inv_d.z, r.o_inv.z, f1z);
    e0 = fmaxf(fmaxf(fmaxf(n0x, n0y), n0z), tmin);
    float x0 = fminf(fminf(fminf(f0x, f0y), f0z), tmax);
    e1 = fmaxf(fmaxf(fmaxf(n1x, n1y), n1z), tmin);
    float x1 = fminf(fminf(fminf(f1x, f1y), f1z), tmax);
    c0 = l.x;
    c1 = l.y;
    return (e0 <= x0 ? 1 : 0) | (e1 <= x1 ? 2 : 0);
}

// Three-input minimum / maximum (PTX min/max.f32 with three operands on
// sm_100 and later): the same value as two nested fminf / fmaxf, NaN operands
// ignored likewise.
__device__ __forceinline__ float fmin3f(float a, float b, float c)
{
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
__device__ __forceinline__ float fmax3f(float a, float b, float c)
{
    float d;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

// One axis of a half-precision 4-wide node: the lower and upper planes of the
// four children as floats (exact: every half is a float).
__device__ __forceinline__ void unpack_planes(const uint4& q, float4& lo, float4& hi)
{
    const float2 l01 = __half22float2(*reinterpret_cast<const __half2*>(&q.x));
    const float2 l23 = __half22float2(*reinterpret_cast<const __half2*>(&q.y));
    const float2 h01 = __half22float2(*reinterpret_cast<const __half2*>(&q.z));
    const float2 h23 = __half22float2(*reinterpret_cast<const __half2*>(&q.w));
    lo = make_float4(l01.x, l01.y, l23.x, l23.y);
    hi = make_float4(h01.x, h01.y, h23.x, h23.y);
}

// Intersect the four child boxes of a 4-wide node; bit k of the result is
// set when child k is hit, e[k] its entry distance.  The boxes contain the
// BVH2's (outward rounding), so a child the BVH2 would enter is entered here
// too and the closest hit is the same.  The far distance is
// scaled once after the minimum over the axes instead of once per axis:
// rounding is monotonic, so min(a s, b s, c s) = min(a, b, c) s for s > 0 and
// the value equals the per-axis form of slab_enter bit for bit.
__device__ __forceinline__ int node4_children(const Bvh4Node* node, const ObjRay& r, float tmin, float tmax, float (&e)[4], int (&c)[4])
{
    const uint4 qx = __ldg(&node->x), qy = __ldg(&node->y), qz = __ldg(&node->z);
    float4 lx, hx, ly, hy, lz, hz;
    unpack_planes(qx, lx, hx);
    unpack_planes(qy, ly, hy);
    unpack_planes(qz, lz, hz);
    const int4 l = ldg4i(&node->link);
    c[0] = l.x;
    c[1] = l.y;
    c[2] = l.z;
    c[3] = l.w;
    int m = 0;
#define PT_NODE4_CHILD(k, q)                                                                     \
    {                                                                                            \
        const float x0 = fmaf(lx.q, r.inv_d.x, -r.o_inv.x), x1 = fmaf(hx.q, r.inv_d.x, -r.o_inv.x); \
        const float y0 = fmaf(ly.q, r.inv_d.y, -r.o_inv.y), y1 = fmaf(hy.q, r.inv_d.y, -r.o_inv.y); \
        const float z0 = fmaf(lz.q, r.inv_d.z, -r.o_inv.z), z1 = fmaf(hz.q, r.inv_d.z, -r.o_inv.z); \
        e[k] = fmaxf(fmax3f(fminf(x0, x1), fminf(y0, y1), fminf(z0, z1)), tmin);                   \
        const float far = fmin3f(fmaxf(x0, x1), fmaxf(y0, y1), fmaxf(z0, z1)) * SLAB_SCALE;      \
        const float x = fminf(far, tmax);                                                        \
        m |= (e[k] <= x && l.q != REF_EMPTY) ? (1 << k) : 0;                                     \
    }
    PT_NODE4_CHILD(0, x)
    PT_NODE4_CHILD(1, y)
    PT_NODE4_CHILD(2, z)
    PT_NODE4_CHILD(3, w)
#undef PT_NODE4_CHILD
    return m;
}

constexpr int STACK_SIZE = 96;

// One interior step of a 4-wide traversal: the nearest hit child becomes
// `ref`, the others are pushed far to near (SORT; else in slot order, for
// any-hit queries whose result does not depend on the order); nothing hit
// pops the stack.  A push that would overflow sets ERR_STACK_OVERFLOW and
// drops those children.
template <bool SORT = true, class Stack>
__device__ __forceinline__ void step4(const DevScene& s, const ObjRay& r, float tmin, float tmax, int& ref, Stack& stack, int& sp)
{
    constexpr int N = STACK_SIZE;
    float e[4];
    int c[4];
    const int m = node4_children(s.nodes4 + ref, r, tmin, tmax, e, c);
    const int cnt = __popc(m);
    if (cnt == 0) {
        ref = stack.get(--sp);
        return;
    }
    if (cnt == 1) {
        ref = c[__ffs(m) - 1];
        return;
    }
    if (!SORT) {
        if (sp + cnt - 1 > N) {
            atomicOr(s.error_word, ERR_STACK_OVERFLOW);
            ref = c[__ffs(m) - 1];
            return;
        }
        int rest = m;
        ref = c[__ffs(rest) - 1];
        rest &= rest - 1;
        while (rest) {
            stack.set(sp++, c[__ffs(rest) - 1]);
            rest &= rest - 1;
        }
        return;
    }
    // sort (entry, child) ascending with misses keyed +inf: a five-exchange network
    const float inf = __int_as_float(0x7f800000);
    float k0 = (m & 1) ? e[0] : inf, k1 = (m & 2) ? e[1] : inf, k2 = (m & 4) ? e[2] : inf, k3 = (m & 8) ? e[3] : inf;
    int r0 = c[0], r1 = c[1], r2 = c[2], r3 = c[3];
#define PT_CSWAP(ka, ra, kb, rb)  \
    if (kb < ka) {                \
        const float tk = ka;      \
        ka = kb;                  \
        kb = tk;                  \
        const int tr = ra;        \
        ra = rb;                  \
        rb = tr;                  \
    }
    PT_CSWAP(k0, r0, k1, r1)
    PT_CSWAP(k2, r2, k3, r3)
    PT_CSWAP(k0, r0, k2, r2)
    PT_CSWAP(k1, r1, k3, r3)
    PT_CSWAP(k1, r1, k2, r2)
#undef PT_CSWAP
    if (sp + cnt - 1 > N) {
        atomicOr(s.error_word, ERR_STACK_OVERFLOW);
    } else {
        if (cnt == 4)
            stack.set(sp++, r3);
        if (cnt >= 3)
            stack.set(sp++, r2);
        stack.set(sp++, r1);
    }
    ref = r0;
}

// Watertight ray/triangle test (Woop, Benthin & Wald 2013) without culling.
__device__ __forceinline__ bool watertight(const ObjRay& r, f3 p0, f3 p1, f3 p2, float& t, float& b1, float& b2)
{
    f3 A = p0 - r.o, B = p1 - r.o, C = p2 - r.o;
    float Akx = comp(A, r.kx), Aky = comp(A, r.ky), Akz = comp(A, r.kz);
    float Bkx = comp(B, r.kx), Bky = comp(B, r.ky), Bkz = comp(B, r.kz);
    float Ckx = comp(C, r.kx), Cky = comp(C, r.ky), Ckz = comp(C, r.kz);
    float Ax = Akx - r.sx * Akz, Ay = Aky - r.sy * Akz;
    float Bx = Bkx - r.sx * Bkz, By = Bky - r.sy * Bkz;
    float Cx = Ckx - r.sx * Ckz, Cy = Cky - r.sy * Ckz;
    float U = Cx * By - Cy * Bx;
    float V = Ax * Cy - Ay * Cx;
    float W = Bx * Ay - By * Ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
        V = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
        W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f))
        return false;
    float det = (U + V) + W;
    if (det == 0.0f)
        return false;
    float Az = r.sz * Akz, Bz = r.sz * Bkz, Cz = r.sz * Ckz;
    float T = (U * Az + V * Bz) + W * Cz;
    float inv = 1.0f / det;
    t = T * inv;
    b1 = V * inv;
    b2 = W * inv;
    return true;
}

__device__ __forceinline__ void to_object(const DevInstance* di, f3 o, f3 d, ObjRay& r)
{
    float4 w0 = ldg4(&di->w2o[0]), w1 = ldg4(&di->w2o[1]), w2 = ldg4(&di->w2o[2]);
    r.o = mk3(((w0.x * o.x + w0.y * o.y) + w0.z * o.z) + w0.w, ((w1.x * o.x + w1.y * o.y) + w1.z * o.z) + w1.w,
              ((w2.x * o.x + w2.y * o.y) + w2.z * o.z) + w2.w);
    r.d = mk3((w0.x * d.x + w0.y * d.y) + w0.z * d.z, (w1.x * d.x + w1.y * d.y) + w1.z * d.z, (w2.x * d.x + w2.y * d.y) + w2.z * d.z);
    setup_slab(r);
    setup_watertight(r);
}

struct Hit {
    float t, b1, b2;
    uint32_t inst, prim;
};

// Traversal work of one ray: interior nodes whose child boxes were tested and
// ray/triangle tests.
struct TraceCounters {
    uint32_t nodes, tris;
};

__device__ __forceinline__ bool better(float t, uint32_t inst, uint32_t prim, const Hit& h)
{
    if (t < h.t)
        return true;
    if (t > h.t)
        return false;
    return inst < h.inst || (inst == h.inst && prim < h.prim);
}


// BVH2 interior step: the nearer hit child becomes `ref`, the farther is
// pushed; nothing hit pops the stack.
template <class Stack>
__device__ __forceinline__ void step2(const DevScene& s, const ObjRay& r, float tmin, float tmax, int& ref, Stack& stack, int& sp)
{
    constexpr int N = STACK_SIZE;
    float e0, e1;
    int c0, c1;
    const int m = node_children(s.nodes + ref, r, tmin, tmax, e0, e1, c0, c1);
    if (m == 3) {
        int near = c0, far = c1;
        if (e1 < e0) {
            near = c1;
            far = c0;
        }
        if (sp < N)
            stack.set(sp++, far);
        else
            atomicOr(s.error_word, ERR_STACK_OVERFLOW);
        ref = near;
    } else if (m == 1) {
        ref = c0;
    } else if (m == 2) {
        ref = c1;
    } else {
        ref = stack.get(--sp);
    }
}

// Closest-hit traversal of one ray as a resumable state: closest_begin sets
// it up and each closest_step advances it by one node visit, leaf or
// instance transition, returning true when the ray is finished.  The hit is
// the (t, instance, primitive) minimum of the oracle whatever the BVH.  The
// stack lives in local memory (L1-resident).  W4 walks the 4-wide nodes
// (s.nodes4, which must be present), else the BVH2.
struct ClosestTrace {
    ObjRay world, r;
    Hit h;
    float tmin;
    int ref, sp;
    uint32_t cur_inst, iter;
    bool in_blas, found;
};
// The traversal stack is kept apart from the state: inside the state it
// would pull every field of the state into local memory with it.  It lives in
// local memory (L1).  Built with PT_SMEM_STACK = k > 0, its first k entries
// live in shared memory instead, entry i of thread x at word i * 128 + x
// (every lane in its own bank whatever its depth); that measured slower on
// the mid scene (extend 72.0 ms per step in local memory, 77.9 with 8 entries
// and 78.6 with 16 in shared memory: the per-access branch and the smaller
// L1 cost more than the bank-parallel accesses save).  Every kernel that
// traverses runs blocks of at most 128 threads; a stack is used by one
// traversal at a time per thread.
#ifndef PT_SMEM_STACK
#define PT_SMEM_STACK 0
#endif
constexpr int STACK_SMEM = PT_SMEM_STACK;
constexpr int STACK_BLOCK = 128;

struct TraceStack {
#if PT_SMEM_STACK
    int* sm; // this thread's column of the block's shared array
    int loc[STACK_SIZE - STACK_SMEM];
    __device__ __forceinline__ TraceStack()
    {
        __shared__ int s_stack[STACK_SMEM * STACK_BLOCK];
        sm = s_stack + threadIdx.x;
    }
    __device__ __forceinline__ int get(int i) const { return i < STACK_SMEM ? sm[i * STACK_BLOCK] : loc[i - STACK_SMEM]; }
    __device__ __forceinline__ void set(int i, int v)
    {
        if (i < STACK_SMEM)
            sm[i * STACK_BLOCK] = v;
        else
            loc[i - STACK_SMEM] = v;
    }
#else
    int loc[STACK_SIZE];
    __device__ __forceinline__ int get(int i) const { return loc[i]; }
    __device__ __forceinline__ void set(int i, int v) { loc[i] = v; }
#endif
};

__device__ __forceinline__ void closest_begin(const DevScene& s, f3 o, f3 d, float tmin, float tmax, ClosestTrace& t, TraceStack& stack)
{
    t.h.t = tmax;
    t.h.inst = 0xFFFFFFFFu;
    t.h.prim = 0xFFFFFFFFu;
    t.h.b1 = t.h.b2 = 0.0f;
    t.found = false;
    t.world.o = o;
    t.world.d = d;
    setup_slab(t.world);
    t.r = t.world;
    t.tmin = tmin;
    t.sp = 0;
    stack.set(t.sp++, REF_DONE);
    t.ref = s.tlas_root == REF_EMPTY ? REF_DONE : s.tlas_root;
    t.in_blas = false;
    t.cur_inst = 0;
    t.iter = 0;
}

template <bool W4>
__device__ __forceinline__ bool closest_step(const DevScene& s, ClosestTrace& t, TraceStack& stack, TraceCounters& tc)
{
    if (t.iter >= s.max_iterations) {
        // A well-formed BVH never gets here; a malformed one must not hang the GPU.
        atomicOr(s.error_word, ERR_WATCHDOG);
        return true;
    }
    t.iter++;
    const int ref = t.ref;
    if (ref >= 0) {
        PT_CHECK_INDEX((uint32_t)ref < s.node_count, s, return true)
        tc.nodes++;
        if (W4)
            step4(s, t.r, t.tmin, t.h.t, t.ref, stack, t.sp);
        else
            step2(s, t.r, t.tmin, t.h.t, t.ref, stack, t.sp);
        return false;
    }
    if (ref == REF_DONE)
        return true;
    if (ref == REF_EXIT_BLAS) {
        t.r = t.world;
        t.in_blas = false;
        t.ref = stack.get(--t.sp);
        return false;
    }
    const uint32_t first = leaf_first(ref), count = leaf_count(ref);
    if (!t.in_blas) {
        // TLAS leaf: instances [first, first + count); one per leaf here.
        PT_CHECK_INDEX(first < s.instance_count, s, return true)
        t.cur_inst = first;
        const DevInstance* di = s.dinst + first;
        const int root = __ldg(&di->blas_root);
        if (root == REF_EMPTY || count != 1) {
            t.ref = stack.get(--t.sp);
            return false;
        }
        to_object(di, t.world.o, t.world.d, t.r);
        if (t.sp >= STACK_SIZE) {
            atomicOr(s.error_word, ERR_STACK_OVERFLOW);
            t.ref = stack.get(--t.sp);
            return false;
        }
        stack.set(t.sp++, REF_EXIT_BLAS);
        t.in_blas = true;
        t.ref = root;
        return false;
    }
    PT_CHECK_INDEX((uint64_t)first + count <= s.tri_count, s, return true)
    tc.tris += count;
    for (uint32_t k = 0; k < count; k++) {
        const TriRec* tr = s.tris + first + k;
        const float4 a = ldg4(&tr->v0), b = ldg4(&tr->v1), c = ldg4(&tr->v2);
        float tt, b1, b2;
        const uint32_t prim = __float_as_uint(a.w);
        if (watertight(t.r, mk3(a.x, a.y, a.z), mk3(b.x, b.y, b.z), mk3(c.x, c.y, c.z), tt, b1, b2) && tt >= t.tmin &&
            tt <= t.h.t && better(tt, t.cur_inst, prim, t.h)) {
            t.h.t = tt;
            t.h.b1 = b1;
            t.h.b2 = b2;
            t.h.inst = t.cur_inst;
            t.h.prim = prim;
            t.found = true;
        }
    }
    t.ref = stack.get(--t.sp);
    return false;
}

// A closest-hit traversal paused after a step budget (its "parking"): what a
// later pass needs to continue it exactly where it stopped.  The world ray is
// rebuilt from the path state and the object-space ray from the instance, so
// a slot holds the node reference, the stack, the instance, the step count and
// the best hit so far; slots are SoA arrays of `cap` entries, the stack
// word-major (stack[k * cap + slot]) so a warp's loads and stores coalesce.
constexpr int PARK_STACK = 32; // deeper stacks finish in the first pass

struct TraceParking {
    uint32_t* path;  // the path of each slot
    int4* state;     // ref, sp | in_blas << 16 | found << 17, cur_inst, iter
    float4* hit;     // t, b1, b2, bits(inst)
    uint32_t* prim;  // primitive of the best hit
    int* stack;      // PARK_STACK words per slot, word-major
    uint32_t cap;    // slots
};

__device__ __forceinline__ void park_closest(const TraceParking& pk, uint32_t slot, uint32_t path, const ClosestTrace& t,
                                             const TraceStack& stack)
{
    pk.path[slot] = path;
    pk.state[slot] = make_int4(t.ref, t.sp | (t.in_blas ? 1 << 16 : 0) | (t.found ? 1 << 17 : 0), (int)t.cur_inst, (int)t.iter);
    pk.hit[slot] = make_float4(t.h.t, t.h.b1, t.h.b2, __uint_as_float(t.h.inst));
    pk.prim[slot] = t.h.prim;
    for (int k = 0; k < t.sp; k++)
        pk.stack[(size_t)k * pk.cap + slot] = stack.get(k);
}

// Restores a parked traversal of the ray (o, d, tmin): the same state the
// first pass left, so closest_step continues the same sequence of steps.
__device__ __forceinline__ void resume_closest(const DevScene& s, const TraceParking& pk, uint32_t slot, f3 o, f3 d, float tmin,
                                               ClosestTrace& t, TraceStack& stack)
{
    const int4 st = pk.state[slot];
    const float4 h = pk.hit[slot];
    t.world.o = o;
    t.world.d = d;
    setup_slab(t.world);
    t.tmin = tmin;
    t.ref = st.x;
    t.sp = st.y & 0xFFFF;
    t.in_blas = (st.y >> 16) & 1;
    t.found = (st.y >> 17) & 1;
    t.cur_inst = (uint32_t)st.z;
    t.iter = (uint32_t)st.w;
    t.h.t = h.x;
    t.h.b1 = h.y;
    t.h.b2 = h.z;
    t.h.inst = __float_as_uint(h.w);
    t.h.prim = pk.prim[slot];
    if (t.in_blas)
        to_object(s.dinst + t.cur_inst, t.world.o, t.world.d, t.r);
    else
        t.r = t.world;
    for (int k = 0; k < t.sp; k++)
        stack.set(k, pk.stack[(size_t)k * pk.cap + slot]);
}

// Closest hit of one ray, traversed to the end.  Returns true on a hit.
template <bool W4>
static __device__ __forceinline__ bool trace_closest_inl(const DevScene& s, f3 o, f3 d, float tmin, float tmax, Hit& h, TraceCounters& tc)
{
    ClosestTrace t;
    TraceStack stack;
    closest_begin(s, o, d, tmin, tmax, t, stack);
    while (!closest_step<W4>(s, t, stack, tc)) {
    }
    h = t.h;
    return t.found;
}

// Closest hit as trace_closest_inl, traversed "while-while" with speculative
// leaves (Aila & Laine 2009): a lane that reaches a BLAS leaf parks it and
// keeps descending interior nodes until every converged lane of the warp holds
// a parked leaf (or has none left), then the warp tests triangles together.
// Instance entry and exit happen in the node phase, but only with no leaf
// parked (a parked leaf belongs to the current instance's object-space ray).
// The hit is the same (t, instance, primitive) minimum: triangles are only
// tested later, never skipped, and culling compares against the best t so far.
static __device__ __forceinline__ bool trace_closest_ww(const DevScene& s, f3 o, f3 d, float tmin, float tmax, Hit& h,
                                                        TraceCounters& tc)
{
    uint32_t n_nodes = 0, n_tris = 0;
    h.t = tmax;
    h.inst = 0xFFFFFFFFu;
    h.prim = 0xFFFFFFFFu;
    h.b1 = h.b2 = 0.0f;
    bool found = false;
    ObjRay world;
    world.o = o;
    world.d = d;
    setup_slab(world);
    ObjRay r = world;
    int stack[STACK_SIZE];
    int sp = 0;
    stack[sp++] = REF_DONE;
    int ref = s.tlas_root;
    bool in_blas = false;
    uint32_t cur_inst = 0;
    if (ref == REF_EMPTY)
        return false;
    int leaf = REF_EMPTY; // parked BLAS leaf (REF_EMPTY: none)
    uint32_t iter = 0;
    for (;;) {
        // node phase
        while (ref != REF_DONE) {
            if (++iter >= s.max_iterations)
                break;
            if (ref >= 0) {
                float e0, e1;
                int c0, c1;
                n_nodes++;
                int m = node_children(s.nodes + ref, r, tmin, h.t, e0, e1, c0, c1);
                if (m == 3) {
                    int near = c0, far = c1;
                    if (e1 < e0) {
                        near = c1;
                        far = c0;
                    }
                    if (sp < STACK_SIZE)
                        stack[sp++] = far;
                    else
                        atomicOr(s.error_word, ERR_STACK_OVERFLOW);
                    ref = near;
                } else if (m == 1) {
                    ref = c0;
                } else if (m == 2) {
                    ref = c1;
                } else {
                    ref = stack[--sp];
                }
            } else if (ref == REF_EXIT_BLAS) {
                if (leaf != REF_EMPTY)
                    break;
                r = world;
                in_blas = false;
                ref = stack[--sp];
            } else if (!in_blas) {
                // TLAS leaf: instances [first, first + count); one per leaf here.
                const uint32_t first = leaf_first(ref), count = leaf_count(ref);
                const DevInstance* di = s.dinst + first;
                const int root = __ldg(&di->blas_root);
                if (root == REF_EMPTY || count != 1 || sp >= STACK_SIZE) {
                    if (sp >= STACK_SIZE)
                        atomicOr(s.error_word, ERR_STACK_OVERFLOW);
                    ref = stack[--sp];
                } else {
                    cur_inst = first;
                    to_object(di, o, d, r);
                    stack[sp++] = REF_EXIT_BLAS;
                    in_blas = true;
                    ref = root;
                }
            } else {
                if (leaf != REF_EMPTY)
                    break;
                leaf = ref;
                ref = stack[--sp];
            }
            if (!__any_sync(__activemask(), leaf == REF_EMPTY))
                break;
        }
        if (iter >= s.max_iterations) {
            // A well-formed BVH never gets here; a malformed one must not hang the GPU.
            atomicOr(s.error_word, ERR_WATCHDOG);
            break;
        }
        // leaf phase
        if (leaf != REF_EMPTY) {
            const uint32_t first = leaf_first(leaf), count = leaf_count(leaf);
            n_tris += count;
            for (uint32_t k = 0; k < count; k++) {
                const TriRec* tr = s.tris + first + k;
                float4 a = ldg4(&tr->v0), b = ldg4(&tr->v1), c = ldg4(&tr->v2);
                float t, b1, b2;
                uint32_t prim = __float_as_uint(a.w);
                if (watertight(r, mk3(a.x, a.y, a.z), mk3(b.x, b.y, b.z), mk3(c.x, c.y, c.z), t, b1, b2) && t >= tmin && t <= h.t &&
                    better(t, cur_inst, prim, h)) {
                    h.t = t;
                    h.b1 = b1;
                    h.b2 = b2;
                    h.inst = cur_inst;
                    h.prim = prim;
                    found = true;
                }
            }
            leaf = REF_EMPTY;
        } else if (ref == REF_DONE) {
            break;
        }
    }
    tc.nodes += n_nodes;
    tc.tris += n_tris;
    return found;
}

// Shadow ray of shadowray.ah.hlsl / shadowray.ms.hlsl: the first opaque hit in
// [tmin, tmax] occludes; transparent instances attenuate by (1 - alpha).
// Returns the visibility throughput (0 = occluded).
// Any-hit shadow traversal of one ray as a resumable state (shadowray.ah.hlsl:
// 12-40): opaque hits end it with visibility 0, transparent instances scale
// the throughput by 1 - alpha and it ends occluded below 1e-5.
struct ShadowTrace {
    ObjRay world, r;
    float tmin, tmax, throughput, alpha_pass;
    int ref, sp;
    uint32_t iter, alpha_tex, alpha_inst, inst;
    bool in_blas, opaque, alpha_map; // alpha_map: the transparent instance's alpha comes from a base colour map
};

__device__ __forceinline__ void shadow_begin(const DevScene& s, f3 o, f3 d, float tmin, float tmax, ShadowTrace& t, TraceStack& stack)
{
    t.world.o = o;
    t.world.d = d;
    setup_slab(t.world);
    t.r = t.world;
    t.tmin = tmin;
    t.tmax = tmax;
    t.sp = 0;
    stack.set(t.sp++, REF_DONE);
    t.ref = s.tlas_root == REF_EMPTY ? REF_DONE : s.tlas_root;
    t.in_blas = false;
    t.opaque = true;
    t.alpha_map = false;
    t.alpha_tex = t.alpha_inst = t.inst = 0;
    t.alpha_pass = 1.0f;
    t.throughput = 1.0f;
    t.iter = 0;
}

// Visibility of a finished shadow ray.
__device__ __forceinline__ float shadow_result(const ShadowTrace& t) { return t.throughput < 1e-5f ? 0.0f : t.throughput; }

template <bool W4>
__device__ __forceinline__ bool shadow_step(const DevScene& s, ShadowTrace& t, TraceStack& stack, TraceCounters& tc)
{
    if (t.iter >= s.max_iterations) {
        // A well-formed BVH never gets here; a malformed one must not hang the GPU.
        atomicOr(s.error_word, ERR_WATCHDOG);
        return true;
    }
    t.iter++;
    const int ref = t.ref;
    if (ref >= 0) {
        PT_CHECK_INDEX((uint32_t)ref < s.node_count, s, return true)
        tc.nodes++;
        if (W4)
            step4<false>(s, t.r, t.tmin, t.tmax, t.ref, stack, t.sp);
        else
            step2(s, t.r, t.tmin, t.tmax, t.ref, stack, t.sp);
        return false;
    }
    if (ref == REF_DONE)
        return true;
    if (ref == REF_EXIT_BLAS) {
        t.r = t.world;
        t.in_blas = false;
        t.ref = stack.get(--t.sp);
        return false;
    }
    const uint32_t first = leaf_first(ref), count = leaf_count(ref);
    if (!t.in_blas) {
        PT_CHECK_INDEX(first < s.instance_count, s, return true)
        const DevInstance* di = s.dinst + first;
        const int root = __ldg(&di->blas_root);
        if (root == REF_EMPTY || count != 1) {
            t.ref = stack.get(--t.sp);
            return false;
        }
        const uint32_t flags = __ldg(&di->flags);
        t.inst = first;
        t.opaque = (flags & 1u) != 0;
        if (!t.opaque) {
            const uint32_t mi = __ldg(&s.inst_data[first].material_index);
            t.alpha_map = (__float_as_uint(__ldg(&s.materials[mi].rmn.w)) & MAP_BASE_COLOUR) != 0;
            t.alpha_tex = __float_as_uint(__ldg(&s.materials[mi].base_colour.x));
            t.alpha_inst = first;
            t.alpha_pass = 1.0f - __ldg(&s.materials[mi].base_colour.w);
        }
        to_object(di, t.world.o, t.world.d, t.r);
        if (t.sp >= STACK_SIZE) {
            atomicOr(s.error_word, ERR_STACK_OVERFLOW);
            t.ref = stack.get(--t.sp);
            return false;
        }
        stack.set(t.sp++, REF_EXIT_BLAS);
        t.in_blas = true;
        t.ref = root;
        return false;
    }
    PT_CHECK_INDEX((uint64_t)first + count <= s.tri_count, s, return true)
    tc.tris += count;
    for (uint32_t k = 0; k < count; k++) {
        const TriRec* tr = s.tris + first + k;
        const float4 a = ldg4(&tr->v0), b = ldg4(&tr->v1), c = ldg4(&tr->v2);
        float tt, b1, b2;
        if (watertight(t.r, mk3(a.x, a.y, a.z), mk3(b.x, b.y, b.z), mk3(c.x, c.y, c.z), tt, b1, b2) && tt >= t.tmin &&
            tt <= t.tmax) {
            if (t.opaque) {
                t.throughput = 0.0f;
                break;
            }
            // shadowray.ah.hlsl:29-34: throughput *= 1 - base colour alpha at the hit
            if (t.alpha_map)
                t.alpha_pass = 1.0f - sample_texture(s, t.alpha_tex, hit_uv(s, t.alpha_inst, __float_as_uint(a.w), b1, b2)).w;
            t.throughput *= t.alpha_pass;
            if (t.throughput < 1e-5f)
                break;
        }
    }
    if (t.throughput == 0.0f || t.throughput < 1e-5f)
        return true;
    t.ref = stack.get(--t.sp);
    return false;
}

// Parking of an any-hit (shadow) traversal in the slots of TraceParking:
// state = ref, sp | in_blas << 16 | opaque << 17 | alpha_map << 18, the
// instance being traversed, iter; hit = throughput, alpha_pass,
// bits(alpha_tex), unused.  The instance's object-space ray is rebuilt on
// resume from the world ray, as on entry.
__device__ __forceinline__ void park_shadow(const TraceParking& pk, uint32_t slot, uint32_t path, const ShadowTrace& t,
                                            const TraceStack& stack)
{
    pk.path[slot] = path;
    pk.state[slot] = make_int4(t.ref,
                               t.sp | (t.in_blas ? 1 << 16 : 0) | (t.opaque ? 1 << 17 : 0) | (t.alpha_map ? 1 << 18 : 0),
                               (int)t.inst, (int)t.iter);
    pk.hit[slot] = make_float4(t.throughput, t.alpha_pass, __uint_as_float(t.alpha_tex), 0.0f);
    for (int k = 0; k < t.sp; k++)
        pk.stack[(size_t)k * pk.cap + slot] = stack.get(k);
}

__device__ __forceinline__ void resume_shadow(const DevScene& s, const TraceParking& pk, uint32_t slot, f3 o, f3 d, float tmin,
                                              float tmax, ShadowTrace& t, TraceStack& stack)
{
    const int4 st = pk.state[slot];
    const float4 h = pk.hit[slot];
    t.world.o = o;
    t.world.d = d;
    setup_slab(t.world);
    t.tmin = tmin;
    t.tmax = tmax;
    t.ref = st.x;
    t.sp = st.y & 0xFFFF;
    t.in_blas = (st.y >> 16) & 1;
    t.opaque = (st.y >> 17) & 1;
    t.alpha_map = (st.y >> 18) & 1;
    t.inst = (uint32_t)st.z;
    t.alpha_inst = t.inst;
    t.iter = (uint32_t)st.w;
    t.throughput = h.x;
    t.alpha_pass = h.y;
    t.alpha_tex = __float_as_uint(h.z);
    if (t.in_blas)
        to_object(s.dinst + t.inst, t.world.o, t.world.d, t.r);
    else
        t.r = t.world;
    for (int k = 0; k < t.sp; k++)
        stack.set(k, pk.stack[(size_t)k * pk.cap + slot]);
}

template <bool W4>
static __device__ __forceinline__ float trace_shadow_inl(const DevScene& s, f3 o, f3 d, float tmin, float tmax, TraceCounters& tc)
{
    ShadowTrace t;
    TraceStack stack;
    shadow_begin(s, o, d, tmin, tmax, t, stack);
    while (!shadow_step<W4>(s, t, stack, tc)) {
    }
    return shadow_result(t);
}

// Out-of-line copies for the megakernel (keeps its code size down); the
// wavefront traversal kernels inline the traversal instead.  The node width
// follows the scene (4-wide when s.nodes4 is present).
template <bool W4>
static __device__ __noinline__ bool trace_closest_out(const DevScene& s, f3 o, f3 d, float tmin, float tmax, Hit& h, TraceCounters& tc)
{
    return trace_closest_inl<W4>(s, o, d, tmin, tmax, h, tc);
}
template <bool W4>
static __device__ __noinline__ float trace_shadow_out(const DevScene& s, f3 o, f3 d, float tmin, float tmax, TraceCounters& tc)
{
    return trace_shadow_inl<W4>(s, o, d, tmin, tmax, tc);
}
static __device__ __forceinline__ bool trace_closest(const DevScene& s, f3 o, f3 d, float tmin, float tmax, Hit& h, TraceCounters& tc)
{
    return s.nodes4 ? trace_closest_out<true>(s, o, d, tmin, tmax, h, tc) : trace_closest_out<false>(s, o, d, tmin, tmax, h, tc);
}
static __device__ __forceinline__ float trace_shadow(const DevScene& s, f3 o, f3 d, float tmin, float tmax, TraceCounters& tc)
{
    return s.nodes4 ? trace_shadow_out<true>(s, o, d, tmin, tmax, tc) : trace_shadow_out<false>(s, o, d, tmin, tmax, tc);
}

} // namespace pt
