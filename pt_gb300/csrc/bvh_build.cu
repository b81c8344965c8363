// bvh_build.cu — two-level BVH construction on the device.
//
// Replaces the driver's acceleration-structure build of the reference
// (vkCmdBuildAccelerationStructuresKHR, src/pathtrace/accstruct.cpp:57-61,
// 69-164 for the per-mesh BLAS, 186-286 for the TLAS).
//
// Method: linear BVH (Karras 2012, "Maximizing parallelism in the
// construction of BVHs, octrees, and k-d trees").  All meshes are built in a
// single pass: each primitive's 64-bit key is (segment << 48 | 48-bit Morton
// code of its centroid within the segment's centroid bounds), so after one
// radix sort every mesh is a contiguous key range and the binary radix tree
// over all keys contains, for every mesh, a node whose range is exactly that
// mesh (the mesh's BLAS root).  Nodes that straddle two meshes are never
// referenced.  Boxes are reduced bottom-up with one atomic counter per node,
// then every node is written with both child boxes padded outward (relative
// 1e-5 of the largest coordinate) so the traversal's box tests stay
// conservative.  The TLAS is the same construction over instance world boxes
// with one segment.
//
// Default topology: PLOC (Meister & Bittner 2018, "Parallel locally-ordered
// clustering for bounding volume hierarchy construction") on the same sorted
// keys: every primitive starts as a cluster; each round, every cluster finds
// the neighbour within a window of positions (same segment) whose merged box
// has the smallest surface area (ties broken by the lower index pair, so the
// globally closest pair in each segment is always mutual), mutual nearest
// neighbours merge into a new node, and the survivors are compacted in
// order, until each segment is one cluster.  Nodes are numbered in merge
// order by prefix sums (deterministic).  PT_BVH=lbvh selects the radix tree
// instead (kept for A/B).
#include <cub/cub.cuh>
#include <cstdlib>
#include <cstring>

#include "device/scene.cuh"
#include "kernels.h"

namespace pt {

namespace {

constexpr int MORTON_BITS = 16;           // per axis
constexpr int KEY_SEG_SHIFT = 3 * MORTON_BITS;

__device__ __forceinline__ int f2ord(float f)
{
    int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7FFFFFFF;
}
__device__ __forceinline__ float ord2f(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7FFFFFFF); }

// Spread the 16 bits of v to every third bit (bit b -> bit 3b), 48 bits wide.
__host__ __device__ __forceinline__ uint64_t expand_bits16(uint32_t v)
{
    uint64_t x = v & 0xFFFFu;
    x = (x | (x << 16)) & 0x0000FF0000FFull;
    x = (x | (x << 8)) & 0x00F00F00F00Full;
    x = (x | (x << 4)) & 0x0C30C30C30C3ull;
    x = (x | (x << 2)) & 0x249249249249ull;
    return x;
}

__device__ __forceinline__ uint32_t upper_segment(const uint32_t* base, uint32_t nseg, uint32_t g)
{
    // largest m with base[m] <= g (base has nseg + 1 entries, base[0] = 0)
    uint32_t lo = 0, hi = nseg;
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (base[mid] <= g)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

struct Scratch {
    float4* lo;      // primitive boxes
    float4* hi;
    uint32_t* seg;   // segment of each primitive
    uint64_t* keys_in;
    uint64_t* keys_out;
    uint32_t* vals_in;
    uint32_t* vals_out;
    int* parent;       // internal nodes (n - 1)
    int* leaf_parent;  // leaves (n)
    int* child0;
    int* child1;
    uint32_t* flags;
    float4* nlo;     // internal node boxes (unpadded)
    float4* nhi;
    int* seg_cb;     // 6 ints per segment: centroid bounds (ordered ints)
    int* seg_box;    // 6 ints per segment: primitive bounds
    uint32_t* seg_base; // segment begin (nseg + 1)
    int* seg_root;
    void* cub_temp;
    size_t cub_bytes;
    // PLOC clusters (double-buffered) and per-round flags / prefix sums
    int* c_ref[2];
    float4* c_lo[2];
    float4* c_hi[2];
    uint32_t* c_seg[2];
    int* nn;
    uint32_t* m_flag;
    uint32_t* a_flag;
    uint32_t* m_scan;
    uint32_t* a_scan;
    uint32_t* counters; // [0] nodes emitted, [1] live clusters, [2] merges in the last round,
                        // [3] 1 once a round merged nothing, [4] buffer holding the clusters
    void* scan_temp;
    size_t scan_bytes;
    // leaf collapse of the BLAS trees
    uint32_t* cnt;      // triangles under a node
    float* sah;         // SAH cost of a node's best form
    uint32_t* collapse; // 1: the node is cheaper as one leaf
    uint32_t* newpos;   // depth-first position of each triangle (sorted position -> TriRec slot)
    uint32_t* node_off; // depth-first position of a node's first triangle
    uint32_t* visits;   // bottom-up arrival counters
    uint32_t blas_nodes; // host: BLAS nodes emitted by PLOC
};

template <typename T>
T* carve(char*& p, size_t count)
{
    uintptr_t a = ((uintptr_t)p + 255) & ~(uintptr_t)255;
    T* r = (T*)a;
    p = (char*)(a + count * sizeof(T));
    return r;
}

size_t cub_sort_bytes(uint32_t n)
{
    size_t bytes = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, bytes, (uint64_t*)nullptr, (uint64_t*)nullptr, (uint32_t*)nullptr, (uint32_t*)nullptr,
                                    (int)n, 0, 64);
    return bytes;
}

size_t cub_scan_bytes(uint32_t n)
{
    size_t bytes = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, bytes, (uint32_t*)nullptr, (uint32_t*)nullptr, (int)n);
    return bytes;
}

Scratch carve_scratch(void* base, uint32_t n, uint32_t nseg)
{
    char* p = (char*)base;
    Scratch s;
    uint32_t nn = n > 0 ? n : 1;
    s.lo = carve<float4>(p, nn);
    s.hi = carve<float4>(p, nn);
    s.seg = carve<uint32_t>(p, nn);
    s.keys_in = carve<uint64_t>(p, nn);
    s.keys_out = carve<uint64_t>(p, nn);
    s.vals_in = carve<uint32_t>(p, nn);
    s.vals_out = carve<uint32_t>(p, nn);
    s.parent = carve<int>(p, nn);
    s.leaf_parent = carve<int>(p, nn);
    s.child0 = carve<int>(p, nn);
    s.child1 = carve<int>(p, nn);
    s.flags = carve<uint32_t>(p, nn);
    s.nlo = carve<float4>(p, nn);
    s.nhi = carve<float4>(p, nn);
    s.seg_cb = carve<int>(p, 6 * (size_t)(nseg + 1));
    s.seg_box = carve<int>(p, 6 * (size_t)(nseg + 1));
    s.seg_base = carve<uint32_t>(p, nseg + 2);
    s.seg_root = carve<int>(p, nseg + 1);
    for (int b = 0; b < 2; b++) {
        s.c_ref[b] = carve<int>(p, nn);
        s.c_lo[b] = carve<float4>(p, nn);
        s.c_hi[b] = carve<float4>(p, nn);
        s.c_seg[b] = carve<uint32_t>(p, nn);
    }
    s.nn = carve<int>(p, nn);
    s.m_flag = carve<uint32_t>(p, nn);
    s.a_flag = carve<uint32_t>(p, nn);
    s.m_scan = carve<uint32_t>(p, nn);
    s.a_scan = carve<uint32_t>(p, nn);
    s.counters = carve<uint32_t>(p, 8);
    s.cnt = carve<uint32_t>(p, nn);
    s.sah = carve<float>(p, nn);
    s.collapse = carve<uint32_t>(p, nn);
    s.newpos = carve<uint32_t>(p, nn);
    s.node_off = carve<uint32_t>(p, nn);
    s.visits = carve<uint32_t>(p, nn);
    s.blas_nodes = 0;
    s.scan_bytes = cub_scan_bytes(nn);
    s.scan_temp = carve<char>(p, s.scan_bytes);
    s.cub_bytes = cub_sort_bytes(nn);
    s.cub_temp = carve<char>(p, s.cub_bytes);
    return s;
}

size_t scratch_bytes_for(uint32_t n, uint32_t nseg)
{
    Scratch s = carve_scratch((void*)0, n, nseg);
    return (size_t)((char*)s.cub_temp - (char*)0) + s.cub_bytes + 256;
}

__global__ void k_init_bounds(int* cb, int* box, int* roots, uint32_t nseg)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nseg)
        return;
    roots[i] = REF_EMPTY;
    for (int k = 0; k < 3; k++) {
        cb[6 * i + k] = f2ord(__int_as_float(0x7f800000));
        cb[6 * i + 3 + k] = f2ord(-__int_as_float(0x7f800000));
        box[6 * i + k] = f2ord(__int_as_float(0x7f800000));
        box[6 * i + 3 + k] = f2ord(-__int_as_float(0x7f800000));
    }
}

__device__ __forceinline__ void atomic_bounds(int* b, float4 lo, float4 hi)
{
    atomicMin(b + 0, f2ord(lo.x));
    atomicMin(b + 1, f2ord(lo.y));
    atomicMin(b + 2, f2ord(lo.z));
    atomicMax(b + 3, f2ord(hi.x));
    atomicMax(b + 4, f2ord(hi.y));
    atomicMax(b + 5, f2ord(hi.z));
}

__global__ void k_tri_boxes(BvhBuildInput in, Scratch s)
{
    uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= in.tri_count)
        return;
    uint32_t m = upper_segment(in.mesh_tri_base, in.mesh_count, g);
    uint32_t local = g - in.mesh_tri_base[m];
    uint32_t ib = in.mesh_index_offset[m] + 3 * local;
    uint32_t vb = in.mesh_vertex_offset[m];
    float4 a = in.vertices[2 * (size_t)(vb + in.indices[ib + 0])];
    float4 b = in.vertices[2 * (size_t)(vb + in.indices[ib + 1])];
    float4 c = in.vertices[2 * (size_t)(vb + in.indices[ib + 2])];
    float4 lo = make_float4(fminf(fminf(a.x, b.x), c.x), fminf(fminf(a.y, b.y), c.y), fminf(fminf(a.z, b.z), c.z), 0.0f);
    float4 hi = make_float4(fmaxf(fmaxf(a.x, b.x), c.x), fmaxf(fmaxf(a.y, b.y), c.y), fmaxf(fmaxf(a.z, b.z), c.z), 0.0f);
    s.lo[g] = lo;
    s.hi[g] = hi;
    s.seg[g] = m;
    float4 cen = make_float4(0.5f * (lo.x + hi.x), 0.5f * (lo.y + hi.y), 0.5f * (lo.z + hi.z), 0.0f);
    atomic_bounds(s.seg_cb + 6 * m, cen, cen);
    atomic_bounds(s.seg_box + 6 * m, lo, hi);
}

// World box of each instance: the 8 corners of its mesh box under the
// object-to-world transform, padded.
__global__ void k_inst_boxes(BvhBuildInput in, const int* mesh_box, Scratch s)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= in.instance_count)
        return;
    uint32_t m = in.inst_mesh[i];
    const int* mb = mesh_box + 6 * m;
    float blo[3] = {ord2f(mb[0]), ord2f(mb[1]), ord2f(mb[2])};
    float bhi[3] = {ord2f(mb[3]), ord2f(mb[4]), ord2f(mb[5])};
    const DevInstanceData& d = in.inst_data[i];
    float4 rows[3] = {d.t0, d.t1, d.t2};
    float4 lo = make_float4(__int_as_float(0x7f800000), __int_as_float(0x7f800000), __int_as_float(0x7f800000), 0.0f);
    float4 hi = make_float4(-lo.x, -lo.y, -lo.z, 0.0f);
    if (!(blo[0] <= bhi[0])) {
        // empty mesh: a point at the instance origin (its BLAS root is empty)
        lo = make_float4(rows[0].w, rows[1].w, rows[2].w, 0.0f);
        hi = lo;
    } else {
        for (int corner = 0; corner < 8; corner++) {
            double p[3] = {(corner & 1) ? bhi[0] : blo[0], (corner & 2) ? bhi[1] : blo[1], (corner & 4) ? bhi[2] : blo[2]};
            float w[3];
            for (int r = 0; r < 3; r++)
                w[r] = (float)((double)rows[r].x * p[0] + (double)rows[r].y * p[1] + (double)rows[r].z * p[2] + (double)rows[r].w);
            lo.x = fminf(lo.x, w[0]);
            lo.y = fminf(lo.y, w[1]);
            lo.z = fminf(lo.z, w[2]);
            hi.x = fmaxf(hi.x, w[0]);
            hi.y = fmaxf(hi.y, w[1]);
            hi.z = fmaxf(hi.z, w[2]);
        }
    }
    s.lo[i] = lo;
    s.hi[i] = hi;
    s.seg[i] = 0;
    float4 cen = make_float4(0.5f * (lo.x + hi.x), 0.5f * (lo.y + hi.y), 0.5f * (lo.z + hi.z), 0.0f);
    atomic_bounds(s.seg_cb, cen, cen);
}

__global__ void k_morton(Scratch s, uint32_t n)
{
    uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n)
        return;
    uint32_t m = s.seg[g];
    const int* cb = s.seg_cb + 6 * m;
    float4 lo = s.lo[g], hi = s.hi[g];
    float c[3] = {0.5f * (lo.x + hi.x), 0.5f * (lo.y + hi.y), 0.5f * (lo.z + hi.z)};
    uint32_t q[3];
    for (int k = 0; k < 3; k++) {
        float a = ord2f(cb[k]), b = ord2f(cb[3 + k]);
        float x = (b > a) ? (c[k] - a) / (b - a) : 0.0f;
        x = fminf(fmaxf(x, 0.0f), 1.0f);
        q[k] = (uint32_t)(x * 65535.0f);
    }
    uint64_t code = (expand_bits16(q[0]) << 2) | (expand_bits16(q[1]) << 1) | expand_bits16(q[2]);
    s.keys_in[g] = ((uint64_t)m << KEY_SEG_SHIFT) | code;
    s.vals_in[g] = g;
}

__device__ __forceinline__ int delta(const uint64_t* keys, int n, int i, int j)
{
    if (j < 0 || j >= n)
        return -1;
    uint64_t a = keys[i], b = keys[j];
    if (a != b)
        return __clzll((long long)(a ^ b));
    return 64 + __clz(i ^ j);
}

// Karras 2012, Algorithm 1 (node ranges and splits of the binary radix tree).
__global__ void k_karras(Scratch s, int n, int node_base, int mode_tlas)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1)
        return;
    const uint64_t* keys = s.keys_out;
    int d = (delta(keys, n, i, i + 1) - delta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
    int dmin = delta(keys, n, i, i - d);
    int lmax = 2;
    while (delta(keys, n, i, i + lmax * d) > dmin)
        lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (delta(keys, n, i, i + (l + t) * d) > dmin)
            l += t;
    int j = i + l * d;
    int dnode = delta(keys, n, i, j);
    int sp = 0;
    for (int div = 2;; div <<= 1) {
        int t = (l + div - 1) / div;
        if (delta(keys, n, i, i + (sp + t) * d) > dnode)
            sp += t;
        if (t <= 1)
            break;
    }
    int gamma = i + sp * d + min(d, 0);
    int lo = min(i, j), hi = max(i, j);
    int c0 = (lo == gamma) ? ~gamma : gamma;
    int c1 = (hi == gamma + 1) ? ~(gamma + 1) : gamma + 1;
    s.child0[i] = c0;
    s.child1[i] = c1;
    if (c0 >= 0)
        s.parent[c0] = i;
    else
        s.leaf_parent[~c0] = i;
    if (c1 >= 0)
        s.parent[c1] = i;
    else
        s.leaf_parent[~c1] = i;
    uint32_t seg_lo = (uint32_t)(keys[lo] >> KEY_SEG_SHIFT), seg_hi = (uint32_t)(keys[hi] >> KEY_SEG_SHIFT);
    // flags: bit 31 marks a node that straddles two segments
    s.flags[i] = (seg_lo != seg_hi) ? 0x80000000u : 0u;
    if (seg_lo == seg_hi && (uint32_t)lo == s.seg_base[seg_lo] && (uint32_t)hi + 1 == s.seg_base[seg_lo + 1])
        s.seg_root[seg_lo] = node_base + i;
    (void)mode_tlas;
}

// Segments with zero or one primitive have no internal root.
__global__ void k_small_roots(Scratch s, uint32_t nseg, int mode_tlas)
{
    uint32_t m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nseg)
        return;
    uint32_t b = s.seg_base[m], e = s.seg_base[m + 1];
    if (e == b)
        s.seg_root[m] = REF_EMPTY;
    else if (e - b == 1)
        s.seg_root[m] = mode_tlas ? make_leaf(s.vals_out[b], 1) : make_leaf(b, 1);
}

__global__ void k_bottom_up(Scratch s, int n)
{
    int pos = blockIdx.x * blockDim.x + threadIdx.x;
    if (pos >= n || n < 2)
        return;
    int node = s.leaf_parent[pos];
    while (node >= 0) {
        if (s.flags[node] & 0x80000000u)
            return; // straddling node: above every mesh root
        __threadfence();
        uint32_t old = atomicAdd(&s.flags[node], 1u);
        if ((old & 0xFFu) == 0)
            return; // first arrival; the sibling finishes this node
        float4 lo = make_float4(__int_as_float(0x7f800000), __int_as_float(0x7f800000), __int_as_float(0x7f800000), 0.0f);
        float4 hi = make_float4(-lo.x, -lo.y, -lo.z, 0.0f);
        int cs[2] = {s.child0[node], s.child1[node]};
        for (int k = 0; k < 2; k++) {
            float4 a, b;
            if (cs[k] < 0) {
                uint32_t p = s.vals_out[~cs[k]];
                a = s.lo[p];
                b = s.hi[p];
            } else {
                a = __ldcg(s.nlo + cs[k]);
                b = __ldcg(s.nhi + cs[k]);
            }
            lo.x = fminf(lo.x, a.x);
            lo.y = fminf(lo.y, a.y);
            lo.z = fminf(lo.z, a.z);
            hi.x = fmaxf(hi.x, b.x);
            hi.y = fmaxf(hi.y, b.y);
            hi.z = fmaxf(hi.z, b.z);
        }
        __stcg(s.nlo + node, lo);
        __stcg(s.nhi + node, hi);
        __threadfence();
        node = s.parent[node];
    }
}

__device__ __forceinline__ void padded(float4 lo, float4 hi, float4& plo, float4& phi)
{
    float mag = fmaxf(fmaxf(fmaxf(fabsf(lo.x), fabsf(hi.x)), fmaxf(fabsf(lo.y), fabsf(hi.y))), fmaxf(fabsf(lo.z), fabsf(hi.z)));
    float eps = mag * 1e-5f + 1e-30f;
    plo = make_float4(lo.x - eps, lo.y - eps, lo.z - eps, 0.0f);
    phi = make_float4(hi.x + eps, hi.y + eps, hi.z + eps, 0.0f);
}

__global__ void k_emit_nodes(Scratch s, int n, BvhNode* nodes, int node_base, int mode_tlas)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1)
        return;
    if (s.flags[i] & 0x80000000u)
        return;
    int cs[2] = {s.child0[i], s.child1[i]};
    float4 blo[2], bhi[2];
    int ref[2];
    for (int k = 0; k < 2; k++) {
        float4 a, b;
        if (cs[k] < 0) {
            int pos = ~cs[k];
            uint32_t p = s.vals_out[pos];
            a = s.lo[p];
            b = s.hi[p];
            ref[k] = mode_tlas ? make_leaf(p, 1) : make_leaf((uint32_t)pos, 1);
        } else {
            a = s.nlo[cs[k]];
            b = s.nhi[cs[k]];
            ref[k] = node_base + cs[k];
        }
        padded(a, b, blo[k], bhi[k]);
    }
    BvhNode nd;
    nd.c0xy = make_float4(blo[0].x, bhi[0].x, blo[0].y, bhi[0].y);
    nd.c1xy = make_float4(blo[1].x, bhi[1].x, blo[1].y, bhi[1].y);
    nd.c01z = make_float4(blo[0].z, bhi[0].z, blo[1].z, bhi[1].z);
    nd.link = make_int4(ref[0], ref[1], 0, 0);
    nodes[node_base + i] = nd;
}

// ---- PLOC
// Neighbour windows of the BLAS and TLAS passes: PT_PLOC_RADIUS and
// PT_PLOC_RADIUS_TLAS (1..256), default 64 for both (measured on the mid and
// heavy scenes against 8..256; wider windows did not lower node visits).
int env_radius(const char* name, int dflt)
{
    const char* e = std::getenv(name);
    const int r = e ? std::atoi(e) : dflt;
    return r < 1 ? 1 : (r > 256 ? 256 : r);
}

int ploc_radius(int mode_tlas)
{
    static const int blas = env_radius("PT_PLOC_RADIUS", 64);
    static const int tlas = env_radius("PT_PLOC_RADIUS_TLAS", 64);
    return mode_tlas ? tlas : blas;
}

__device__ __forceinline__ float half_area(float4 lo, float4 hi)
{
    const float dx = hi.x - lo.x, dy = hi.y - lo.y, dz = hi.z - lo.z;
    return dx * dy + dy * dz + dz * dx;
}

__device__ __forceinline__ float4 box_min(float4 a, float4 b) { return make_float4(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z), 0.0f); }
__device__ __forceinline__ float4 box_max(float4 a, float4 b) { return make_float4(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z), 0.0f); }

// Initial clusters: one per primitive, in sorted order.
__global__ void k_ploc_init(Scratch s, uint32_t n, int mode_tlas)
{
    uint32_t pos = blockIdx.x * blockDim.x + threadIdx.x;
    if (pos >= n)
        return;
    const uint32_t p = s.vals_out[pos];
    s.c_ref[0][pos] = mode_tlas ? make_leaf(p, 1) : make_leaf(pos, 1);
    s.c_lo[0][pos] = s.lo[p];
    s.c_hi[0][pos] = s.hi[p];
    s.c_seg[0][pos] = (uint32_t)(s.keys_out[pos] >> KEY_SEG_SHIFT);
}

// (min, max) index pair order for ties between equal distances
__device__ __forceinline__ bool pair_before(int i, int j, int k)
{
    const int a0 = min(i, j), a1 = max(i, j), b0 = min(i, k), b1 = max(i, k);
    return a0 < b0 || (a0 == b0 && a1 < b1);
}

// The round kernels read the live cluster count (counters[1]) and whether
// the rounds are over (counters[3]) from device memory, so rounds run back to
// back without the host; grids and scans cover `cap` >= live positions.
__global__ void k_ploc_nn(const float4* lo, const float4* hi, const uint32_t* seg, const uint32_t* counters, int radius, int* nn)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = (int)counters[1];
    if (counters[3] || i >= n)
        return;
    const float4 li = lo[i], hi_i = hi[i];
    const uint32_t si = seg[i];
    float best = 0.0f;
    int bj = -1;
    const int j0 = max(0, i - radius), j1 = min(n - 1, i + radius);
    for (int j = j0; j <= j1; j++) {
        if (j == i || seg[j] != si)
            continue;
        const float d = half_area(box_min(li, lo[j]), box_max(hi_i, hi[j]));
        if (bj < 0 || d < best || (d == best && pair_before(i, j, bj))) {
            best = d;
            bj = j;
        }
    }
    nn[i] = bj;
}

// Mutual nearest neighbours merge; the lower index of a pair keeps the merged
// cluster.  Positions past the live count get zero flags (the scans cover cap).
__global__ void k_ploc_flags(const int* nn, const uint32_t* counters, int cap, uint32_t* m_flag, uint32_t* a_flag)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cap || counters[3])
        return;
    if (i >= (int)counters[1]) {
        m_flag[i] = 0u;
        a_flag[i] = 0u;
        return;
    }
    const int j = nn[i];
    const bool mutual = j >= 0 && nn[j] == i;
    m_flag[i] = (mutual && i < j) ? 1u : 0u;
    a_flag[i] = (mutual && i > j) ? 0u : 1u;
}

__global__ void k_ploc_merge(Scratch s, int cur, BvhNode* nodes, int node_base)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (s.counters[3] || i >= (int)s.counters[1] || !s.a_flag[i])
        return;
    const int nxt = cur ^ 1;
    const uint32_t o = s.a_scan[i];
    const float4 lo = s.c_lo[cur][i], hi = s.c_hi[cur][i];
    if (s.m_flag[i]) {
        const int j = s.nn[i];
        const float4 lo_j = s.c_lo[cur][j], hi_j = s.c_hi[cur][j];
        const int node = (int)(s.counters[0] + s.m_scan[i]);
        float4 blo[2], bhi[2];
        padded(lo, hi, blo[0], bhi[0]);
        padded(lo_j, hi_j, blo[1], bhi[1]);
        BvhNode nd;
        nd.c0xy = make_float4(blo[0].x, bhi[0].x, blo[0].y, bhi[0].y);
        nd.c1xy = make_float4(blo[1].x, bhi[1].x, blo[1].y, bhi[1].y);
        nd.c01z = make_float4(blo[0].z, bhi[0].z, blo[1].z, bhi[1].z);
        nd.link = make_int4(s.c_ref[cur][i], s.c_ref[cur][j], 0, 0);
        nodes[node_base + node] = nd;
        s.c_ref[nxt][o] = node_base + node;
        s.c_lo[nxt][o] = box_min(lo, lo_j);
        s.c_hi[nxt][o] = box_max(hi, hi_j);
    } else {
        s.c_ref[nxt][o] = s.c_ref[cur][i];
        s.c_lo[nxt][o] = lo;
        s.c_hi[nxt][o] = hi;
    }
    s.c_seg[nxt][o] = s.c_seg[cur][i];
}

// End of a round: the clusters now sit in buffer `nxt`; a round without a
// merge ends the rounds (every non-empty segment is one cluster).
__global__ void k_ploc_count(Scratch s, int nxt)
{
    if (s.counters[3])
        return;
    const int n = (int)s.counters[1];
    const uint32_t merges = s.m_scan[n - 1] + s.m_flag[n - 1];
    s.counters[0] += merges;
    s.counters[1] = s.a_scan[n - 1] + s.a_flag[n - 1];
    s.counters[2] = merges;
    s.counters[4] = (uint32_t)nxt;
    if (merges == 0 || s.counters[1] <= 1)
        s.counters[3] = 1u;
}

__global__ void k_ploc_roots(Scratch s)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int cur = (int)s.counters[4];
    if (i < (int)s.counters[1])
        s.seg_root[s.c_seg[cur][i]] = s.c_ref[cur][i];
}

// ---- SAH leaf collapse of the BLAS trees (PLOC output, leaves of one triangle)
constexpr int TREE_DEPTH_CAP = 1 << 16; // walks of a valid tree end far earlier
// Cost model (unnormalised SAH): leaf of n triangles = CT * n * A, interior
// node = CI * A + cost(c0) + cost(c1), A the node's surface area.  A node
// whose best form is a leaf of at most LEAF_MAX triangles is collapsed; the
// triangles are then laid out depth-first so every leaf is a contiguous range.

__global__ void k_link_parents(Scratch s, const BvhNode* nodes, uint32_t nb)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nb)
        return;
    const int4 l = nodes[i].link;
    const int cs[2] = {l.x, l.y};
    for (int k = 0; k < 2; k++) {
        if (cs[k] >= 0)
            s.parent[cs[k]] = (int)i;
        else
            s.leaf_parent[leaf_first(cs[k])] = (int)i;
    }
    s.visits[i] = 0;
}

__device__ __forceinline__ float child_area(const BvhNode& nd, int k)
{
    return k == 0 ? half_area(make_float4(nd.c0xy.x, nd.c0xy.z, nd.c01z.x, 0.0f), make_float4(nd.c0xy.y, nd.c0xy.w, nd.c01z.y, 0.0f))
                  : half_area(make_float4(nd.c1xy.x, nd.c1xy.z, nd.c01z.z, 0.0f), make_float4(nd.c1xy.y, nd.c1xy.w, nd.c01z.w, 0.0f));
}

__device__ __forceinline__ float node_area(const BvhNode& nd)
{
    const float4 lo = make_float4(fminf(nd.c0xy.x, nd.c1xy.x), fminf(nd.c0xy.z, nd.c1xy.z), fminf(nd.c01z.x, nd.c01z.z), 0.0f);
    const float4 hi = make_float4(fmaxf(nd.c0xy.y, nd.c1xy.y), fmaxf(nd.c0xy.w, nd.c1xy.w), fmaxf(nd.c01z.y, nd.c01z.w), 0.0f);
    return half_area(lo, hi);
}

// Bottom-up from every triangle: the second arrival at a node evaluates it.
__global__ void k_sah_up(Scratch s, const BvhNode* nodes, uint32_t n, float ci, float ct, uint32_t leaf_max)
{
    const uint32_t pos = blockIdx.x * blockDim.x + threadIdx.x;
    if (pos >= n)
        return;
    int node = s.leaf_parent[pos];
    for (int depth = 0; node >= 0 && depth < TREE_DEPTH_CAP; depth++) {
        __threadfence();
        if (atomicAdd(&s.visits[node], 1u) == 0)
            return; // the sibling subtree finishes this node
        const BvhNode nd = nodes[node];
        const int cs[2] = {nd.link.x, nd.link.y};
        uint32_t cnt = 0;
        float sub = 0.0f;
        for (int k = 0; k < 2; k++) {
            if (cs[k] < 0) {
                cnt += 1;
                sub += ct * child_area(nd, k);
            } else {
                cnt += __ldcg(&s.cnt[cs[k]]);
                sub += __ldcg(&s.sah[cs[k]]);
            }
        }
        const float a = node_area(nd);
        const float inner = ci * a + sub;
        const float leaf = ct * (float)cnt * a;
        const bool col = cnt <= leaf_max && leaf <= inner;
        __stcg(&s.cnt[node], cnt);
        __stcg(&s.sah[node], col ? leaf : inner);
        __stcg(&s.collapse[node], col ? 1u : 0u);
        __threadfence();
        node = s.parent[node];
    }
}

// Depth-first positions: a triangle's (or node's) offset inside its mesh is
// the sum of the left siblings' triangle counts along the path to the root.
__device__ __forceinline__ uint32_t dfs_offset(const Scratch& s, const BvhNode* nodes, int node, int from_ref, int& root)
{
    uint32_t off = 0;
    int child = from_ref;
    for (int depth = 0; node >= 0 && depth < TREE_DEPTH_CAP; depth++) {
        const int4 l = nodes[node].link;
        if (child == l.y)
            off += l.x < 0 ? 1u : s.cnt[l.x];
        root = node;
        child = node;
        node = s.parent[node];
    }
    return off;
}

__global__ void k_dfs_positions(Scratch s, const BvhNode* nodes, uint32_t n)
{
    const uint32_t pos = blockIdx.x * blockDim.x + threadIdx.x;
    if (pos >= n)
        return;
    const uint32_t seg = (uint32_t)(s.keys_out[pos] >> KEY_SEG_SHIFT);
    int root = -1;
    const uint32_t off = dfs_offset(s, nodes, s.leaf_parent[pos], make_leaf(pos, 1), root);
    s.newpos[pos] = s.seg_base[seg] + off;
}

// A subtree's first depth-first slot is its leftmost triangle's.
__global__ void k_node_offsets(Scratch s, const BvhNode* nodes, uint32_t nb)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nb)
        return;
    int c = (int)i;
    for (int depth = 0; c >= 0 && depth < TREE_DEPTH_CAP; depth++)
        c = nodes[c].link.x;
    s.node_off[i] = c < 0 ? s.newpos[leaf_first(c)] : 0u;
}

__global__ void k_rewrite_links(Scratch s, BvhNode* nodes, uint32_t nb)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nb)
        return;
    int4 l = nodes[i].link;
    int* cs[2] = {&l.x, &l.y};
    for (int k = 0; k < 2; k++) {
        const int c = *cs[k];
        if (c < 0)
            *cs[k] = make_leaf(s.newpos[leaf_first(c)], 1);
        else if (s.collapse[c])
            *cs[k] = make_leaf(s.node_off[c], s.cnt[c]);
    }
    nodes[i].link = l;
}

__global__ void k_rewrite_roots(Scratch s, uint32_t nseg)
{
    const uint32_t m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nseg)
        return;
    const int r = s.seg_root[m];
    if (r >= 0) {
        if (s.collapse[r])
            s.seg_root[m] = make_leaf(s.node_off[r], s.cnt[r]);
    } else if (ref_is_leaf(r)) {
        s.seg_root[m] = make_leaf(s.newpos[leaf_first(r)], 1);
    }
}

__global__ void k_identity_positions(Scratch s, uint32_t n)
{
    const uint32_t pos = blockIdx.x * blockDim.x + threadIdx.x;
    if (pos < n)
        s.newpos[pos] = pos;
}

__global__ void k_write_tris(BvhBuildInput in, Scratch s, TriRec* tris)
{
    uint32_t pos = blockIdx.x * blockDim.x + threadIdx.x;
    if (pos >= in.tri_count)
        return;
    uint32_t g = s.vals_out[pos];
    uint32_t m = s.seg[g];
    uint32_t local = g - in.mesh_tri_base[m];
    uint32_t ib = in.mesh_index_offset[m] + 3 * local;
    uint32_t vb = in.mesh_vertex_offset[m];
    float4 a = in.vertices[2 * (size_t)(vb + in.indices[ib + 0])];
    float4 b = in.vertices[2 * (size_t)(vb + in.indices[ib + 1])];
    float4 c = in.vertices[2 * (size_t)(vb + in.indices[ib + 2])];
    TriRec r;
    r.v0 = make_float4(a.x, a.y, a.z, __uint_as_float(local));
    r.v1 = make_float4(b.x, b.y, b.z, 0.0f);
    r.v2 = make_float4(c.x, c.y, c.z, 0.0f);
    tris[s.newpos[pos]] = r;
}

__global__ void k_set_roots(BvhBuildInput in, const int* mesh_root, DevInstance* dinst)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= in.instance_count)
        return;
    uint32_t m = in.inst_mesh[i];
    dinst[i].blas_root = m < in.mesh_count ? mesh_root[m] : REF_EMPTY;
    dinst[i].mesh = m;
}

inline unsigned blocks(uint64_t n, unsigned t) { return (unsigned)((n + t - 1) / t); }

int bits_for(uint32_t v)
{
    int b = 0;
    while ((1ull << b) < (uint64_t)v)
        b++;
    return b;
}

bool use_ploc()
{
    static const bool v = [] {
        const char* e = std::getenv("PT_BVH");
        return !(e && std::strcmp(e, "lbvh") == 0);
    }();
    return v;
}

// The TLAS builder may differ (PT_BVH_TLAS=lbvh|ploc; default: as PT_BVH).
bool use_ploc_tlas()
{
    static const bool v = [] {
        const char* e = std::getenv("PT_BVH_TLAS");
        if (e && std::strcmp(e, "lbvh") == 0)
            return false;
        if (e && std::strcmp(e, "ploc") == 0)
            return true;
        return use_ploc();
    }();
    return v;
}

// PLOC rounds over the sorted primitives; they end when a round merges
// nothing (then every non-empty segment is one cluster).  The rounds run in
// chunks of PLOC_CHUNK back to back on the device (a round after the end does
// nothing); the host reads the counters once per chunk, not once per round.
constexpr uint32_t PLOC_CHUNK = 8;

cudaError_t build_ploc(Scratch& s, uint32_t n, BvhNode* nodes, int node_base, int mode_tlas, cudaStream_t st)
{
    k_ploc_init<<<blocks(n, 256), 256, 0, st>>>(s, n, mode_tlas);
    cudaMemsetAsync(s.counters, 0, 8 * sizeof(uint32_t), st);
    const uint32_t init[4] = {0u, n, 0u, n <= 1 ? 1u : 0u};
    cudaError_t e = cudaMemcpyAsync(s.counters, init, sizeof(init), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess)
        return e;
    int cur = 0;
    uint32_t cap = n, rounds = 0;
    uint32_t c[5] = {0u, n, 0u, n <= 1 ? 1u : 0u, 0u};
    while (!c[3]) {
        if (rounds > n + PLOC_CHUNK)
            return cudaErrorUnknown; // every round merges at least one pair while a segment has two clusters
        for (uint32_t k = 0; k < PLOC_CHUNK; k++, rounds++) {
            k_ploc_nn<<<blocks(cap, 128), 128, 0, st>>>(s.c_lo[cur], s.c_hi[cur], s.c_seg[cur], s.counters,
                                                          ploc_radius(mode_tlas), s.nn);
            k_ploc_flags<<<blocks(cap, 256), 256, 0, st>>>(s.nn, s.counters, (int)cap, s.m_flag, s.a_flag);
            size_t bytes = s.scan_bytes;
            e = cub::DeviceScan::ExclusiveSum(s.scan_temp, bytes, s.m_flag, s.m_scan, (int)cap, st);
            if (e == cudaSuccess)
                e = cub::DeviceScan::ExclusiveSum(s.scan_temp, bytes, s.a_flag, s.a_scan, (int)cap, st);
            if (e != cudaSuccess)
                return e;
            k_ploc_merge<<<blocks(cap, 128), 128, 0, st>>>(s, cur, nodes, node_base);
            k_ploc_count<<<1, 1, 0, st>>>(s, cur ^ 1);
            cur ^= 1;
        }
        e = cudaMemcpyAsync(c, s.counters, 5 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(st);
        if (e != cudaSuccess)
            return e;
        cap = c[1];
    }
    s.blas_nodes = c[0];
    k_ploc_roots<<<blocks(c[1], 128), 128, 0, st>>>(s);
    return cudaGetLastError();
}

float env_float(const char* name, float dflt)
{
    const char* e = std::getenv(name);
    return e ? (float)std::atof(e) : dflt;
}

// Collapses the BLAS trees of `nb` nodes over n triangles and fills newpos
// (identity when collapse is off: PT_LEAF_MAX=1 or the radix tree).
cudaError_t collapse_leaves(Scratch& s, uint32_t n, uint32_t nseg, BvhNode* nodes, uint32_t nb, cudaStream_t st)
{
    // Off by default (PT_LEAF_MAX=1): on the mid scene leaves of up to 2-4
    // triangles cut node visits per ray from 28.8 to 27.4 but raised triangle
    // tests from 2.5 to 2.9 and ran 1 % slower (11 % slower at PT_SAH_CT=0.5).
    static const uint32_t leaf_max = (uint32_t)std::min(4, std::max(1, (int)env_float("PT_LEAF_MAX", 1.0f)));
    static const float ct = env_float("PT_SAH_CT", 1.0f);
    if (n == 0)
        return cudaSuccess;
    if (!use_ploc() || leaf_max <= 1 || nb == 0) {
        k_identity_positions<<<blocks(n, 256), 256, 0, st>>>(s, n);
        return cudaGetLastError();
    }
    cudaMemsetAsync(s.parent, 0xFF, sizeof(int) * nb, st);
    cudaMemsetAsync(s.leaf_parent, 0xFF, sizeof(int) * n, st); // single-triangle meshes have no parent node
    k_link_parents<<<blocks(nb, 256), 256, 0, st>>>(s, nodes, nb);
    k_sah_up<<<blocks(n, 256), 256, 0, st>>>(s, nodes, n, 1.0f, ct, leaf_max);
    k_dfs_positions<<<blocks(n, 256), 256, 0, st>>>(s, nodes, n);
    k_node_offsets<<<blocks(nb, 256), 256, 0, st>>>(s, nodes, nb);
    k_rewrite_links<<<blocks(nb, 256), 256, 0, st>>>(s, nodes, nb);
    k_rewrite_roots<<<blocks(nseg, 128), 128, 0, st>>>(s, nseg);
    return cudaGetLastError();
}

// Sort + tree topology + node emission for one key set.
cudaError_t build_tree(Scratch& s, uint32_t n, uint32_t nseg, BvhNode* nodes, int node_base, int mode_tlas, cudaStream_t st)
{
    if (n == 0) {
        k_small_roots<<<blocks(nseg, 128), 128, 0, st>>>(s, nseg, mode_tlas);
        return cudaGetLastError();
    }
    k_morton<<<blocks(n, 256), 256, 0, st>>>(s, n);
    int end_bit = KEY_SEG_SHIFT + bits_for(nseg);
    if (end_bit > 64)
        return cudaErrorInvalidValue;
    size_t bytes = s.cub_bytes;
    cudaError_t e = cub::DeviceRadixSort::SortPairs(s.cub_temp, bytes, s.keys_in, s.keys_out, s.vals_in, s.vals_out, (int)n, 0, end_bit, st);
    if (e != cudaSuccess)
        return e;
    if (mode_tlas ? use_ploc_tlas() : use_ploc()) {
        k_small_roots<<<blocks(nseg, 128), 128, 0, st>>>(s, nseg, mode_tlas);
        return build_ploc(s, n, nodes, node_base, mode_tlas, st);
    }
    cudaMemsetAsync(s.parent, 0xFF, sizeof(int) * n, st);
    if (n > 1)
        k_karras<<<blocks(n - 1, 256), 256, 0, st>>>(s, (int)n, node_base, mode_tlas);
    k_small_roots<<<blocks(nseg, 128), 128, 0, st>>>(s, nseg, mode_tlas);
    if (n > 1) {
        k_bottom_up<<<blocks(n, 256), 256, 0, st>>>(s, (int)n);
        k_emit_nodes<<<blocks(n - 1, 256), 256, 0, st>>>(s, (int)n, nodes, node_base, mode_tlas);
    }
    return cudaGetLastError();
}

} // namespace

size_t bvh_node_count(uint32_t tri_count, uint32_t instance_count)
{
    return (size_t)(tri_count > 1 ? tri_count - 1 : 0) + (instance_count > 1 ? instance_count - 1 : 0) + 1;
}

// 4-wide nodes from the finished BVH2, one per BVH2 node (same index): the
// children of node i's children in order (c00, c01, c10, c11), a child that
// is a leaf standing for itself.  (Filling the four slots greedily by box
// surface instead measured 1.3 % slower on the mid scene, and the order
// c00, c10, c01, c11 1.2 % slower: sibling boxes stay next to each other.)
// Boxes are the BVH2's rounded outwards to half precision (lower planes
// toward -inf, upper toward +inf), so every 4-wide box contains the one the
// BVH2 tests and no hit is lost; the node takes 64 bytes instead of 128 (mid
// scene 1,024x1,024 at 128 spp: 1,582 -> 1,609 Mpath-segs/s, heavy scene
// 470 -> 509, node visits per ray +3.7 %).  A plane beyond the half range
// (|x| > 65504) rounds to an infinity; the node stays conservative, but
// `*overflow` is set so that the caller traverses the BVH2 instead (an
// infinite plane times the infinite inverse direction of an axis-parallel ray
// gives NaN slab distances).  Slots of the node array that no tree uses hold
// zeros (the caller clears the array before the build); the bounds check
// keeps their derivation inside the array.
__global__ void k_make_bvh4(const BvhNode* nodes, uint32_t n, Bvh4Node* out, uint32_t* overflow)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const BvhNode nd = nodes[i];
    float b[6][4];
    int ref[4];
    int k = 0;
    auto put = [&](float4 xy, float zlo, float zhi, int r) {
        b[0][k] = xy.x;
        b[1][k] = xy.y;
        b[2][k] = xy.z;
        b[3][k] = xy.w;
        b[4][k] = zlo;
        b[5][k] = zhi;
        ref[k] = r;
        k++;
    };
    for (int c = 0; c < 2; c++) {
        const int cr = c == 0 ? nd.link.x : nd.link.y;
        if (cr >= 0 && (uint32_t)cr < n) {
            const BvhNode g = nodes[cr];
            put(g.c0xy, g.c01z.x, g.c01z.y, g.link.x);
            put(g.c1xy, g.c01z.z, g.c01z.w, g.link.y);
        } else if (c == 0) {
            put(nd.c0xy, nd.c01z.x, nd.c01z.y, cr);
        } else {
            put(nd.c1xy, nd.c01z.z, nd.c01z.w, cr);
        }
    }
    for (; k < 4; k++) {
        for (int a = 0; a < 6; a++)
            b[a][k] = 0.0f;
        ref[k] = REF_EMPTY;
    }
    Bvh4Node o;
    uint32_t q[6][2];
    for (int a = 0; a < 6; a++) {
        for (int j = 0; j < 2; j++) {
            // lower planes (even a) rounded toward -inf, upper toward +inf
            const __half h0 = (a & 1) ? __float2half_ru(b[a][2 * j]) : __float2half_rd(b[a][2 * j]);
            const __half h1 = (a & 1) ? __float2half_ru(b[a][2 * j + 1]) : __float2half_rd(b[a][2 * j + 1]);
            q[a][j] = (uint32_t)__half_as_ushort(h0) | ((uint32_t)__half_as_ushort(h1) << 16);
            if (__hisinf(h0) || __hisinf(h1))
                *overflow = 1u;
        }
    }
    o.x = make_uint4(q[0][0], q[0][1], q[1][0], q[1][1]);
    o.y = make_uint4(q[2][0], q[2][1], q[3][0], q[3][1]);
    o.z = make_uint4(q[4][0], q[4][1], q[5][0], q[5][1]);
    o.link = make_int4(ref[0], ref[1], ref[2], ref[3]);
    out[i] = o;
}

cudaError_t build_bvh4(const BvhNode* nodes, uint32_t n, Bvh4Node* out, uint32_t* overflow, cudaStream_t st)
{
    if (n == 0)
        return cudaSuccess;
    k_make_bvh4<<<blocks(n, 128), 128, 0, st>>>(nodes, n, out, overflow);
    return cudaGetLastError();
}

bool use_bvh4()
{
    static const bool on = [] {
        const char* e = std::getenv("PT_BVH_WIDTH");
        return !(e && std::atoi(e) == 2);
    }();
    return on;
}

size_t bvh_scratch_bytes(uint32_t mesh_count, uint32_t tri_count, uint32_t instance_count)
{
    uint32_t n = tri_count > instance_count ? tri_count : instance_count;
    uint32_t nseg = mesh_count > 1 ? mesh_count : 1;
    return scratch_bytes_for(n, nseg) + 6 * sizeof(int) * (size_t)(nseg + 1) + 512;
}

cudaError_t bvh_build(const BvhBuildInput& in, BvhBuildOutput& out, void* scratch, size_t scratch_bytes, cudaStream_t st)
{
    if (scratch_bytes < bvh_scratch_bytes(in.mesh_count, in.tri_count, in.instance_count))
        return cudaErrorInvalidValue;
    uint32_t n_max = in.tri_count > in.instance_count ? in.tri_count : in.instance_count;
    uint32_t nseg_max = in.mesh_count > 1 ? in.mesh_count : 1;
    Scratch s = carve_scratch(scratch, n_max, nseg_max);
    // per-mesh primitive boxes survive the TLAS pass: keep them after the scratch
    size_t used = (size_t)((char*)s.cub_temp - (char*)scratch) + s.cub_bytes;
    int* mesh_box = (int*)(((uintptr_t)scratch + used + 255) & ~(uintptr_t)255);
    cudaError_t e;

    // ---- BLAS: every mesh in one key set
    if (in.mesh_count > 0) {
        k_init_bounds<<<blocks(in.mesh_count, 128), 128, 0, st>>>(s.seg_cb, mesh_box, s.seg_root, in.mesh_count);
        cudaMemcpyAsync(s.seg_base, in.mesh_tri_base, sizeof(uint32_t) * (in.mesh_count + 1), cudaMemcpyDeviceToDevice, st);
        if (in.tri_count > 0) {
            Scratch sb = s;
            sb.seg_box = mesh_box;
            k_tri_boxes<<<blocks(in.tri_count, 256), 256, 0, st>>>(in, sb);
        }
        s.blas_nodes = 0;
        e = build_tree(s, in.tri_count, in.mesh_count, out.nodes, 0, 0, st);
        if (e == cudaSuccess)
            e = collapse_leaves(s, in.tri_count, in.mesh_count, out.nodes, s.blas_nodes, st);
        if (e != cudaSuccess)
            return e;
        if (in.tri_count > 0)
            k_write_tris<<<blocks(in.tri_count, 256), 256, 0, st>>>(in, s, out.tris);
        cudaMemcpyAsync(out.mesh_root, s.seg_root, sizeof(int) * in.mesh_count, cudaMemcpyDeviceToDevice, st);
    }
    if (in.instance_count == 0) {
        out.tlas_root = REF_EMPTY;
        return cudaGetLastError();
    }
    k_set_roots<<<blocks(in.instance_count, 128), 128, 0, st>>>(in, out.mesh_root, out.dinst);

    // ---- TLAS over instance world boxes (one segment)
    int tlas_base = (int)(in.tri_count > 1 ? in.tri_count - 1 : 0);
    uint32_t tb[2] = {0, in.instance_count};
    k_init_bounds<<<1, 32, 0, st>>>(s.seg_cb, s.seg_box, s.seg_root, 1);
    cudaMemcpyAsync(s.seg_base, tb, sizeof(tb), cudaMemcpyHostToDevice, st);
    k_inst_boxes<<<blocks(in.instance_count, 128), 128, 0, st>>>(in, mesh_box, s);
    e = build_tree(s, in.instance_count, 1, out.nodes, tlas_base, 1, st);
    if (e != cudaSuccess)
        return e;
    int root = REF_EMPTY;
    e = cudaMemcpyAsync(&root, s.seg_root, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess)
        return e;
    e = cudaStreamSynchronize(st);
    out.tlas_root = root;
    return e;
}

} // namespace pt
