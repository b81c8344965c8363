// render_wave.cu — wavefront path tracer.
//
// A wave renders `k` consecutive samples of every pixel: N = k * W * H paths.
// Path state lives in structure-of-arrays buffers indexed by path id; stages
// exchange compact queues of path ids:
//
//   raygen      camera rays of all N paths (pathtrace.rg.hlsl:18-35)
//   extend      closest hit of every queued path (TraceRay, rg.hlsl:35,51)
//   split       finishes escaped rays (pathtrace.ms.hlsl) and queues the hits
//   shade       hit shading up to the NEE shadow ray, BSDF sampling and
//               Russian roulette (pathtrace.ch.hlsl:227-360,
//               pathtrace.hlsli:118-139); pushes continuing paths and shadow
//               requests (ballot + popc per warp, one atomic per block)
//   shadow      any-hit traversal + the light term (ch.hlsl:190-224)
//   accumulate  running mean of the wave's samples in sample order
//               (rg.hlsl:59-67), optional FP64 sums
//
// The per-segment sampler needs no stored state: the reference restarts it at
// every segment from (pixel, sample, segment + 1) (rg.hlsl:45), so `shade`
// restarts it itself.  Radiance terms are added in the reference's order: the
// shadow stage of segment s runs before the shade stage of segment s + 1.
// Queue lengths stay on the device; every kernel reads its own count, so the
// host issues a fixed sequence of launches per wave (CUDA-graph friendly).
//
// The stages are templates over the source of a wave's paths: one render
// (`OneJob`: path id -> sample and pixel of the call's camera) or a batch
// (`ManyJobs`: a wave holds shares of several jobs, each with its own scene,
// camera, size and sample range; raygen records each path's share).
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "device/render.cuh"
#include "kernels.h"

namespace pt {

// Pixel and sample of a path, and the job it belongs to.
struct PathLoc {
    uint32_t job, pix, si;
};

struct OneJob {
    RenderArgs r;
    uint32_t first_sample; // sample index of path ids [0, W*H)
    uint32_t samples;      // k
    uint32_t pixels;       // W * H
    uint32_t n_paths;      // k * W * H
    __device__ __forceinline__ PathLoc assign(uint32_t p) const
    {
        uint32_t j = p / pixels;
        return PathLoc{0u, p - j * pixels, first_sample + j};
    }
    __device__ __forceinline__ PathLoc locate(uint32_t p) const { return assign(p); }
    __device__ __forceinline__ uint32_t job_of(uint32_t) const { return 0u; }
    __device__ __forceinline__ const RenderArgs& args(uint32_t) const { return r; }
    __device__ __forceinline__ unsigned long long* counters() const { return r.counters; }
    __device__ __forceinline__ uint32_t accum_threads() const { return pixels; }
    // the share (the whole wave) and the pixel of accumulation thread t
    __device__ __forceinline__ const WaveShare share_of_pixel(uint32_t t, uint32_t& pix) const
    {
        pix = t;
        return WaveShare{0u, 0u, 0u, first_sample, samples, pixels};
    }
};

struct ManyJobs {
    const RenderArgs* jobs;    // device table, one per job
    const WaveShare* shares;   // this wave's shares, ascending path_base / pixel_base
    uint32_t* path_share;      // per path: index of its share (written by raygen)
    uint32_t share_count;
    uint32_t n_paths;          // sum of the shares' samples * pixels
    uint32_t n_pixels;         // sum of the shares' pixels
    unsigned long long* ctr;   // batch counters
    __device__ __forceinline__ PathLoc from_share(uint32_t e, uint32_t p) const
    {
        const WaveShare& E = shares[e];
        uint32_t lp = p - E.path_base;
        uint32_t j = lp / E.pixels;
        return PathLoc{E.job, lp - j * E.pixels, E.first_sample + j};
    }
    __device__ __forceinline__ PathLoc assign(uint32_t p) const
    {
        uint32_t lo = 0, hi = share_count; // last share with path_base <= p
        while (hi - lo > 1) {
            uint32_t mid = (lo + hi) >> 1;
            if (shares[mid].path_base <= p)
                lo = mid;
            else
                hi = mid;
        }
        path_share[p] = lo;
        return from_share(lo, p);
    }
    __device__ __forceinline__ PathLoc locate(uint32_t p) const { return from_share(path_share[p], p); }
    __device__ __forceinline__ uint32_t job_of(uint32_t p) const { return shares[path_share[p]].job; }
    __device__ __forceinline__ const RenderArgs& args(uint32_t job) const { return jobs[job]; }
    __device__ __forceinline__ unsigned long long* counters() const { return ctr; }
    __device__ __forceinline__ uint32_t accum_threads() const { return n_pixels; }
    __device__ __forceinline__ const WaveShare share_of_pixel(uint32_t t, uint32_t& pix) const
    {
        uint32_t lo = 0, hi = share_count;
        while (hi - lo > 1) {
            uint32_t mid = (lo + hi) >> 1;
            if (shares[mid].pixel_base <= t)
                lo = mid;
            else
                hi = mid;
        }
        const WaveShare E = shares[lo];
        pix = t - E.pixel_base;
        return E;
    }
};

struct WaveState {
    // per path
    float4* ray_o;      // xyz origin, w = tmin
    float4* ray_d;      // xyz direction, w = tmax
    float4* tp;         // throughput xyz, w = brdf pdf (< 0 on the first ray)
    float4* rad;        // radiance xyz, w unused
    uint32_t* seg;      // current segment index
    float4* hit;        // t, b1, b2, bits(inst)
    uint32_t* hit_prim; // primitive, ~0 for a miss
    // NEE requests (per path, valid when queued in the shadow queue)
    float4* nee_o;      // origin, w = tmax
    float4* nee_d;      // direction, w = w (< 0: delta light)
    float4* nee_e;      // emission, w = cos_i
    float4* nee_b;      // brdf, w = pdf
    float4* nee_tp;     // throughput before the BSDF update
    float4* f_a;        // first-hit features (PT_RENDER_FEATURES): base colour, hit distance
    float4* f_n;        //   shading normal
    // queues
    uint32_t* queue[2];
    uint32_t* shadow_queue;
    uint32_t* hit_queue; // paths whose ray hit something this segment (shade's input)
    uint32_t* counts;   // [0],[1] path queues, [2] shadow queue, [3] work fetch, [4] shadow fetch, [5] hit queue,
                        // [6] parked closest-hit traversals, [7] their fetch, [8] parked shadow
                        // traversals, [9] their fetch
    TraceParking park;  // closest-hit traversals paused by the first extend pass
};

template <class Src>
struct WaveArgs {
    Src src;
    WaveState w;
};

// Two queue pushes for a whole block at once: one atomic per queue per block.
// Every thread of the block must call it (block-uniform control flow).
template <int WARPS>
__device__ __forceinline__ void push_block2(uint32_t* q0, uint32_t* n0, bool p0, uint32_t* q1, uint32_t* n1, bool p1,
                                            uint32_t value)
{
    __shared__ uint32_t s_off[2][WARPS];
    __shared__ uint32_t s_base[2];
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned m0 = __ballot_sync(0xffffffffu, p0), m1 = __ballot_sync(0xffffffffu, p1);
    if (lane == 0) {
        s_off[0][warp] = __popc(m0);
        s_off[1][warp] = __popc(m1);
    }
    __syncthreads();
    if (threadIdx.x < 2) {
        uint32_t total = 0;
        for (int w = 0; w < WARPS; w++) {
            const uint32_t c = s_off[threadIdx.x][w];
            s_off[threadIdx.x][w] = total;
            total += c;
        }
        s_base[threadIdx.x] = total ? atomicAdd(threadIdx.x == 0 ? n0 : n1, total) : 0u;
    }
    __syncthreads();
    const unsigned lt = (1u << lane) - 1u;
    if (p0)
        q0[s_base[0] + s_off[0][warp] + __popc(m0 & lt)] = value;
    if (p1)
        q1[s_base[1] + s_off[1][warp] + __popc(m1 & lt)] = value;
    __syncthreads();
}

template <class Src>
__global__ void __launch_bounds__(256) k_wf_raygen(WaveArgs<Src> a)
{
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < a.src.n_paths; p += gridDim.x * blockDim.x) {
        const PathLoc L = a.src.assign(p);
        const RenderArgs& R = a.src.args(L.job);
        uint32_t px = L.pix % R.width, py = L.pix / R.width;
        uint32_t si = L.si;
        Sampler smp;
        sampler_start(smp, px, py, si, 0);
        f2 u_pixel = sample_2d(smp);
        f2 u_lens = sample_2d(smp);
        f3 ro, rd;
        camera_ray(R, px, py, u_pixel, u_lens, ro, rd);
        a.w.ray_o[p] = make_float4(ro.x, ro.y, ro.z, R.near_plane);
        a.w.ray_d[p] = make_float4(rd.x, rd.y, rd.z, R.far_plane);
        a.w.tp[p] = make_float4(1.0f, 1.0f, 1.0f, -1.0f);
        a.w.rad[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        a.w.seg[p] = 0;
        a.w.queue[0][p] = p;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.w.counts[0] = a.src.n_paths;
        a.w.counts[1] = 0;
        a.w.counts[2] = 0;
        a.w.counts[3] = 0;
        a.w.counts[4] = 0;
        a.w.counts[5] = 0;
        a.w.counts[6] = 0;
        a.w.counts[7] = 0;
        a.w.counts[8] = 0;
        a.w.counts[9] = 0;
    }
}

// Checked builds: a queue entry must name a path of the wave; a bad one sets
// ERR_BAD_INDEX and the entry is dropped (`valid` cleared) instead of used.
#ifdef PT_CHECKED
#define PT_CHECK_ENTRY(valid, p, a)                                      \
    if ((valid) && (p) >= (a).src.n_paths) {                             \
        atomicOr((a).src.args(0u).s.error_word, ERR_BAD_INDEX);         \
        (valid) = false;                                                 \
        (p) = 0u;                                                        \
    }
#else
#define PT_CHECK_ENTRY(valid, p, a)
#endif

// Closest-hit traversal of a launch: over the 4-wide nodes, the BVH2 one
// node-or-leaf step per iteration, or the BVH2 while-while with speculative
// leaves.
enum Traversal : int { TRAV_BVH4 = 0, TRAV_BVH2 = 1, TRAV_BVH2_WW = 2 };

// Persistent traversal: warps fetch 32 queue entries at a time.
// Only traces: k_wf_split then separates hits from misses.
//
// With a step budget (4-wide nodes, budget > 0) this is the first of two
// passes: a ray still traversing after `budget` steps is parked (its state
// saved to a slot of a.w.park, slots taken by one atomic per warp) and the
// lane moves on, so a warp's rays no longer wait for its slowest one;
// k_wf_extend_resume finishes the parked rays 32 to a warp.  A ray whose stack
// is deeper than PARK_STACK, or that finds no free slot, finishes here.  The
// hit is the same either way: the resumed traversal continues the same
// sequence of steps.
// Residency: 8 blocks of 128 per SM (64 registers, 40-52 B of spills) over
// the half-precision 4-wide nodes; 7 blocks measured 74.2 against 71.9 ms of
// extend per step on the mid scene (the shadow kernel is faster at 7).
template <class Src, int TRAV, bool BUDGET = false>
__global__ void __launch_bounds__(128, TRAV == TRAV_BVH4 ? 8 : 1) k_wf_extend(WaveArgs<Src> a, uint32_t qi, uint32_t budget)
{
    const uint32_t* queue = a.w.queue[qi];
    const uint32_t count = *(volatile uint32_t*)&a.w.counts[qi];
    unsigned lane = threadIdx.x & 31;
    TraceCounters tc{0u, 0u};
    uint32_t misses = 0;
    while (true) {
        uint32_t base = 0;
        if (lane == 0)
            base = atomicAdd(&a.w.counts[3], 32u);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= count)
            break;
        uint32_t i = base + lane;
        uint32_t p = 0;
        bool hit = false;
        bool ok = i < count;
        if (ok) {
            p = queue[i];
            PT_CHECK_ENTRY(ok, p, a)
        }
        if (TRAV == TRAV_BVH4 && BUDGET) {
            // one warp-uniform loop (a single copy of the step code): at
            // iteration `budget` the lanes still traversing park together
            ClosestTrace t;
            TraceStack stack;
            const uint32_t job = ok ? a.src.job_of(p) : 0u;
            bool live = ok;
            if (ok) {
                const float4 o = a.w.ray_o[p], d = a.w.ray_d[p];
                closest_begin(a.src.args(job).s, mk3(o.x, o.y, o.z), mk3(d.x, d.y, d.z), o.w, d.w, t, stack);
            }
            for (uint32_t k = 0;; k++) {
                if (k == budget) {
                    const bool park = live && t.sp <= PARK_STACK;
                    const unsigned want = __ballot_sync(0xffffffffu, park);
                    if (want) {
                        uint32_t slot0 = 0;
                        const int leader = __ffs(want) - 1;
                        if ((int)lane == leader)
                            slot0 = atomicAdd(&a.w.counts[6], (uint32_t)__popc(want));
                        slot0 = __shfl_sync(0xffffffffu, slot0, leader);
                        const uint32_t slot = slot0 + __popc(want & ((1u << lane) - 1u));
                        if (park && slot < a.w.park.cap) {
                            park_closest(a.w.park, slot, p, t, stack);
                            live = false;
                        }
                    }
                }
                if (!__any_sync(0xffffffffu, live))
                    break;
                if (live && closest_step<true>(a.src.args(job).s, t, stack, tc)) {
                    a.w.hit[p] = make_float4(t.h.t, t.h.b1, t.h.b2, __uint_as_float(t.h.inst));
                    a.w.hit_prim[p] = t.found ? t.h.prim : 0xFFFFFFFFu;
                    live = false;
                }
            }
            continue;
        }
        if (!BUDGET && ok) {
            const DevScene& s = a.src.args(a.src.job_of(p)).s;
            float4 o = a.w.ray_o[p], d = a.w.ray_d[p];
            Hit h;
            if (TRAV == TRAV_BVH2_WW)
                hit = trace_closest_ww(s, mk3(o.x, o.y, o.z), mk3(d.x, d.y, d.z), o.w, d.w, h, tc);
            else
                hit = trace_closest_inl<TRAV == TRAV_BVH4>(s, mk3(o.x, o.y, o.z), mk3(d.x, d.y, d.z), o.w, d.w, h, tc);
            a.w.hit[p] = make_float4(h.t, h.b1, h.b2, __uint_as_float(h.inst));
            a.w.hit_prim[p] = hit ? h.prim : 0xFFFFFFFFu;
        }
    }
    uint32_t nodes = __reduce_add_sync(0xffffffffu, tc.nodes);
    uint32_t tris = __reduce_add_sync(0xffffffffu, tc.tris);
    if (lane == 0) {
        atomicAdd(a.src.counters() + 3, (unsigned long long)nodes);
        atomicAdd(a.src.counters() + 4, (unsigned long long)tris);
    }
}

// Second extend pass: finishes the traversals the first pass parked, 32 to a
// warp (persistent warps over the parked slots).
template <class Src>
__global__ void __launch_bounds__(128, 8) k_wf_extend_resume(WaveArgs<Src> a)
{
    const uint32_t parked = *(volatile uint32_t*)&a.w.counts[6];
    const uint32_t count = parked < a.w.park.cap ? parked : a.w.park.cap;
    const unsigned lane = threadIdx.x & 31;
    TraceCounters tc{0u, 0u};
    while (true) {
        uint32_t base = 0;
        if (lane == 0)
            base = atomicAdd(&a.w.counts[7], 32u);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= count)
            break;
        const uint32_t slot = base + lane;
        bool ok = slot < count;
        uint32_t p = ok ? a.w.park.path[slot] : 0u;
        PT_CHECK_ENTRY(ok, p, a)
        if (ok) {
            const DevScene& s = a.src.args(a.src.job_of(p)).s;
            const float4 o = a.w.ray_o[p], d = a.w.ray_d[p];
            ClosestTrace t;
            TraceStack stack;
            resume_closest(s, a.w.park, slot, mk3(o.x, o.y, o.z), mk3(d.x, d.y, d.z), o.w, t, stack);
            while (!closest_step<true>(s, t, stack, tc)) {
            }
            a.w.hit[p] = make_float4(t.h.t, t.h.b1, t.h.b2, __uint_as_float(t.h.inst));
            a.w.hit_prim[p] = t.found ? t.h.prim : 0xFFFFFFFFu;
        }
    }
    const uint32_t nodes = __reduce_add_sync(0xffffffffu, tc.nodes);
    const uint32_t tris = __reduce_add_sync(0xffffffffu, tc.tris);
    if (lane == 0) {
        atomicAdd(a.src.counters() + 3, (unsigned long long)nodes);
        atomicAdd(a.src.counters() + 4, (unsigned long long)tris);
    }
}

// Splits the segment's queue: escaped rays are finished here
// (pathtrace.ms.hlsl:6-11: radiance += throughput * envcol, the path ends;
// a camera ray that escapes has zero first-hit features), hits go to the hit
// queue, so shade runs on hit paths only.  One atomic per block of 256 paths.
// The previous segment's shadow stage ran before this segment's extend, so
// the radiance terms keep the reference's order.
template <class Src>
__global__ void __launch_bounds__(256) k_wf_split(WaveArgs<Src> a, uint32_t qi)
{
    __shared__ uint32_t s_warp[8];
    __shared__ uint32_t s_base;
    const uint32_t* queue = a.w.queue[qi];
    const uint32_t count = a.w.counts[qi];
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t misses = 0;
    // the loop bound is the same for the whole block, so the barriers below are uniform
    for (uint32_t base = blockIdx.x * blockDim.x; base < count; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        bool valid = i < count;
        uint32_t p = valid ? queue[i] : 0u;
        PT_CHECK_ENTRY(valid, p, a)
        const bool hit = valid && a.w.hit_prim[p] != 0xFFFFFFFFu;
        if (valid && !hit) {
            const RenderArgs& R = a.src.args(a.src.job_of(p));
            PathState pl;
            const float4 t4 = a.w.tp[p], r4 = a.w.rad[p];
            pl.throughput = mk3(t4.x, t4.y, t4.z);
            pl.radiance = mk3(r4.x, r4.y, r4.z);
            shade_miss(R.s, pl);
            a.w.rad[p] = make_float4(pl.radiance.x, pl.radiance.y, pl.radiance.z, 0.0f);
            if (R.feat_a && a.w.seg[p] == 0) {
                a.w.f_a[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                a.w.f_n[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            }
            misses++;
        }
        const unsigned m = __ballot_sync(0xffffffffu, hit);
        if (lane == 0)
            s_warp[warp] = __popc(m);
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t total = 0;
            for (uint32_t w = 0; w < blockDim.x / 32; w++) {
                const uint32_t c = s_warp[w];
                s_warp[w] = total;
                total += c;
            }
            s_base = total ? atomicAdd(&a.w.counts[5], total) : 0u;
        }
        __syncthreads();
        if (hit)
            a.w.hit_queue[s_base + s_warp[warp] + __popc(m & ((1u << lane) - 1u))] = p;
        __syncthreads();
    }
    misses = __reduce_add_sync(0xffffffffu, misses);
    if (lane == 0 && misses)
        atomicAdd(a.src.counters() + 0, (unsigned long long)misses);
}

// shade_hit's NEE output in the wavefront: a request with a shadow ray goes
// straight to the path's NEE slots (the shadow stage finishes it), one
// without is finished at once, so the shader carries neither through its
// BSDF sampling.  The radiance sum keeps the reference's order: nothing in
// the shader adds to it after the light term.
template <class Src>
struct NeeToWave {
    const WaveArgs<Src>& a;
    uint32_t p;
    bool traced;
    __device__ __forceinline__ void operator()(PathState& pl, const NeeRequest& nee)
    {
        if (nee.add && nee.trace) {
            a.w.nee_o[p] = make_float4(nee.origin.x, nee.origin.y, nee.origin.z, nee.tmax);
            a.w.nee_d[p] = make_float4(nee.dir.x, nee.dir.y, nee.dir.z, nee.w);
            a.w.nee_e[p] = make_float4(nee.emission.x, nee.emission.y, nee.emission.z, nee.cos_i);
            a.w.nee_b[p] = make_float4(nee.brdf.x, nee.brdf.y, nee.brdf.z, nee.pdf);
            a.w.nee_tp[p] = make_float4(nee.tp_before.x, nee.tp_before.y, nee.tp_before.z, 0.0f);
            traced = true;
        } else if (nee.add) {
            finish_nee(pl.radiance, nee, 0.0f);
        }
    }
};

template <class Src, int MINB>
__global__ void __launch_bounds__(128, MINB) k_wf_shade(WaveArgs<Src> a, uint32_t qi)
{
    const uint32_t* qin = a.w.hit_queue;
    uint32_t* qout = a.w.queue[qi ^ 1];
    const uint32_t count = a.w.counts[5];
    uint32_t segments = 0, shadow_rays = 0;
    // grid-stride over whole warps so the warp-wide pushes see full warps
    // block-uniform loop: the queue pushes below synchronise the block
    for (uint32_t base = blockIdx.x * blockDim.x; base < count; base += gridDim.x * blockDim.x) {
        uint32_t i = base + threadIdx.x;
        bool active = i < count;
        bool cont = false, trace = false;
        uint32_t p = active ? qin[i] : 0;
        PT_CHECK_ENTRY(active, p, a)
        if (active) {
            segments++;
            uint32_t sg = a.w.seg[p];
            const PathLoc L = a.src.locate(p);
            const RenderArgs& R = a.src.args(L.job);
            const DevScene& s = R.s;
            uint32_t px = L.pix % R.width, py = L.pix / R.width;
            uint32_t si = L.si;
            PathState pl;
            float4 t4 = a.w.tp[p], r4 = a.w.rad[p];
            pl.throughput = mk3(t4.x, t4.y, t4.z);
            pl.brdf_pdf = t4.w;
            pl.radiance = mk3(r4.x, r4.y, r4.z);
            pl.final_segment = sg >= R.max_bounces;
            sampler_start(pl.smp, px, py, si, sg + 1);
            float4 o = a.w.ray_o[p], d = a.w.ray_d[p];
            f3 ro = mk3(o.x, o.y, o.z), rd = mk3(d.x, d.y, d.z);
            uint32_t prim = a.w.hit_prim[p];
            NeeToWave<Src> nee_out{a, p, false};
            {
                // the hit queue holds hits only (extend finished the misses)
                float4 hh = a.w.hit[p];
                Hit h;
                h.t = hh.x;
                h.b1 = hh.y;
                h.b2 = hh.z;
                h.inst = __float_as_uint(hh.w);
                h.prim = prim;
                if (sg == 0 && R.feat_a) {
                    f3 alb, nrm;
                    hit_features(s, h, rd, alb, nrm);
                    a.w.f_a[p] = make_float4(alb.x, alb.y, alb.z, h.t);
                    a.w.f_n[p] = make_float4(nrm.x, nrm.y, nrm.z, 0.0f);
                }
                shade_hit(s, pl, ro, rd, h, nee_out);
            }
            trace = nee_out.traced;
            if (trace)
                shadow_rays++;
            // continuation (rg.hlsl:38-55): RR from segment rr_start >= 1
            if (!pl.final_segment) {
                bool killed = false;
                if (sg >= 1 && sg >= R.rr_start)
                    killed = russian_roulette(pl);
                cont = !killed && sg + 1 <= R.max_bounces;
            }
            a.w.tp[p] = make_float4(pl.throughput.x, pl.throughput.y, pl.throughput.z, pl.brdf_pdf);
            a.w.rad[p] = make_float4(pl.radiance.x, pl.radiance.y, pl.radiance.z, 0.0f);
            if (cont) {
                a.w.seg[p] = sg + 1;
                a.w.ray_o[p] = make_float4(pl.next_o.x, pl.next_o.y, pl.next_o.z, 0.0f);
                a.w.ray_d[p] = make_float4(pl.next_d.x, pl.next_d.y, pl.next_d.z, __int_as_float(0x7f800000));
            }
        }
        push_block2<4>(qout, &a.w.counts[qi ^ 1], cont, a.w.shadow_queue, &a.w.counts[2], trace, p);
    }
    segments = __reduce_add_sync(0xffffffffu, segments);
    shadow_rays = __reduce_add_sync(0xffffffffu, shadow_rays);
    if ((threadIdx.x & 31) == 0 && (segments | shadow_rays)) {
        atomicAdd(a.src.counters() + 0, (unsigned long long)segments);
        atomicAdd(a.src.counters() + 1, (unsigned long long)shadow_rays);
    }
}

// Persistent traversal with per-lane refill (the dynamic ray fetch of Aila &
// Laine 2009): each lane keeps one ray's traversal state and advances it one
// step per loop iteration; once at least `refill` lanes of the warp are idle
// they take the next queue entries with one warp-aggregated atomic, so lanes
// whose ray finished early do not wait for the warp's longest ray.  Every ray
// is traversed exactly as by trace_closest_inl (same steps, same result).
template <class Src, bool W4>
__global__ void __launch_bounds__(128) k_wf_extend_refill(WaveArgs<Src> a, uint32_t qi, uint32_t refill)
{
    const uint32_t* queue = a.w.queue[qi];
    const uint32_t count = *(volatile uint32_t*)&a.w.counts[qi];
    const unsigned lane = threadIdx.x & 31;
    const unsigned lower = (1u << lane) - 1u;
    TraceCounters tc{0u, 0u};
    ClosestTrace t;
    TraceStack stack;
    const DevScene* sc = nullptr;
    uint32_t p = 0;
    bool active = false, exhausted = false;
    while (true) {
        const unsigned idle = __ballot_sync(0xffffffffu, !active);
        if (!exhausted && (uint32_t)__popc(idle) >= refill) {
            const int leader = __ffs(idle) - 1;
            uint32_t base = 0;
            if ((int)lane == leader)
                base = atomicAdd(&a.w.counts[3], (uint32_t)__popc(idle));
            base = __shfl_sync(0xffffffffu, base, leader);
            exhausted = base + (uint32_t)__popc(idle) >= count;
            if (!active) {
                const uint32_t i = base + (uint32_t)__popc(idle & lower);
                if (i < count) {
                    p = queue[i];
                    sc = &a.src.args(a.src.job_of(p)).s;
                    const float4 o = a.w.ray_o[p], d = a.w.ray_d[p];
                    closest_begin(*sc, mk3(o.x, o.y, o.z), mk3(d.x, d.y, d.z), o.w, d.w, t, stack);
                    active = true;
                }
            }
        }
        if (__ballot_sync(0xffffffffu, active) == 0) {
            if (exhausted)
                break;
            continue;
        }
        if (active && closest_step<W4>(*sc, t, stack, tc)) {
            a.w.hit[p] = make_float4(t.h.t, t.h.b1, t.h.b2, __uint_as_float(t.h.inst));
            a.w.hit_prim[p] = t.found ? t.h.prim : 0xFFFFFFFFu;
            active = false;
        }
    }
    const uint32_t nodes = __reduce_add_sync(0xffffffffu, tc.nodes);
    const uint32_t tris = __reduce_add_sync(0xffffffffu, tc.tris);
    if (lane == 0) {
        atomicAdd(a.src.counters() + 3, (unsigned long long)nodes);
        atomicAdd(a.src.counters() + 4, (unsigned long long)tris);
    }
}

// Adds the light term of shadow-queue entry p with visibility vis.
template <class Src>
__device__ __forceinline__ void finish_shadow_entry(WaveArgs<Src>& a, uint32_t p, float vis)
{
    NeeRequest nee;
    nee.add = true;
    nee.trace = true;
    const float4 e = a.w.nee_e[p], b = a.w.nee_b[p], t = a.w.nee_tp[p];
    nee.emission = mk3(e.x, e.y, e.z);
    nee.cos_i = e.w;
    nee.brdf = mk3(b.x, b.y, b.z);
    nee.pdf = b.w;
    nee.w = a.w.nee_d[p].w;
    nee.tp_before = mk3(t.x, t.y, t.z);
    const float4 r4 = a.w.rad[p];
    f3 rad = mk3(r4.x, r4.y, r4.z);
    finish_nee(rad, nee, vis);
    a.w.rad[p] = make_float4(rad.x, rad.y, rad.z, 0.0f);
}

// Shadow rays with per-lane refill, as k_wf_extend_refill.
template <class Src, bool W4>
__global__ void __launch_bounds__(128) k_wf_shadow_refill(WaveArgs<Src> a, uint32_t refill)
{
    const uint32_t count = a.w.counts[2];
    const unsigned lane = threadIdx.x & 31;
    const unsigned lower = (1u << lane) - 1u;
    TraceCounters tc{0u, 0u};
    ShadowTrace t;
    TraceStack stack;
    const DevScene* sc = nullptr;
    uint32_t p = 0;
    bool active = false, exhausted = false;
    while (true) {
        const unsigned idle = __ballot_sync(0xffffffffu, !active);
        if (!exhausted && (uint32_t)__popc(idle) >= refill) {
            const int leader = __ffs(idle) - 1;
            uint32_t base = 0;
            if ((int)lane == leader)
                base = atomicAdd(&a.w.counts[4], (uint32_t)__popc(idle));
            base = __shfl_sync(0xffffffffu, base, leader);
            exhausted = base + (uint32_t)__popc(idle) >= count;
            if (!active) {
                const uint32_t i = base + (uint32_t)__popc(idle & lower);
                if (i < count) {
                    p = a.w.shadow_queue[i];
                    sc = &a.src.args(a.src.job_of(p)).s;
                    const float4 o = a.w.nee_o[p], d = a.w.nee_d[p];
                    shadow_begin(*sc, mk3(o.x, o.y, o.z), mk3(d.x, d.y, d.z), 0.0f, o.w, t, stack);
                    active = true;
                }
            }
        }
        if (__ballot_sync(0xffffffffu, active) == 0) {
            if (exhausted)
                break;
            continue;
        }
        if (active && shadow_step<W4>(*sc, t, stack, tc)) {
            finish_shadow_entry(a, p, shadow_result(t));
            active = false;
        }
    }
    const uint32_t nodes = __reduce_add_sync(0xffffffffu, tc.nodes);
    const uint32_t tris = __reduce_add_sync(0xffffffffu, tc.tris);
    if (lane == 0) {
        atomicAdd(a.src.counters() + 3, (unsigned long long)nodes);
        atomicAdd(a.src.counters() + 4, (unsigned long long)tris);
    }
}

// Completes the NEE term of path p with the shadow ray's visibility.
template <class Src>
__device__ __forceinline__ void shadow_finish(const WaveArgs<Src>& a, uint32_t p, float vis)
{
    NeeRequest nee;
    nee.add = true;
    nee.trace = true;
    const float4 e = a.w.nee_e[p], b = a.w.nee_b[p], t = a.w.nee_tp[p];
    nee.emission = mk3(e.x, e.y, e.z);
    nee.cos_i = e.w;
    nee.brdf = mk3(b.x, b.y, b.z);
    nee.pdf = b.w;
    nee.w = a.w.nee_d[p].w;
    nee.tp_before = mk3(t.x, t.y, t.z);
    const float4 r4 = a.w.rad[p];
    f3 rad = mk3(r4.x, r4.y, r4.z);
    finish_nee(rad, nee, vis);
    a.w.rad[p] = make_float4(rad.x, rad.y, rad.z, 0.0f);
}

// Persistent shadow (any-hit) traversal.  With BUDGET (4-wide nodes) the
// first of two passes, as k_wf_extend: rays still traversing after `budget`
// steps park (counters [8]/[9]) and k_wf_shadow_resume finishes them.
template <class Src, bool W4, bool BUDGET = false>
__global__ void __launch_bounds__(128, W4 ? 7 : 1) k_wf_shadow(WaveArgs<Src> a, uint32_t budget)
{
    const uint32_t count = a.w.counts[2];
    unsigned lane = threadIdx.x & 31;
    TraceCounters tc{0u, 0u};
    while (true) {
        uint32_t base = 0;
        if (lane == 0)
            base = atomicAdd(&a.w.counts[4], 32u);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= count)
            break;
        uint32_t i = base + lane;
        bool ok = i < count;
        uint32_t p = ok ? a.w.shadow_queue[i] : 0u;
        PT_CHECK_ENTRY(ok, p, a)
        if (W4 && BUDGET) {
            ShadowTrace t;
            TraceStack stack;
            const uint32_t job = ok ? a.src.job_of(p) : 0u;
            bool live = ok;
            if (ok) {
                const float4 o = a.w.nee_o[p], d = a.w.nee_d[p];
                shadow_begin(a.src.args(job).s, mk3(o.x, o.y, o.z), mk3(d.x, d.y, d.z), 0.0f, o.w, t, stack);
            }
            for (uint32_t k = 0;; k++) {
                if (k == budget) {
                    const bool park = live && t.sp <= PARK_STACK;
                    const unsigned want = __ballot_sync(0xffffffffu, park);
                    if (want) {
                        uint32_t slot0 = 0;
                        const int leader = __ffs(want) - 1;
                        if ((int)lane == leader)
                            slot0 = atomicAdd(&a.w.counts[8], (uint32_t)__popc(want));
                        slot0 = __shfl_sync(0xffffffffu, slot0, leader);
                        const uint32_t slot = slot0 + __popc(want & ((1u << lane) - 1u));
                        if (park && slot < a.w.park.cap) {
                            park_shadow(a.w.park, slot, p, t, stack);
                            live = false;
                        }
                    }
                }
                if (!__any_sync(0xffffffffu, live))
                    break;
                if (live && shadow_step<true>(a.src.args(job).s, t, stack, tc)) {
                    shadow_finish(a, p, shadow_result(t));
                    live = false;
                }
            }
            continue;
        }
        if (ok) {
            const DevScene& s = a.src.args(a.src.job_of(p)).s;
            float4 o = a.w.nee_o[p], d = a.w.nee_d[p];
            float vis = trace_shadow_inl<W4>(s, mk3(o.x, o.y, o.z), mk3(d.x, d.y, d.z), 0.0f, o.w, tc);
            shadow_finish(a, p, vis);
        }
    }
    uint32_t nodes = __reduce_add_sync(0xffffffffu, tc.nodes);
    uint32_t tris = __reduce_add_sync(0xffffffffu, tc.tris);
    if (lane == 0) {
        atomicAdd(a.src.counters() + 3, (unsigned long long)nodes);
        atomicAdd(a.src.counters() + 4, (unsigned long long)tris);
    }
}

// Second shadow pass: finishes the shadow traversals the first pass parked.
template <class Src>
__global__ void __launch_bounds__(128, 7) k_wf_shadow_resume(WaveArgs<Src> a)
{
    const uint32_t parked = *(volatile uint32_t*)&a.w.counts[8];
    const uint32_t count = parked < a.w.park.cap ? parked : a.w.park.cap;
    const unsigned lane = threadIdx.x & 31;
    TraceCounters tc{0u, 0u};
    while (true) {
        uint32_t base = 0;
        if (lane == 0)
            base = atomicAdd(&a.w.counts[9], 32u);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= count)
            break;
        const uint32_t slot = base + lane;
        bool ok = slot < count;
        uint32_t p = ok ? a.w.park.path[slot] : 0u;
        PT_CHECK_ENTRY(ok, p, a)
        if (ok) {
            const DevScene& s = a.src.args(a.src.job_of(p)).s;
            const float4 o = a.w.nee_o[p], d = a.w.nee_d[p];
            ShadowTrace t;
            TraceStack stack;
            resume_shadow(s, a.w.park, slot, mk3(o.x, o.y, o.z), mk3(d.x, d.y, d.z), 0.0f, o.w, t, stack);
            while (!shadow_step<true>(s, t, stack, tc)) {
            }
            shadow_finish(a, p, shadow_result(t));
        }
    }
    const uint32_t nodes = __reduce_add_sync(0xffffffffu, tc.nodes);
    const uint32_t tris = __reduce_add_sync(0xffffffffu, tc.tris);
    if (lane == 0) {
        atomicAdd(a.src.counters() + 3, (unsigned long long)nodes);
        atomicAdd(a.src.counters() + 4, (unsigned long long)tris);
    }
}

// Clears the consumed queue count and the fetch counters between stages.
__global__ void k_wf_reset(uint32_t* counts, uint32_t qi)
{
    counts[qi] = 0; // the queue just consumed by extend
    counts[2] = 0;  // shadow queue consumed
    counts[3] = 0;
    counts[4] = 0;
    counts[5] = 0;  // hit queue consumed by shade
    counts[6] = 0;  // parked traversals finished
    counts[7] = 0;
    counts[8] = 0;
    counts[9] = 0;
}

template <class Src>
__global__ void __launch_bounds__(256) k_wf_accumulate(WaveArgs<Src> a)
{
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < a.src.accum_threads(); t += gridDim.x * blockDim.x) {
        uint32_t pix;
        const WaveShare E = a.src.share_of_pixel(t, pix);
        const RenderArgs& R = a.src.args(E.job);
        float4 acc = R.image[pix];
        double s64[3] = {0.0, 0.0, 0.0};
        if (R.sum64) {
            s64[0] = R.sum64[4 * (size_t)pix + 0];
            s64[1] = R.sum64[4 * (size_t)pix + 1];
            s64[2] = R.sum64[4 * (size_t)pix + 2];
        }
        float4 fa = make_float4(0.0f, 0.0f, 0.0f, 0.0f), fn = fa;
        if (R.feat_a) {
            fa = feat_load(R.feat_a, pix, R.fp16_features);
            fn = feat_load(R.feat_n, pix, R.fp16_features);
            for (uint32_t j = 0; j < E.samples; j++) {
                const size_t q = E.path_base + (size_t)j * E.pixels + pix;
                feature_mean(fa, a.w.f_a[q], E.first_sample + j);
                feature_mean(fn, a.w.f_n[q], E.first_sample + j);
            }
            feat_store(R.feat_a, pix, fa, R.fp16_features);
            feat_store(R.feat_n, pix, fn, R.fp16_features);
        }
        // FP64 sums only when the render keeps them: FP64 adds are slow on this GPU
        const bool want64 = R.sum64 != nullptr;
        for (uint32_t j = 0; j < E.samples; j++) {
            float4 r4 = a.w.rad[E.path_base + (size_t)j * E.pixels + pix];
            f3 r = correct_radiance(mk3(r4.x, r4.y, r4.z) * R.exposure);
            accumulate(acc, r, E.first_sample + j);
            if (R.snapshot && E.first_sample + j + 1 == R.snapshot_after)
                feat_store(R.snapshot, pix, acc, R.fp16_features);
            if (want64) {
                s64[0] += (double)r.x;
                s64[1] += (double)r.y;
                s64[2] += (double)r.z;
            }
        }
        R.image[pix] = acc;
        if (R.sum64) {
            double* d = R.sum64 + 4 * (size_t)pix;
            d[0] = s64[0];
            d[1] = s64[1];
            d[2] = s64[2];
            d[3] += (double)E.samples;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0)
        atomicAdd(a.src.counters() + 2, (unsigned long long)a.src.n_paths);
}

// Parking slots for a quarter of a wave's paths (a multiple of 32).
static inline size_t park_slots(size_t n_paths) { return ((n_paths / 4) + 31) / 32 * 32; }

size_t wave_state_bytes(uint32_t n_paths)
{
    const size_t park = park_slots(n_paths) * (4 + 16 + 16 + 4 + 4 * (size_t)PARK_STACK);
    return (size_t)n_paths * (16 * 13 + 4 * 6) + park + 8192;
}

static inline char* bump(char*& p, size_t bytes)
{
    uintptr_t a = ((uintptr_t)p + 255) & ~(uintptr_t)255;
    p = (char*)(a + bytes);
    return (char*)a;
}

// Carves the SoA path state for n paths out of `state`.
static bool carve_state(WaveState& w, void* state, size_t state_bytes, size_t n)
{
    if (state_bytes < wave_state_bytes((uint32_t)n))
        return false;
    char* p = (char*)state;
    w.ray_o = (float4*)bump(p, 16 * n);
    w.ray_d = (float4*)bump(p, 16 * n);
    w.tp = (float4*)bump(p, 16 * n);
    w.rad = (float4*)bump(p, 16 * n);
    w.seg = (uint32_t*)bump(p, 4 * n);
    w.hit = (float4*)bump(p, 16 * n);
    w.hit_prim = (uint32_t*)bump(p, 4 * n);
    w.nee_o = (float4*)bump(p, 16 * n);
    w.nee_d = (float4*)bump(p, 16 * n);
    w.nee_e = (float4*)bump(p, 16 * n);
    w.nee_b = (float4*)bump(p, 16 * n);
    w.nee_tp = (float4*)bump(p, 16 * n);
    w.f_a = (float4*)bump(p, 16 * n);
    w.f_n = (float4*)bump(p, 16 * n);
    w.queue[0] = (uint32_t*)bump(p, 4 * n);
    w.queue[1] = (uint32_t*)bump(p, 4 * n);
    w.shadow_queue = (uint32_t*)bump(p, 4 * n);
    w.hit_queue = (uint32_t*)bump(p, 4 * n);
    w.counts = (uint32_t*)bump(p, 64);
    const size_t slots = park_slots(n);
    w.park.cap = (uint32_t)slots;
    w.park.path = (uint32_t*)bump(p, 4 * slots);
    w.park.state = (int4*)bump(p, 16 * slots);
    w.park.hit = (float4*)bump(p, 16 * slots);
    w.park.prim = (uint32_t*)bump(p, 4 * slots);
    w.park.stack = (int*)bump(p, 4 * (size_t)PARK_STACK * slots);
    return (size_t)(p - (char*)state) <= state_bytes;
}

static inline uint32_t capped_grid(uint64_t threads, uint32_t block, int sm_count)
{
    uint64_t g = (threads + block - 1) / block;
    uint64_t cap = (uint64_t)sm_count * 16;
    return (uint32_t)(g < cap ? (g == 0 ? 1 : g) : cap);
}

// Launch variants of the stage kernels, fixed per process: the BVH2
// closest-hit traversal when the scene has no 4-wide nodes (one
// node-or-leaf step per iteration, or while-while with speculative leaves
// with PT_TRAVERSAL=ww: on the mid scene the latter ran 24 % slower, its
// extra node visits and triangle tests costing more than the coherence
// gained), the per-lane refill of the traversal kernels (PT_REFILL = idle
// lanes that trigger a fetch, 1-32; 0 = whole-warp fetches of 32 rays) and
// the resident-block target of shade (PT_MINB=5 or 6, 0 for none; default 6:
// 0.45 % faster than the 4 blocks its natural register count gives, 5
// blocks slower).  The alternatives stay for A/B measurements.
struct StageVariant {
    bool ww = false;
    int shade = 6;       // resident-block target of shade (0: none)
    uint32_t refill = 0; // 0: no refill; else 1..32
    uint32_t budget = 48; // extend's first-pass step budget over 4-wide nodes (PT_EXTEND_BUDGET; 0: one pass)
    // two passes only for waves of at least 2^budget_min_log2 paths
    // (PT_EXTEND_BUDGET_MIN_LOG2): smaller waves ran 2-11 % faster in one
    // pass (the resume launch's latency tail), waves of 2^25 paths and more
    // 0.3-0.5 % slower
    uint32_t budget_min_log2 = 25;
    uint32_t shadow_budget = 0; // the same for shadow rays (PT_SHADOW_BUDGET; measured slower, off)
};

static StageVariant stage_variant()
{
    static const StageVariant v = [] {
        StageVariant r;
        const char* t = std::getenv("PT_TRAVERSAL");
        r.ww = t && std::strcmp(t, "ww") == 0;
        if (const char* m = std::getenv("PT_MINB")) {
            const int h = std::atoi(m);
            r.shade = (h == 5 || h == 6) ? h : 0;
        }
        if (const char* f = std::getenv("PT_REFILL")) {
            const int k = std::atoi(f);
            r.refill = k <= 0 ? 0u : (uint32_t)std::min(k, 32);
        }
        if (const char* b = std::getenv("PT_EXTEND_BUDGET")) {
            const int k = std::atoi(b);
            r.budget = k <= 0 ? 0u : (uint32_t)std::min(k, 1 << 20);
        }
        if (const char* b = std::getenv("PT_EXTEND_BUDGET_MIN_LOG2")) {
            const int k = std::atoi(b);
            r.budget_min_log2 = (uint32_t)std::max(0, std::min(k, 32));
        }
        if (const char* b = std::getenv("PT_SHADOW_BUDGET")) {
            const int k = std::atoi(b);
            r.shadow_budget = k <= 0 ? 0u : (uint32_t)std::min(k, 1 << 20);
        }
        return r;
    }();
    return v;
}

template <typename K>
static int resident_blocks(K kernel)
{
    int b = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kernel, 128, 0);
    return b < 1 ? 1 : b;
}

// The extend variant for scenes with (w4) or without 4-wide nodes.
static int traversal_of(bool w4)
{
#ifdef PT_CHECKED
    return w4 ? TRAV_BVH4 : TRAV_BVH2; // the while-while traversal has no checked form
#else
    return w4 ? TRAV_BVH4 : stage_variant().ww ? TRAV_BVH2_WW : TRAV_BVH2;
#endif
}

// Whether the process's extend and shadow launches are the refill kernels
// (the while-while BVH2 traversal has no refill form).
static bool refill_for(bool w4)
{
#ifdef PT_CHECKED
    (void)w4;
    return false; // the refill kernels have no checked form
#else
    return stage_variant().refill != 0 && traversal_of(w4) != TRAV_BVH2_WW;
#endif
}

// Resident 128-thread blocks per SM of the persistent traversal kernels
// (extend, shadow) the process launches for both node widths (queried once;
// thread-safe initialisation).
template <class Src>
static int2 traversal_blocks_per_sm(bool w4)
{
    static const int4 v = [] {
        int4 r;
        if (refill_for(true)) {
            r.x = resident_blocks(k_wf_extend_refill<Src, true>);
            r.y = resident_blocks(k_wf_shadow_refill<Src, true>);
        } else {
            r.x = resident_blocks(k_wf_extend<Src, TRAV_BVH4>);
            r.y = resident_blocks(k_wf_shadow<Src, true>);
        }
        if (refill_for(false)) {
            r.z = resident_blocks(k_wf_extend_refill<Src, false>);
            r.w = resident_blocks(k_wf_shadow_refill<Src, false>);
        } else {
            r.z = traversal_of(false) == TRAV_BVH2_WW ? resident_blocks(k_wf_extend<Src, TRAV_BVH2_WW>)
                                                      : resident_blocks(k_wf_extend<Src, TRAV_BVH2>);
            r.w = resident_blocks(k_wf_shadow<Src, false>);
        }
        return r;
    }();
    return w4 ? make_int2(v.x, v.y) : make_int2(v.z, v.w);
}

cudaError_t wave_batch_prepare()
{
    traversal_blocks_per_sm<ManyJobs>(true);
    return cudaGetLastError();
}

// One wave: raygen, (extend, shade, shadow, reset) per segment, accumulate.
// acc_wait / acc_done (optional) order the accumulation after an earlier
// wave's on another stream and mark its completion.
template <class Src>
static uint32_t launch_wave(const WaveArgs<Src>& a, bool w4, uint32_t max_bounces, uint32_t accum_threads, int sm_count,
                            cudaStream_t st, StageTimer* tm = nullptr, cudaEvent_t acc_wait = nullptr,
                            cudaEvent_t acc_done = nullptr)
{
    auto mark = [&](uint8_t s) {
        if (tm)
            tm->mark(st, s);
    };
    // persistent traversal grids: exactly the resident blocks of every SM
    const StageVariant sv = stage_variant();
    const int trav = traversal_of(w4);
    const bool refill = refill_for(w4);
    const int2 per_sm = traversal_blocks_per_sm<Src>(w4);
    const int trace_blocks = sm_count * per_sm.x;
    const int shadow_blocks = sm_count * per_sm.y;
    uint32_t nl = 0;
    mark(0);
    k_wf_raygen<Src><<<capped_grid(a.src.n_paths, 256, sm_count), 256, 0, st>>>(a);
    nl++;
    uint32_t qi = 0;
    const uint32_t sgrid = capped_grid(a.src.n_paths, 128, sm_count);
    for (uint32_t sg = 0; sg <= max_bounces; sg++) {
        mark(1);
        if (refill && w4)
            k_wf_extend_refill<Src, true><<<trace_blocks, 128, 0, st>>>(a, qi, sv.refill);
        else if (refill)
            k_wf_extend_refill<Src, false><<<trace_blocks, 128, 0, st>>>(a, qi, sv.refill);
        else if (trav == TRAV_BVH4) {
            if (sv.budget && (uint64_t)a.src.n_paths >= (1ull << sv.budget_min_log2)) {
                k_wf_extend<Src, TRAV_BVH4, true><<<trace_blocks, 128, 0, st>>>(a, qi, sv.budget);
                k_wf_extend_resume<Src><<<trace_blocks, 128, 0, st>>>(a);
                nl++;
            } else {
                k_wf_extend<Src, TRAV_BVH4><<<trace_blocks, 128, 0, st>>>(a, qi, 0u);
            }
        } else if (trav == TRAV_BVH2_WW)
            k_wf_extend<Src, TRAV_BVH2_WW><<<trace_blocks, 128, 0, st>>>(a, qi, 0u);
        else
            k_wf_extend<Src, TRAV_BVH2><<<trace_blocks, 128, 0, st>>>(a, qi, 0u);
        mark(2);
        k_wf_split<Src><<<capped_grid(a.src.n_paths, 256, sm_count), 256, 0, st>>>(a, qi);
        if (sv.shade == 5)
            k_wf_shade<Src, 5><<<sgrid, 128, 0, st>>>(a, qi);
        else if (sv.shade == 6)
            k_wf_shade<Src, 6><<<sgrid, 128, 0, st>>>(a, qi);
        else
            k_wf_shade<Src, 0><<<sgrid, 128, 0, st>>>(a, qi);
        mark(3);
        if (refill && w4)
            k_wf_shadow_refill<Src, true><<<shadow_blocks, 128, 0, st>>>(a, sv.refill);
        else if (refill)
            k_wf_shadow_refill<Src, false><<<shadow_blocks, 128, 0, st>>>(a, sv.refill);
        else if (w4 && sv.shadow_budget) {
            k_wf_shadow<Src, true, true><<<shadow_blocks, 128, 0, st>>>(a, sv.shadow_budget);
            k_wf_shadow_resume<Src><<<shadow_blocks, 128, 0, st>>>(a);
            nl++;
        } else if (w4)
            k_wf_shadow<Src, true><<<shadow_blocks, 128, 0, st>>>(a, 0u);
        else
            k_wf_shadow<Src, false><<<shadow_blocks, 128, 0, st>>>(a, 0u);
        mark(4);
        k_wf_reset<<<1, 1, 0, st>>>(a.w.counts, qi);
        nl += 5;
        qi ^= 1;
    }
    mark(5);
    if (acc_wait)
        cudaStreamWaitEvent(st, acc_wait, 0);
    k_wf_accumulate<Src><<<capped_grid(accum_threads, 256, sm_count), 256, 0, st>>>(a);
    if (acc_done)
        cudaEventRecord(acc_done, st);
    nl++;
    mark(6);
    return nl;
}

cudaError_t launch_wavefront(const RenderArgs& r, void* state, size_t state_bytes, uint32_t n_paths_max, int sm_count,
                             uint32_t* launches, cudaStream_t st, StageTimer* timer, const WaveMulti* multi)
{
    WaveArgs<OneJob> a[MAX_WAVE_WAYS];
    a[0].src.r = r;
    if (!carve_state(a[0].w, state, state_bytes, n_paths_max))
        return cudaErrorInvalidValue;
    a[0].src.pixels = r.width * r.height;
    const uint32_t k_max = n_paths_max / a[0].src.pixels;
    if (k_max == 0)
        return cudaErrorInvalidValue;
    // ways in use: no more than the waves the render needs
    const uint32_t waves = (r.samples + k_max - 1) / k_max;
    int ways = 1;
    if (multi != nullptr && timer == nullptr && multi->ways > 1 && multi->ways <= MAX_WAVE_WAYS)
        ways = (int)(waves < (uint32_t)multi->ways ? waves : (uint32_t)multi->ways);
    for (int k = 1; k < ways; k++) {
        a[k] = a[0];
        if (!carve_state(a[k].w, multi->state[k], multi->state_bytes[k], n_paths_max))
            return cudaErrorInvalidValue;
    }
    if (ways > 1) {
        cudaEventRecord(multi->fork, st);
        for (int k = 1; k < ways; k++)
            cudaStreamWaitEvent(multi->stream[k], multi->fork, 0);
    }
    const bool w4 = r.s.nodes4 != nullptr;
    uint32_t nl = 0, w = 0;
    for (uint32_t done = 0; done < r.samples; w++) {
        const int k = (int)(w % (uint32_t)ways);
        WaveArgs<OneJob>& x = a[k];
        x.src.samples = r.samples - done < k_max ? r.samples - done : k_max;
        x.src.first_sample = r.sample_index + done;
        x.src.n_paths = x.src.samples * x.src.pixels;
        if (ways > 1)
            nl += launch_wave(x, w4, r.max_bounces, x.src.pixels, sm_count, k ? multi->stream[k] : st, nullptr,
                              w ? multi->acc[(w - 1) % (uint32_t)ways] : nullptr, multi->acc[k]);
        else
            nl += launch_wave(x, w4, r.max_bounces, x.src.pixels, sm_count, st, timer);
        done += x.src.samples;
    }
    if (ways > 1) {
        for (int k = 1; k < ways; k++) {
            cudaEventRecord(multi->join[k], multi->stream[k]);
            cudaStreamWaitEvent(st, multi->join[k], 0);
        }
    }
    if (launches)
        *launches = nl;
    return cudaGetLastError();
}

cudaError_t launch_wavefront_batch(const RenderArgs* jobs, const WaveShare* shares, const BatchWave* waves, uint32_t wave_count,
                                   uint32_t* path_share, unsigned long long* counters, void* state, size_t state_bytes,
                                   uint32_t n_paths_max, bool w4, int sm_count, uint32_t* launches, cudaStream_t st,
                                   const WaveMulti* multi, uint32_t* path_share2, cudaEvent_t* wave_done)
{
    WaveArgs<ManyJobs> a[2];
    if (!carve_state(a[0].w, state, state_bytes, n_paths_max))
        return cudaErrorInvalidValue;
    a[0].src.jobs = jobs;
    a[0].src.path_share = path_share;
    a[0].src.ctr = counters;
    const int ways = (multi != nullptr && multi->ways >= 2 && path_share2 != nullptr && wave_count >= 2) ? 2 : 1;
    if (ways == 2) {
        a[1] = a[0];
        a[1].src.path_share = path_share2;
        if (!carve_state(a[1].w, multi->state[1], multi->state_bytes[1], n_paths_max))
            return cudaErrorInvalidValue;
        cudaEventRecord(multi->fork, st);
        cudaStreamWaitEvent(multi->stream[1], multi->fork, 0);
    }
    uint32_t nl = 0;
    for (uint32_t i = 0; i < wave_count; i++) {
        const BatchWave& bw = waves[i];
        if (bw.n_paths > n_paths_max || bw.share_count == 0)
            return cudaErrorInvalidValue;
        WaveArgs<ManyJobs>& x = a[ways == 2 ? (i & 1) : 0];
        x.src.shares = shares + bw.share_offset;
        x.src.share_count = bw.share_count;
        x.src.n_paths = bw.n_paths;
        x.src.n_pixels = bw.n_pixels;
        const cudaStream_t ws = (ways == 2 && (i & 1)) ? multi->stream[1] : st;
        if (ways == 2)
            nl += launch_wave(x, w4, bw.max_bounces, bw.n_pixels, sm_count, ws, nullptr,
                              i ? multi->acc[(i - 1) & 1] : nullptr, multi->acc[i & 1]);
        else
            nl += launch_wave(x, w4, bw.max_bounces, bw.n_pixels, sm_count, ws);
        if (wave_done) // after the wave's accumulation, the last of its launches
            record_timed(wave_done[i], ws);
    }
    if (ways == 2) {
        cudaEventRecord(multi->join[1], multi->stream[1]);
        cudaStreamWaitEvent(st, multi->join[1], 0);
    }
    if (launches)
        *launches = nl;
    return cudaGetLastError();
}

cudaError_t wave_init_tables(const uint32_t* table128, const float* srgb256, cudaStream_t stream)
{
    uint32_t bytes[4][4][256];
    sobol_byte_tables(table128, bytes);
    cudaError_t e = cudaMemcpyToSymbol(g_sobol_bytes, bytes, sizeof(bytes)); // synchronous: `bytes` is local
    if (e == cudaSuccess)
        e = cudaMemcpyToSymbolAsync(c_srgb, srgb256, sizeof(float) * 256, 0, cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess)
        return e;
    return cudaStreamSynchronize(stream);
}

} // namespace pt
