// batch.cu — pt_render_batch: many render jobs in one launch sequence.
//
// Jobs (scene, camera, size, samples, bounces) are packed into waves of the
// batched wavefront (render_wave.cu): a wave holds consecutive samples of
// several jobs, up to the wave capacity in paths, so small jobs fill the GPU
// together and the tail segments of one job overlap another's.  Each job's
// samples go through the waves in increasing order, so its running mean is
// updated in sample order and its image equals rendering the job alone.
// Jobs below a work threshold may run as megakernel launches on a side
// stream instead; both branches are captured into one CUDA graph, which is
// cached and launched again when the same batch comes back.
//
// The autotuner times trial batches (each job at 1/32 of its samples, at
// least 1) for a few candidate settings and keeps the fastest, per batch:
//   1. wave capacity 2^26, 2^25, 2^23, 2^21 paths (all jobs on the wavefront;
//      a smaller capacity must be more than 3 % faster to be kept);
//   2. megakernel threshold 0, 2^18, 2^21 on a job's trial work, pixels x
//      trial samples x (bounces + 1) (tile 16x8);
//   3. if a threshold won: megakernel tile 8x16 or 32x4 against 16x8.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/pt_gpu.h"
#include "ctx.h"
#include "kernels.h"

namespace pt {

struct BatchChoice {
    uint32_t capacity = 1u << 23;
    uint32_t tile_w = 16;
    uint64_t mega_threshold = 0;
};

struct BatchState {
    // images of the last batch, back to back
    DevBuf<float4> image;
    DevBuf<double> sum64;
    std::vector<size_t> img_off, sum_off; // per job (sum_off = SIZE_MAX: no FP64 sums)
    std::vector<uint32_t> width, height;
    // launch data
    DevBuf<RenderArgs> jobs;
    DevBuf<WaveShare> shares;
    DevBuf<uint32_t> path_share;
    DevBuf<char> state;
    uint32_t state_paths = 0;
    // the second wave state in flight (plans of two or more waves), on wave_side
    DevBuf<char> state2;
    DevBuf<uint32_t> path_share2;
    uint32_t state2_paths = 0;
    cudaStream_t wave_side = nullptr;
    cudaEvent_t wfork = nullptr, wjoin = nullptr, wacc[2] = {nullptr, nullptr};
    bool w4 = true; // every job's scene has 4-wide nodes (else the BVH2 kernels run)
    DevBuf<unsigned long long> counters;
    DevBuf<uint32_t> error_word;
    cudaStream_t side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr, ev0 = nullptr, ev1 = nullptr;
    // completion events: one per wave, then one per megakernel job; job_done[j]
    // indexes the event after which job j's image is final
    std::vector<cudaEvent_t> done_ev;
    std::vector<uint32_t> job_done;
    // the captured graph and what it was captured for
    cudaGraphExec_t exec = nullptr;
    std::string graph_key;
    uint32_t graph_launches = 0, graph_waves = 0, graph_mega = 0;
    std::map<std::string, BatchChoice> tune_cache;
};

void batch_free(BatchState* b)
{
    if (!b)
        return;
    b->image.release();
    b->sum64.release();
    b->jobs.release();
    b->shares.release();
    b->path_share.release();
    b->state.release();
    b->state2.release();
    b->path_share2.release();
    b->counters.release();
    b->error_word.release();
    if (b->exec)
        cudaGraphExecDestroy(b->exec);
    if (b->side)
        cudaStreamDestroy(b->side);
    if (b->wave_side)
        cudaStreamDestroy(b->wave_side);
    for (cudaEvent_t e : {b->fork, b->join, b->ev0, b->ev1, b->wfork, b->wjoin, b->wacc[0], b->wacc[1]})
        if (e)
            cudaEventDestroy(e);
    for (cudaEvent_t e : b->done_ev)
        cudaEventDestroy(e);
    delete b;
}

namespace {

// The tuner's trial batch renders every job at max(1, samples / 32) samples;
// the megakernel threshold compares that trial work (path segments at most),
// so the job set it selects is the one the trial timed.
constexpr uint32_t TRIAL_DIVISOR = 32;
uint32_t trial_samples(uint32_t samples) { return std::max<uint32_t>(1, samples / TRIAL_DIVISOR); }
uint64_t job_work(const pt_render_params& p)
{
    return (uint64_t)p.width * p.height * trial_samples(p.samples) * (p.max_bounces + 1ull);
}

bool on_megakernel(const pt_render_params& p, const BatchChoice& ch)
{
    if (p.kernel == PT_KERNEL_MEGA)
        return true;
    if (p.kernel == PT_KERNEL_WAVEFRONT)
        return false;
    return job_work(p) < ch.mega_threshold;
}

// A launch plan: the waves of the wavefront jobs and the megakernel jobs.
struct Plan {
    std::vector<WaveShare> shares;
    std::vector<BatchWave> waves;
    std::vector<uint32_t> mega; // job indices
};

// Packs the wavefront jobs' samples into waves of at most `capacity` paths.
// Jobs with less work (pixels x samples) go first, so small jobs finish in
// the first waves; a job joins a wave with as many whole samples as the
// remaining capacity holds.
bool plan_batch(const std::vector<pt_render_params>& p, const BatchChoice& ch, Plan& plan, std::string& err)
{
    plan = Plan{};
    std::vector<uint32_t> order;
    for (uint32_t j = 0; j < p.size(); j++) {
        if (on_megakernel(p[j], ch))
            plan.mega.push_back(j);
        else
            order.push_back(j);
    }
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) {
        return (uint64_t)p[a].width * p[a].height * p[a].samples < (uint64_t)p[b].width * p[b].height * p[b].samples;
    });
    std::vector<uint32_t> done(p.size(), 0);
    size_t remaining = order.size();
    while (remaining > 0) {
        BatchWave w{(uint32_t)plan.shares.size(), 0u, 0u, 0u, 0u};
        uint64_t left = ch.capacity;
        for (uint32_t j : order) {
            if (done[j] == p[j].samples)
                continue;
            const uint64_t px = (uint64_t)p[j].width * p[j].height;
            const uint64_t k = std::min<uint64_t>(p[j].samples - done[j], left / px);
            if (k == 0)
                continue;
            plan.shares.push_back(WaveShare{j, w.n_paths, w.n_pixels, done[j], (uint32_t)k, (uint32_t)px});
            w.share_count++;
            w.n_paths += (uint32_t)(k * px);
            w.n_pixels += (uint32_t)px;
            w.max_bounces = std::max(w.max_bounces, p[j].max_bounces);
            left -= k * px;
            done[j] += (uint32_t)k;
            if (done[j] == p[j].samples)
                remaining--;
        }
        if (w.share_count == 0) {
            err = "a job has more pixels than the wave capacity";
            return false;
        }
        plan.waves.push_back(w);
    }
    return true;
}

std::string key_of(const pt_batch_job* jobs, uint32_t count, const void* extra, size_t extra_bytes)
{
    std::string k;
    for (uint32_t j = 0; j < count; j++) {
        k.append((const char*)&jobs[j].scene, sizeof(jobs[j].scene));
        k.append((const char*)&jobs[j].scene->scene_generation, sizeof(uint64_t)); // device addresses change with it
        k.append((const char*)&jobs[j].params, sizeof(pt_render_params));
    }
    k.append((const char*)extra, extra_bytes);
    return k;
}

double now_ms()
{
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

} // namespace
} // namespace pt

using namespace pt;

namespace {

// Device memory for the images of `p` (all jobs back to back).
int ensure_images(pt_ctx* c, BatchState* b, const std::vector<pt_render_params>& p)
{
    size_t px = 0, px64 = 0;
    b->img_off.assign(p.size(), 0);
    b->sum_off.assign(p.size(), SIZE_MAX);
    b->width.resize(p.size());
    b->height.resize(p.size());
    for (size_t j = 0; j < p.size(); j++) {
        b->img_off[j] = px;
        px += (size_t)p[j].width * p[j].height;
        b->width[j] = p[j].width;
        b->height[j] = p[j].height;
        if (p[j].accum_mode == PT_ACCUM_FP32_FP64) {
            b->sum_off[j] = px64;
            px64 += (size_t)p[j].width * p[j].height;
        }
    }
    cudaError_t e = cudaSuccess;
    if (b->image.n < px) {
        b->graph_key.clear(); // the cached graph holds the old addresses
        e = b->image.alloc(px);
    }
    if (e == cudaSuccess && px64 && b->sum64.n < 4 * px64) {
        b->graph_key.clear();
        e = b->sum64.alloc(4 * px64);
    }
    return e == cudaSuccess ? PT_OK : c->cuda_fail(e, "batch image allocation");
}

// Uploads the plan's job table and shares and makes room for its waves.  The
// cached graph reads these tables, so it is dropped here and recaptured.
int prepare(pt_ctx* c, BatchState* b, const pt_batch_job* jobs, const std::vector<pt_render_params>& p, const Plan& plan,
            uint32_t capacity)
{
    b->graph_key.clear();
    std::vector<RenderArgs> args(p.size());
    b->w4 = true;
    for (size_t j = 0; j < p.size(); j++) {
        RenderArgs a = render_args(jobs[j].scene, &p[j], false);
        b->w4 = b->w4 && a.s.nodes4 != nullptr;
        a.image = b->image.p + b->img_off[j];
        a.sum64 = b->sum_off[j] == SIZE_MAX ? nullptr : b->sum64.p + 4 * b->sum_off[j];
        a.counters = b->counters.p;
        a.s.error_word = b->error_word.p;
        a.sample_index = 0;
        a.samples = p[j].samples;
        args[j] = a;
    }
    cudaError_t e = cudaSuccess;
    if (b->jobs.n < args.size())
        e = b->jobs.alloc(args.size());
    if (e == cudaSuccess && b->shares.n < std::max<size_t>(plan.shares.size(), 1))
        e = b->shares.alloc(std::max<size_t>(plan.shares.size(), 1));
    // the state is sized to the capacity exactly: a wave's arrays stay close together
    if (e == cudaSuccess && !plan.waves.empty() && b->state_paths != capacity) {
        b->state.release();
        b->path_share.release();
        e = b->state.alloc(wave_state_bytes(capacity));
        if (e == cudaSuccess)
            e = b->path_share.alloc(capacity);
        b->state_paths = e == cudaSuccess ? capacity : 0;
    }
    // a second state for plans of two or more waves (they alternate over two streams)
    if (e == cudaSuccess && plan.waves.size() >= 2 && b->state2_paths != capacity) {
        b->state2.release();
        b->path_share2.release();
        e = b->state2.alloc(wave_state_bytes(capacity));
        if (e == cudaSuccess)
            e = b->path_share2.alloc(capacity);
        b->state2_paths = e == cudaSuccess ? capacity : 0;
    }
    if (e != cudaSuccess)
        return c->cuda_fail(e, "batch allocation");
    // completion events (created before any capture), and each job's last one
    const size_t need = plan.waves.size() + plan.mega.size();
    while (b->done_ev.size() < need) {
        cudaEvent_t ev;
        if ((e = cudaEventCreate(&ev)) != cudaSuccess)
            return c->cuda_fail(e, "batch events");
        b->done_ev.push_back(ev);
    }
    b->job_done.assign(p.size(), 0);
    for (size_t w = 0; w < plan.waves.size(); w++)
        for (uint32_t s = 0; s < plan.waves[w].share_count; s++)
            b->job_done[plan.shares[plan.waves[w].share_offset + s].job] = (uint32_t)w;
    for (size_t k = 0; k < plan.mega.size(); k++)
        b->job_done[plan.mega[k]] = (uint32_t)(plan.waves.size() + k);
    e = cudaMemcpyAsync(b->jobs.p, args.data(), args.size() * sizeof(RenderArgs), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess && !plan.shares.empty())
        e = cudaMemcpyAsync(b->shares.p, plan.shares.data(), plan.shares.size() * sizeof(WaveShare), cudaMemcpyHostToDevice,
                            c->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(c->stream); // the host arrays above go out of scope
    return e == cudaSuccess ? PT_OK : c->cuda_fail(e, "batch upload");
}

// The batch's launch sequence on c->stream (and b->side for megakernel jobs):
// image/counter resets, the waves, the megakernel launches, the join.
cudaError_t issue(pt_ctx* c, BatchState* b, const pt_batch_job* jobs, const std::vector<pt_render_params>& p, const Plan& plan,
                  const BatchChoice& ch, uint32_t* launches)
{
    cudaStream_t st = c->stream;
    uint32_t nl = 0;
    size_t px = 0, px64 = 0;
    for (size_t j = 0; j < p.size(); j++) {
        px = std::max(px, b->img_off[j] + (size_t)p[j].width * p[j].height);
        if (b->sum_off[j] != SIZE_MAX)
            px64 = std::max(px64, b->sum_off[j] + (size_t)p[j].width * p[j].height);
    }
    cudaError_t e = cudaMemsetAsync(b->image.p, 0, px * sizeof(float4), st);
    if (e == cudaSuccess && px64)
        e = cudaMemsetAsync(b->sum64.p, 0, 4 * px64 * sizeof(double), st);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(b->counters.p, 0, 8 * sizeof(unsigned long long), st);
    if (e != cudaSuccess)
        return e;
    if (!plan.mega.empty()) {
        cudaEventRecord(b->fork, st);
        cudaStreamWaitEvent(b->side, b->fork, 0);
        for (uint32_t j : plan.mega) {
            RenderArgs a = render_args(jobs[j].scene, &p[j], false);
            a.image = b->image.p + b->img_off[j];
            a.sum64 = b->sum_off[j] == SIZE_MAX ? nullptr : b->sum64.p + 4 * b->sum_off[j];
            a.counters = b->counters.p;
            a.s.error_word = b->error_word.p;
            const uint64_t pixels = (uint64_t)p[j].width * p[j].height;
            const uint32_t per_launch = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(p[j].samples, (1ull << 26) / pixels));
            for (uint32_t d = 0; d < p[j].samples; d += per_launch) {
                a.sample_index = d;
                a.samples = std::min(per_launch, p[j].samples - d);
                if ((e = launch_megakernel_tiled(a, ch.tile_w, b->side)) != cudaSuccess)
                    return e;
                nl++;
            }
            record_timed(b->done_ev[b->job_done[j]], b->side);
        }
    }
    if (!plan.waves.empty()) {
        uint32_t wl = 0;
        WaveMulti wm{};
        const bool two = plan.waves.size() >= 2 && b->state2_paths == b->state_paths;
        if (two) {
            wm.ways = 2;
            wm.state[1] = b->state2.p;
            wm.state_bytes[1] = b->state2.n;
            wm.stream[1] = b->wave_side;
            wm.fork = b->wfork;
            wm.join[1] = b->wjoin;
            wm.acc[0] = b->wacc[0];
            wm.acc[1] = b->wacc[1];
        }
        e = launch_wavefront_batch(b->jobs.p, b->shares.p, plan.waves.data(), (uint32_t)plan.waves.size(), b->path_share.p,
                                   b->counters.p, b->state.p, b->state.n, b->state_paths, b->w4, c->sm_count, &wl, st,
                                   two ? &wm : nullptr, two ? b->path_share2.p : nullptr, b->done_ev.data());
        if (e != cudaSuccess)
            return e;
        nl += wl;
    }
    if (!plan.mega.empty()) {
        cudaEventRecord(b->join, b->side);
        cudaStreamWaitEvent(st, b->join, 0);
    }
    if (launches)
        *launches = nl;
    return cudaGetLastError();
}

// Runs one batch (plan + issue) directly and returns its device time.
int trial(pt_ctx* c, BatchState* b, const pt_batch_job* jobs, const std::vector<pt_render_params>& p, const BatchChoice& ch,
          float& ms)
{
    Plan plan;
    std::string err;
    if (!plan_batch(p, ch, plan, err))
        return c->fail(PT_ERR_INVALID, err);
    int rc = prepare(c, b, jobs, p, plan, ch.capacity);
    if (rc != PT_OK)
        return rc;
    cudaEventRecord(b->ev0, c->stream);
    cudaError_t e = issue(c, b, jobs, p, plan, ch, nullptr);
    if (e != cudaSuccess)
        return c->cuda_fail(e, "batch trial");
    cudaEventRecord(b->ev1, c->stream);
    if ((e = cudaEventSynchronize(b->ev1)) != cudaSuccess)
        return c->cuda_fail(e, "batch trial");
    cudaEventElapsedTime(&ms, b->ev0, b->ev1);
    return PT_OK;
}

// `fixed_capacity` != 0 skips the capacity stage.
int tune(pt_ctx* c, BatchState* b, const pt_batch_job* jobs, const std::vector<pt_render_params>& p, uint32_t fixed_capacity,
         BatchChoice& best)
{
    std::vector<pt_render_params> tp = p;
    for (auto& q : tp)
        q.samples = trial_samples(q.samples);
    uint64_t max_px = 0;
    for (auto& q : p)
        max_px = std::max<uint64_t>(max_px, (uint64_t)q.width * q.height);
    float best_ms = 0.0f;
    bool have = false;
    // capacities whose two path states would take more than a quarter of the free memory are skipped
    size_t free_b = 0, total_b = 0;
    uint64_t mem_paths = ~0ull;
    if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess)
        mem_paths = ((uint64_t)free_b + (uint64_t)b->state.n + (uint64_t)b->state2.n) / 8 / (wave_state_bytes(1u << 20) >> 20);
    // times one setting; `ran` is false when the setting does not apply
    auto measure = [&](const BatchChoice& ch, float& ms, bool& ran) -> int {
        ran = false;
        if (max_px > ch.capacity)
            return PT_OK; // the largest job would not fit a wave
        if (ch.capacity > mem_paths && ch.capacity > (1u << 21))
            return PT_OK;
        const int rc = trial(c, b, jobs, tp, ch, ms);
        ran = rc == PT_OK;
        return rc;
    };
    auto consider = [&](const BatchChoice& ch) -> int {
        float ms = 0.0f;
        bool ran = false;
        const int rc = measure(ch, ms, ran);
        if (rc != PT_OK || !ran)
            return rc;
        if (!have || ms < best_ms) {
            best_ms = ms;
            best = ch;
            have = true;
        }
        return PT_OK;
    };
    int rc;
    // Capacity: the trial batch holds 1/32 of the samples, so its waves are
    // emptier than the real batch's and it understates what larger waves gain
    // (fuller late segments, fewer launches per sample); a larger capacity is
    // kept unless a smaller one is more than 3 % faster in the trial.
    for (uint32_t lg : {26u, 25u, 23u, 21u}) {
        BatchChoice ch;
        ch.capacity = fixed_capacity ? fixed_capacity : 1u << lg;
        float ms = 0.0f;
        bool ran = false;
        if ((rc = measure(ch, ms, ran)) != PT_OK)
            return rc;
        if (ran && (!have || ms * 1.03f < best_ms)) {
            best_ms = ms;
            best = ch;
            have = true;
        }
        if (fixed_capacity)
            break;
    }
    if (!have)
        return c->fail(PT_ERR_UNSUPPORTED, "a job has more pixels than the wave capacity");
    // the trial batch has 1/32 of the samples: scale the thresholds the same way
    const BatchChoice base = best;
    for (uint64_t thr : {1ull << 18, 1ull << 21}) {
        BatchChoice ch = base;
        ch.mega_threshold = thr;
        if ((rc = consider(ch)) != PT_OK)
            return rc;
    }
    if (best.mega_threshold) {
        const BatchChoice with = best;
        for (uint32_t tw : {8u, 32u}) {
            BatchChoice ch = with;
            ch.tile_w = tw;
            if ((rc = consider(ch)) != PT_OK)
                return rc;
        }
    }
    return PT_OK;
}

} // namespace

extern "C" {

int pt_render_batch(pt_ctx* c, const pt_batch_job* jobs, uint32_t count, uint32_t flags, pt_batch_stats* stats)
{
    if (!c || (!jobs && count))
        return PT_ERR_INVALID;
    if (count == 0)
        return c->fail(PT_ERR_INVALID, "empty batch");
    if (flags & ~(PT_BATCH_NO_TUNE | PT_BATCH_NO_GRAPH | PT_BATCH_RETUNE | PT_BATCH_CAPACITY_LOG2(31)))
        return c->fail(PT_ERR_INVALID, "unknown batch flags");
    const uint32_t cap_log2 = (flags >> 8) & 31u;
    if (cap_log2 && (cap_log2 < 10 || cap_log2 > 25))
        return c->fail(PT_ERR_INVALID, "wave capacity must be 2^10 .. 2^25 paths");
    const uint32_t fixed_capacity = cap_log2 ? 1u << cap_log2 : 0u;
    cudaSetDevice(c->device);
    std::vector<pt_render_params> p(count);
    for (uint32_t j = 0; j < count; j++) {
        const pt_render_params& q = jobs[j].params;
        const pt_ctx* s = jobs[j].scene;
        const std::string at = "job " + std::to_string(j) + ": ";
        if (!s || !s->accel_ok)
            return c->fail(PT_ERR_STATE, at + "scene without an acceleration structure");
        if (s->device != c->device)
            return c->fail(PT_ERR_INVALID, at + "scene on another device");
        if (q.width == 0 || q.height == 0 || q.samples == 0)
            return c->fail(PT_ERR_INVALID, at + "zero width, height or sample count");
        if ((uint64_t)q.width * q.height > (1ull << 25))
            return c->fail(PT_ERR_UNSUPPORTED, at + "more than 2^25 pixels");
        if (q.sample_index != 0 || q.flags != 0)
            return c->fail(PT_ERR_INVALID, at + "batch jobs start at sample 0 and take no flags");
        if (q.accum_mode > PT_ACCUM_FP32_FP64 || q.kernel > PT_KERNEL_WAVEFRONT)
            return c->fail(PT_ERR_INVALID, at + "unknown accumulation mode or kernel");
        p[j] = q;
    }
    if (!c->batch) {
        BatchState* b = new (std::nothrow) BatchState();
        if (!b)
            return c->fail(PT_ERR_OOM, "batch state");
        cudaError_t e = cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking);
        if (e == cudaSuccess)
            e = cudaStreamCreateWithFlags(&b->wave_side, cudaStreamNonBlocking);
        for (cudaEvent_t* ev : {&b->fork, &b->join, &b->wfork, &b->wjoin, &b->wacc[0], &b->wacc[1]})
            if (e == cudaSuccess)
                e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
        for (cudaEvent_t* ev : {&b->ev0, &b->ev1})
            if (e == cudaSuccess)
                e = cudaEventCreate(ev);
        if (e == cudaSuccess)
            e = b->counters.alloc(8);
        if (e == cudaSuccess)
            e = b->error_word.alloc(1);
        if (e == cudaSuccess)
            e = cudaMemset(b->error_word.p, 0, sizeof(uint32_t));
        if (e != cudaSuccess) {
            batch_free(b);
            return c->cuda_fail(e, "batch state");
        }
        c->batch = b;
    }
    BatchState* b = c->batch;
    int rc = ensure_images(c, b, p);
    if (rc != PT_OK)
        return rc;

    // settings: default, cached or tuned
    const std::string tune_key = key_of(jobs, count, &fixed_capacity, sizeof(fixed_capacity));
    BatchChoice ch;
    if (fixed_capacity)
        ch.capacity = fixed_capacity;
    for (const auto& q : p)
        if ((uint64_t)q.width * q.height > ch.capacity)
            return c->fail(PT_ERR_UNSUPPORTED, "a job has more pixels than the wave capacity");
    double tune_ms = 0.0;
    if (!(flags & PT_BATCH_NO_TUNE)) {
        auto it = b->tune_cache.find(tune_key);
        if (it != b->tune_cache.end() && !(flags & PT_BATCH_RETUNE)) {
            ch = it->second;
        } else {
            const double t0 = now_ms();
            if ((rc = tune(c, b, jobs, p, fixed_capacity, ch)) != PT_OK)
                return rc;
            tune_ms = now_ms() - t0;
            b->tune_cache[tune_key] = ch;
        }
    }

    const bool graph = !(flags & PT_BATCH_NO_GRAPH);
    const std::string graph_key = key_of(jobs, count, &ch, sizeof(ch));
    const bool reuse = graph && b->exec && graph_key == b->graph_key;
    double build_ms = 0.0;
    uint32_t launches = 0, waves = 0, mega = 0;
    cudaError_t e = cudaSuccess;
    if (reuse) {
        launches = b->graph_launches;
        waves = b->graph_waves;
        mega = b->graph_mega;
    } else {
        const double t0 = now_ms();
        Plan plan;
        std::string err;
        if (!plan_batch(p, ch, plan, err))
            return c->fail(PT_ERR_INVALID, err);
        if ((rc = prepare(c, b, jobs, p, plan, ch.capacity)) != PT_OK)
            return rc;
        waves = (uint32_t)plan.waves.size();
        mega = (uint32_t)plan.mega.size();
        if (graph) {
            if (b->exec) {
                cudaGraphExecDestroy(b->exec);
                b->exec = nullptr;
                b->graph_key.clear();
            }
            // occupancy queries happen outside the capture
            cudaGraph_t g = nullptr;
            e = wave_batch_prepare();
            if (e == cudaSuccess)
                e = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal);
            if (e == cudaSuccess) {
                cudaError_t ei = issue(c, b, jobs, p, plan, ch, &launches);
                e = cudaStreamEndCapture(c->stream, &g);
                if (ei != cudaSuccess)
                    e = ei;
            }
            if (e == cudaSuccess)
                e = cudaGraphInstantiate(&b->exec, g, 0);
            if (g)
                cudaGraphDestroy(g);
            if (e != cudaSuccess) {
                b->exec = nullptr;
                return c->cuda_fail(e, "batch graph capture");
            }
            b->graph_key = graph_key;
            b->graph_launches = launches;
            b->graph_waves = waves;
            b->graph_mega = mega;
        }
        build_ms = now_ms() - t0;
        if (!graph) {
            cudaEventRecord(b->ev0, c->stream);
            e = issue(c, b, jobs, p, plan, ch, &launches);
            if (e != cudaSuccess)
                return c->cuda_fail(e, "batch launch");
            cudaEventRecord(b->ev1, c->stream);
        }
    }
    if (graph) {
        cudaEventRecord(b->ev0, c->stream);
        if ((e = cudaGraphLaunch(b->exec, c->stream)) != cudaSuccess)
            return c->cuda_fail(e, "batch graph launch");
        cudaEventRecord(b->ev1, c->stream);
    }
    if ((e = cudaStreamSynchronize(c->stream)) != cudaSuccess)
        return c->cuda_fail(e, "batch render");
    unsigned long long cnt[8];
    uint32_t ew = 0;
    cudaMemcpy(cnt, b->counters.p, sizeof(cnt), cudaMemcpyDeviceToHost);
    cudaMemcpy(&ew, b->error_word.p, sizeof(ew), cudaMemcpyDeviceToHost);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, b->ev0, b->ev1);
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        stats->segments = cnt[0];
        stats->shadow_rays = cnt[1];
        stats->paths = cnt[2];
        stats->milliseconds = ms;
        stats->tune_milliseconds = (float)tune_ms;
        stats->build_milliseconds = (float)build_ms;
        stats->waves = waves;
        stats->kernel_launches = launches;
        stats->mega_jobs = mega;
        stats->wave_capacity = ch.capacity;
        stats->tile_w = ch.tile_w;
        stats->graph_reused = reuse ? 1u : 0u;
        stats->mega_threshold = ch.mega_threshold;
        stats->error_word = ew;
    }
    if (ew != 0)
        return c->fail((ew & ERR_WATCHDOG) ? PT_ERR_TIMEOUT : PT_ERR_DEVICE,
                      std::string((ew & ERR_WATCHDOG) ? "traversal iteration cap hit" : "device error") + " (error word " +
                          std::to_string(ew) + ")");
    return PT_OK;
}

int pt_batch_job_times(pt_ctx* c, float* ms, uint32_t count)
{
    if (!c || !ms)
        return PT_ERR_INVALID;
    BatchState* b = c->batch;
    if (!b || b->job_done.empty())
        return c->fail(PT_ERR_STATE, "no batch rendered");
    if (count != b->job_done.size())
        return c->fail(PT_ERR_INVALID, "count differs from the last batch's job count");
    cudaSetDevice(c->device);
    for (uint32_t j = 0; j < count; j++) {
        cudaError_t e = cudaEventElapsedTime(&ms[j], b->ev0, b->done_ev[b->job_done[j]]);
        if (e != cudaSuccess)
            return c->cuda_fail(e, "batch job times");
    }
    return PT_OK;
}

int pt_read_batch_image(pt_ctx* c, uint32_t job, void* rgba, size_t pitch, int fp64)
{
    if (!c || !rgba)
        return PT_ERR_INVALID;
    BatchState* b = c->batch;
    if (!b || job >= b->img_off.size())
        return c->fail(PT_ERR_STATE, "no such batch job");
    cudaSetDevice(c->device);
    const uint32_t w = b->width[job], h = b->height[job];
    cudaError_t e;
    if (!fp64) {
        if (pitch < (size_t)w * 16)
            return c->fail(PT_ERR_INVALID, "pitch smaller than a row");
        e = cudaMemcpy2DAsync(rgba, pitch, b->image.p + b->img_off[job], (size_t)w * 16, (size_t)w * 16, h, cudaMemcpyDeviceToHost,
                              c->stream);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(c->stream);
        return e == cudaSuccess ? PT_OK : c->cuda_fail(e, "batch image read-back");
    }
    if (fp64 != 1)
        return c->fail(PT_ERR_INVALID, "fp64 must be 0 or 1");
    if (b->sum_off[job] == SIZE_MAX)
        return c->fail(PT_ERR_STATE, "job rendered without FP64 sums (PT_ACCUM_FP32_FP64)");
    if (pitch < (size_t)w * 32)
        return c->fail(PT_ERR_INVALID, "pitch smaller than a row");
    const size_t n = (size_t)w * h;
    std::vector<double> sums(4 * n);
    e = cudaMemcpyAsync(sums.data(), b->sum64.p + 4 * b->sum_off[job], 4 * n * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess)
        return c->cuda_fail(e, "batch FP64 read-back");
    for (uint32_t y = 0; y < h; y++) {
        double* row = (double*)((char*)rgba + pitch * y);
        for (uint32_t x = 0; x < w; x++) {
            const double* s = &sums[4 * ((size_t)y * w + x)];
            const double cnt = s[3] > 0.0 ? s[3] : 1.0;
            row[4 * x + 0] = s[0] / cnt;
            row[4 * x + 1] = s[1] / cnt;
            row[4 * x + 2] = s[2] / cnt;
            row[4 * x + 3] = 1.0;
        }
    }
    return PT_OK;
}

} // extern "C"
