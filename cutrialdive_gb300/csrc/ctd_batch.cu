// ctd_batch.cu -- many jobs at once: the batched runner and the server.
//
// The reference runs one job per process (src/main.cpp:94-146) and one
// kernel launch per sieve segment (src/trial_factoring.cuh:437-488); it has
// no batching or serving layer.  Here:
//
// * ctd_batch_run walks the union of the jobs' prime ranges segment by
//   segment ("chunk-major"): each aligned segment is sieved once and
//   consumed by every job whose range covers it: persistent walk launches
//   over (job, 32 primes, index tile) work items, one per walk group present
//   (doubling over power-residue classes, doubling over every term,
//   Smarandache, the rest: each group's kernel has the code, occupancy and
//   registers its families need; launch_batch, ctd_residue.cu).  The whole schedule -- sieves, class and
//   plan kernels, walks -- is captured once into a CUDA graph; a later call
//   with the same schedule replays it, one with the same shape updates the
//   instantiated graph in place, and the device buffers stay with the
//   context (grown, never freed per call).
// * ctd_serve_* keeps a device job table with a progress cursor per job
//   (advanced by the kernels), admits queued jobs by slots and a device
//   memory budget (ctd_admission.h) while earlier ticks still run, and
//   queues each tick's work without waiting for the previous one: ticks
//   overlap with the host's admission and result handling, and a finished
//   job's results travel back by an asynchronous copy the host collects
//   when its event has completed.
#include "ctd_admission.h"
#include "ctd_internal.h"

#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <map>
#include <new>
#include <string>
#include <vector>

using namespace ctd;

namespace {

#define CTX_TRY(expr)                                                                     \
    do {                                                                                  \
        cudaError_t e_ = (expr);                                                          \
        if (e_ != cudaSuccess)                                                            \
            return ctx_fail(ctx, e_ == cudaErrorMemoryAllocation ? CTD_ERR_OUT_OF_MEMORY \
                                                                  : CTD_ERR_CUDA,         \
                            std::string(#expr ": ") + cudaGetErrorString(e_));            \
    } while (0)

constexpr uint32_t MAX_ACTIVE_PER_LAUNCH = 1 << 16;

// counts padded to 256 bytes so the factors that follow stay aligned
uint64_t counts_bytes(const ctd_job &j) { return ((j.n1 - j.n0) * sizeof(uint32_t) + 255) & ~uint64_t{255}; }

uint64_t job_bytes(const ctd_job &j)
{
    return counts_bytes(j) + (j.n1 - j.n0) * (uint64_t)j.max_factors * sizeof(uint64_t);
}

// odd-prime range of a job after the prime 2 is handled separately
uint64_t odd_f0(const ctd_job &j) { return j.f0 <= 2 ? 3 : j.f0; }

bool is_doubling(uint32_t f) { return f == CTD_PROTH || f == CTD_RIESEL || f == CTD_MERSENNE; }

// Index tiles of a batched job: the longest units a warp item may take, so
// a long range spreads over many warps.  Each tile starts with the family's
// O(log n) jump, which for Smarandache costs about a seventh of a
// 4096-term walk (measured: 4096-term tiles ran the batched Smarandache walk
// 10 % slower than the untiled per-job kernel), so Smarandache and the
// doubling walks are cut at 32768 terms and tribonacci at 16384; the
// rank-of-apparition (Fibonacci, Lucas) and closed-form (fixed-n) paths
// depend on the whole range and stay whole.
uint64_t tile_limit(uint32_t family)
{
    switch (family) {
    case CTD_SMARANDACHE: return 32768;
    case CTD_TRIBONACCI: return 16384;
    case CTD_PROTH:
    case CTD_RIESEL:
    case CTD_MERSENNE: return 32768;
    default: return ~0ull;
    }
}

// relative cost of one term, for ordering a segment's jobs heaviest first
double term_cost(uint32_t family)
{
    switch (family) {
    case CTD_SMARANDACHE: return 11.0;
    case CTD_TRIBONACCI: return 3.2;
    case CTD_FIBONACCI:
    case CTD_LUCAS: return 0.5;
    case CTD_PROTH:
    case CTD_RIESEL:
    case CTD_MERSENNE: return 0.2;
    default: return 0.01;
    }
}

BatchJob batch_job_of(ctd_ctx *ctx, const ctd_job &j, uint32_t *counts, uint64_t *factors)
{
    BatchJob b{};
    JobView &v = b.view;
    const ctd_tuning t = ctx_tuning(ctx, j.family, j.f0);
    v.family = j.family;
    v.variant = t.variant;
    v.classify_min = t.classify_min ? t.classify_min : DEFAULT_CLASSIFY_MIN;
    v.refine_q = t.refine_q;
    v.param = j.param;
    v.n0 = j.n0;
    v.n1 = j.n1;
    const uint64_t N = j.n1 - j.n0;
    // index tiles: the family's limit, raised to the tuned shortest tile
    const uint64_t lim = tile_limit(j.family) == ~0ull ? ~0ull : std::max<uint64_t>(tile_limit(j.family), t.min_tile);
    v.tiles = (uint32_t)(N <= lim ? 1 : std::min<uint64_t>((N + lim - 1) / lim, 1u << 20));
    v.tile_len = (N + v.tiles - 1) / v.tiles;
    v.tiles = (uint32_t)((N + v.tile_len - 1) / v.tile_len);
    v.fb.counts = counts;
    v.fb.factors = factors;
    v.fb.max_factors = j.max_factors;
    b.f0 = odd_f0(j);
    b.f1 = j.f1;
    b.cursor = b.f0;
    b.classified = is_doubling(j.family) && v.variant == CTD_VARIANT_AUTO && N >= v.classify_min;
    return b;
}

template <class T>
cudaError_t grow(T *&p, size_t &cap, size_t n)
{
    if (n <= cap && p)
        return cudaSuccess;
    cudaFree(p);
    p = nullptr;
    cap = 0;
    cudaError_t e = cudaMalloc(&p, (n ? n : 1) * sizeof(T));
    if (e == cudaSuccess)
        cap = n;
    return e;
}

// FNV-1a, for the key of a captured schedule
struct Hasher {
    uint64_t h = 1469598103934665603ull;
    template <class T>
    void add(const T &x)
    {
        const unsigned char *b = reinterpret_cast<const unsigned char *>(&x);
        for (size_t i = 0; i < sizeof(T); ++i) {
            h ^= b[i];
            h *= 1099511628211ull;
        }
    }
};

}  // namespace

namespace ctd {

// Device buffers of the batched runner, kept across calls, and the
// instantiated graph of the last schedule with its key.
struct BatchCache {
    unsigned char *fb = nullptr;
    size_t fb_cap = 0;
    BatchJob *jobs = nullptr;
    size_t jobs_cap = 0;
    uint32_t *active = nullptr;
    size_t active_cap = 0;
    uint64_t *primes = nullptr;
    size_t primes_cap = 0;
    BatchSpan *spans = nullptr;
    size_t spans_cap = 0;
    BatchControl *ctl = nullptr;
    size_t ctl_cap = 0;
    uint32_t *codes = nullptr;
    size_t codes_cap = 0;
    ClassItem *items = nullptr;
    size_t items_cap = 0;
    uint32_t *bucket = nullptr;  // counts, cursors, bases: 3 x nactive x CLASS_BUCKETS
    size_t bucket_cap = 0;
    cudaGraphExec_t exec = nullptr;
    uint64_t key = 0;
    uint64_t graph_launches = 0;  // kernel launches in the captured schedule
    uint64_t replays = 0, updates = 0, instantiations = 0;

    BatchScratch scratch(uint32_t nactive) const
    {
        BatchScratch s;
        s.spans = spans;
        s.ctl = ctl;
        s.codes = codes;
        s.items = items;
        s.class_cap = std::min<uint64_t>(codes_cap, items_cap);
        s.bucket_count = bucket;
        s.bucket_base = bucket + 2ull * nactive * CLASS_BUCKETS;
        return s;
    }
};

void batch_cache_destroy(BatchCache *bc)
{
    if (!bc)
        return;
    if (bc->exec)
        cudaGraphExecDestroy(bc->exec);
    cudaFree(bc->fb);
    cudaFree(bc->jobs);
    cudaFree(bc->active);
    cudaFree(bc->primes);
    cudaFree(bc->spans);
    cudaFree(bc->ctl);
    cudaFree(bc->codes);
    cudaFree(bc->items);
    cudaFree(bc->bucket);
    delete bc;
}

}  // namespace ctd

namespace {

// One segment of a schedule: its range and its active jobs (a slice of the
// concatenated active list), heaviest first.
struct Segment {
    uint64_t lo, hi;
    uint32_t first, count;
    uint32_t gcount[BATCH_GROUPS];  // jobs per walk group (the slice is group-major)
    bool any_classified;
};

// a segment's active jobs ordered walk group by walk group, heaviest work
// per prime first within a group (the walks hand out items in this order)
template <class Terms, class Family, class Group>
void order_active(std::vector<uint32_t> &act, uint32_t gcount[BATCH_GROUPS], Terms terms, Family family, Group group)
{
    std::stable_sort(act.begin(), act.end(), [&](uint32_t x, uint32_t y) {
        const int gx = group(x), gy = group(y);
        if (gx != gy)
            return gx < gy;
        return (double)terms(x) * term_cost(family(x)) > (double)terms(y) * term_cost(family(y));
    });
    for (int g = 0; g < BATCH_GROUPS; ++g)
        gcount[g] = 0;
    for (uint32_t x : act)
        ++gcount[group(x)];
}

// The segments of [lo, hi) aligned to S that some job covers, and their
// active jobs; also the largest per-segment needs for sizing scratch.
struct Schedule {
    std::vector<Segment> segs;
    std::vector<uint32_t> active;
    uint64_t primes_cap = 0;
    uint64_t class_cap = 0;
    uint32_t max_active = 1;
};

Schedule plan_schedule(const std::vector<BatchJob> &hjobs, const ctd_job *jobs, uint64_t S)
{
    Schedule sc;
    uint64_t lo = ~0ull, hi = 0;
    for (const BatchJob &b : hjobs)
        if (b.f0 < b.f1) {
            lo = std::min(lo, b.f0);
            hi = std::max(hi, b.f1);
        }
    if (lo >= hi)
        return sc;
    for (uint64_t k = lo / S; k * S < hi && k <= (~0ull / S); ++k) {
        Segment sg;
        sg.lo = std::max(k * S, lo);
        sg.hi = (k + 1 > ~0ull / S) ? hi : std::min((k + 1) * S, hi);
        std::vector<uint32_t> act;
        uint64_t ncls = 0;
        for (uint32_t i = 0; i < hjobs.size(); ++i)
            if (hjobs[i].f0 < sg.hi && hjobs[i].f1 > sg.lo) {
                act.push_back(i);
                if (hjobs[i].classified)
                    ncls += prime_count_upper_bound(std::max(sg.lo, hjobs[i].f0), std::min(sg.hi, hjobs[i].f1));
            }
        if (act.empty())
            continue;
        for (size_t b = 0; b < act.size(); b += MAX_ACTIVE_PER_LAUNCH) {
            Segment part = sg;
            part.first = (uint32_t)sc.active.size();
            part.count = (uint32_t)std::min<size_t>(MAX_ACTIVE_PER_LAUNCH, act.size() - b);
            std::vector<uint32_t> slice(act.begin() + b, act.begin() + b + part.count);
            order_active(
                slice, part.gcount, [&](uint32_t x) { return jobs[x].n1 - jobs[x].n0; },
                [&](uint32_t x) { return jobs[x].family; },
                [&](uint32_t x) { return batch_group(jobs[x].family, hjobs[x].classified != 0); });
            part.any_classified = false;
            for (uint32_t x : slice)
                part.any_classified |= hjobs[x].classified != 0;
            sc.active.insert(sc.active.end(), slice.begin(), slice.end());
            sc.max_active = std::max(sc.max_active, part.count);
            sc.segs.push_back(part);
        }
        sc.primes_cap = std::max(sc.primes_cap, prime_count_upper_bound(sg.lo, sg.hi));
        sc.class_cap = std::max(sc.class_cap, ncls);
    }
    return sc;
}

}  // namespace

extern "C" {

int ctd_batch_run(ctd_ctx *ctx, const ctd_job *jobs, uint32_t njobs, uint32_t *const *counts_inout,
                  uint64_t *const *factors_inout, uint64_t segment_length, int use_graph)
{
    if (!ctx || (!jobs && njobs) || (njobs && (!counts_inout || !factors_inout)))
        return ctx ? ctx_fail(ctx, CTD_ERR_INVALID_ARGUMENT, "ctd_batch_run: bad arguments")
                   : CTD_ERR_INVALID_ARGUMENT;
    if (!njobs)
        return CTD_OK;
    for (uint32_t i = 0; i < njobs; ++i)
        if (ctd_check_job(&jobs[i]) || jobs[i].f1 <= jobs[i].f0 || !counts_inout[i] || !factors_inout[i])
            return ctx_fail(ctx, CTD_ERR_INVALID_ARGUMENT, "ctd_batch_run: invalid job " + std::to_string(i));
    const uint64_t S = segment_length ? segment_length : (1ull << 30);
    CTX_TRY(cudaSetDevice(ctx_device(ctx)));
    cudaStream_t st = ctx_stream(ctx);
    std::string err;
    BatchCache *&bcref = ctx_batch_cache(ctx);
    if (!bcref) {
        bcref = new (std::nothrow) BatchCache();
        if (!bcref)
            return ctx_fail(ctx, CTD_ERR_OUT_OF_MEMORY, "ctd_batch_run: host allocation");
    }
    BatchCache &bc = *bcref;

    // factors buffers: one region, grown across calls
    std::vector<uint64_t> off(njobs + 1, 0);
    for (uint32_t i = 0; i < njobs; ++i)
        off[i + 1] = off[i] + job_bytes(jobs[i]);
    CTX_TRY(grow(bc.fb, bc.fb_cap, off[njobs]));
    std::vector<BatchJob> hjobs(njobs);
    for (uint32_t i = 0; i < njobs; ++i) {
        auto *dc = reinterpret_cast<uint32_t *>(bc.fb + off[i]);
        auto *df = reinterpret_cast<uint64_t *>(bc.fb + off[i] + counts_bytes(jobs[i]));
        hjobs[i] = batch_job_of(ctx, jobs[i], dc, df);
    }
    const Schedule sc = plan_schedule(hjobs, jobs, S);
    CTX_TRY(grow(bc.jobs, bc.jobs_cap, njobs));
    CTX_TRY(grow(bc.active, bc.active_cap, std::max<size_t>(sc.active.size(), 1)));
    CTX_TRY(grow(bc.primes, bc.primes_cap, std::max<uint64_t>(sc.primes_cap, 1)));
    CTX_TRY(grow(bc.spans, bc.spans_cap, sc.max_active + 1));
    CTX_TRY(grow(bc.ctl, bc.ctl_cap, 1));
    CTX_TRY(grow(bc.codes, bc.codes_cap, std::max<uint64_t>(sc.class_cap, 1)));
    CTX_TRY(grow(bc.items, bc.items_cap, std::max<uint64_t>(sc.class_cap, 1)));
    CTX_TRY(grow(bc.bucket, bc.bucket_cap, 3ull * sc.max_active * CLASS_BUCKETS));
    if (!sc.segs.empty()) {
        uint64_t hi = 0;
        for (const Segment &g : sc.segs)
            hi = std::max(hi, g.hi);
        int rc = sieve_prepare_base(ctx_workspace(ctx), hi, st, err);
        if (!rc)
            rc = sieve_prepare_windows(ctx_workspace(ctx), S, err);
        if (rc)
            return ctx_fail(ctx, rc, err);
    }

    // inputs of this call: resume states, job table (cursors reset), active lists
    for (uint32_t i = 0; i < njobs; ++i) {
        const ctd_job &j = jobs[i];
        const uint64_t N = j.n1 - j.n0;
        CTX_TRY(cudaMemcpyAsync(hjobs[i].view.fb.counts, counts_inout[i], N * sizeof(uint32_t), cudaMemcpyHostToDevice,
                                st));
        CTX_TRY(cudaMemcpyAsync(hjobs[i].view.fb.factors, factors_inout[i], N * j.max_factors * sizeof(uint64_t),
                                cudaMemcpyHostToDevice, st));
    }
    CTX_TRY(cudaMemcpyAsync(bc.jobs, hjobs.data(), njobs * sizeof(BatchJob), cudaMemcpyHostToDevice, st));
    if (!sc.active.empty())
        CTX_TRY(cudaMemcpyAsync(bc.active, sc.active.data(), sc.active.size() * sizeof(uint32_t),
                                cudaMemcpyHostToDevice, st));

    // the schedule: the prime 2 of the jobs that include it, then per segment
    // the sieve and one batched launch
    auto enqueue = [&]() -> int {
        for (uint32_t i = 0; i < njobs; ++i)
            if (jobs[i].f0 <= 2 && jobs[i].f1 > 2) {
                int rc = launch_mod2(hjobs[i].view, st, err);
                if (rc)
                    return rc;
            }
        for (const Segment &g : sc.segs) {
            const uint64_t *d_count = nullptr;
            int rc = sieve_odd_async(ctx_workspace(ctx), g.lo, g.hi, bc.primes, bc.primes_cap, &d_count, st, err);
            if (!rc)
                rc = launch_batch(bc.jobs, bc.active + g.first, g.gcount, g.any_classified, bc.primes, d_count, g.lo,
                                  g.hi, bc.scratch(g.count), ctx_sm_count(ctx), st, err);
            if (rc)
                return rc;
        }
        return CTD_OK;
    };
    if (!use_graph) {
        int rc = enqueue();
        if (rc)
            return ctx_fail(ctx, rc, err);
    } else {
        // the key: every argument the captured launches take
        Hasher h;
        h.add(sieve_state_key(ctx_workspace(ctx)));
        h.add(ctx_sm_count(ctx));
        for (const void *p : {(const void *)bc.fb, (const void *)bc.jobs, (const void *)bc.active,
                              (const void *)bc.primes, (const void *)bc.spans, (const void *)bc.ctl,
                              (const void *)bc.codes, (const void *)bc.items, (const void *)bc.bucket})
            h.add(p);
        h.add(bc.primes_cap);
        h.add(bc.codes_cap);  // the pair lists sit in the items buffer at class_cap
        h.add(bc.items_cap);
        for (uint32_t i = 0; i < njobs; ++i)
            if (jobs[i].f0 <= 2 && jobs[i].f1 > 2)
                h.add(hjobs[i].view);
        for (const Segment &g : sc.segs) {
            h.add(g.lo);
            h.add(g.hi);
            h.add(g.first);
            h.add(g.count);
            h.add(g.gcount);
            h.add(g.any_classified);
        }
        if (!bc.exec || bc.key != h.h) {
            cudaGraph_t graph = nullptr;
            CTX_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            const uint64_t l0 = kernel_launch_count();
            int rc = enqueue();
            bc.graph_launches = kernel_launch_count() - l0;
            cudaError_t e = cudaStreamEndCapture(st, &graph);
            if (rc) {
                if (graph)
                    cudaGraphDestroy(graph);
                return ctx_fail(ctx, rc, err);
            }
            CTX_TRY(e);
            bool updated = false;
            if (bc.exec) {
                cudaGraphExecUpdateResultInfo info;
                updated = cudaGraphExecUpdate(bc.exec, graph, &info) == cudaSuccess;
                if (!updated) {
                    cudaGetLastError();  // clear the update's error
                    cudaGraphExecDestroy(bc.exec);
                    bc.exec = nullptr;
                }
            }
            if (!updated) {
                e = cudaGraphInstantiate(&bc.exec, graph, 0);
                if (e != cudaSuccess) {
                    cudaGraphDestroy(graph);
                    bc.exec = nullptr;
                    CTX_TRY(e);
                }
                ++bc.instantiations;
            } else {
                ++bc.updates;
            }
            cudaGraphDestroy(graph);
            bc.key = h.h;
        } else {
            ++bc.replays;
            note_kernel_launches(bc.graph_launches);  // the kernels the replay runs
        }
        CTX_TRY(cudaGraphLaunch(bc.exec, st));
    }
    for (uint32_t i = 0; i < njobs; ++i) {
        const ctd_job &j = jobs[i];
        const uint64_t N = j.n1 - j.n0;
        CTX_TRY(cudaMemcpyAsync(counts_inout[i], hjobs[i].view.fb.counts, N * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                st));
        CTX_TRY(cudaMemcpyAsync(factors_inout[i], hjobs[i].view.fb.factors, N * j.max_factors * sizeof(uint64_t),
                                cudaMemcpyDeviceToHost, st));
    }
    CTX_TRY(cudaStreamSynchronize(st));
    return CTD_OK;
}

int ctd_batch_graph_stats(ctd_ctx *ctx, uint64_t *instantiations, uint64_t *updates, uint64_t *replays)
{
    if (!ctx)
        return CTD_ERR_INVALID_ARGUMENT;
    const BatchCache *bc = ctx_batch_cache(ctx);
    if (instantiations)
        *instantiations = bc ? bc->instantiations : 0;
    if (updates)
        *updates = bc ? bc->updates : 0;
    if (replays)
        *replays = bc ? bc->replays : 0;
    return CTD_OK;
}

}  // extern "C"

// ------------------------------------------------------------ the server
//
// Slots: the device job table holds max_active entries; a job admitted into
// a slot keeps it until its results are collected.  Each tick advances every
// running job over one aligned segment of its prime range; the running jobs
// that are on the same segment share its sieve and its walk launches, and
// the kernels record each job's progress in its device cursor.  A job's
// result does not depend on the order of its segments, so an admitted job
// joins the segment that the most running jobs covering it are on and takes
// its remaining segments in rotated order (wrapping from its last segment to
// its first): jobs of overlapping ranges move in step and keep sharing
// sieves however far apart their arrivals were.  The host plans each tick
// from its own copy of the segment order, so it never reads the device
// between ticks.  At most TICKS_IN_FLIGHT ticks are queued ahead of the GPU.

struct ctd_server {
    ctd_ctx *ctx = nullptr;
    uint64_t seg = 0;
    uint64_t next_id = 1;
    struct Job {
        uint64_t id = 0;
        ctd_job job{};
        uint32_t slot = 0;
        uint32_t *d_counts = nullptr;
        uint64_t *d_factors = nullptr;
        // the job's aligned segments seg_first..seg_last, taken in rotated
        // order from next_seg; segs_left of them remain
        uint64_t seg_first = 0, seg_last = 0, next_seg = 0, segs_left = 0;
        bool finishing = false;
        cudaEvent_t done_event = nullptr;
        uint32_t *h_counts = nullptr;  // pinned, filled by the final copy
        uint64_t *h_factors = nullptr;
    };
    Admission<Job> adm;
    std::vector<Job> running;  // admitted, not yet collected
    std::vector<uint32_t> free_slots;
    std::map<uint64_t, Job> done;
    // device
    BatchJob *d_jobs = nullptr;
    uint32_t *d_active = nullptr;
    uint64_t *d_primes = nullptr;
    uint64_t primes_cap = 0;
    BatchSpan *d_spans = nullptr;
    BatchControl *d_ctl = nullptr;
    uint32_t *d_codes = nullptr;
    ClassItem *d_items = nullptr;
    uint64_t class_cap = 0;
    uint32_t *d_bucket = nullptr;
    BatchJob *h_stage = nullptr;   // pinned staging for slot descriptors
    uint32_t *h_active = nullptr;  // pinned active lists, one region per tick in flight
    std::deque<cudaEvent_t> inflight;
    uint64_t tick_count = 0;
    static constexpr int TICKS_IN_FLIGHT = 2;
};

namespace {

void free_job_host(ctd_server::Job &j)
{
    if (j.done_event)
        cudaEventDestroy(j.done_event);
    cudaFreeHost(j.h_counts);
    cudaFreeHost(j.h_factors);
    j.done_event = nullptr;
    j.h_counts = nullptr;
    j.h_factors = nullptr;
}

}  // namespace

extern "C" {

int ctd_serve_open(ctd_ctx *ctx, uint64_t memory_budget, uint32_t max_active, uint64_t segment_length,
                   ctd_server **out)
{
    if (!ctx || !out || !max_active || max_active > MAX_ACTIVE_PER_LAUNCH)
        return ctx ? ctx_fail(ctx, CTD_ERR_INVALID_ARGUMENT, "ctd_serve_open: bad arguments")
                   : CTD_ERR_INVALID_ARGUMENT;
    CTX_TRY(cudaSetDevice(ctx_device(ctx)));
    auto *srv = new (std::nothrow) ctd_server();
    if (!srv)
        return CTD_ERR_OUT_OF_MEMORY;
    srv->ctx = ctx;
    srv->adm.budget = memory_budget;
    srv->adm.max_active = max_active;
    srv->seg = segment_length ? segment_length : (1ull << 30);
    cudaError_t e = cudaMalloc(&srv->d_jobs, max_active * sizeof(BatchJob));
    if (e == cudaSuccess)
        e = cudaMalloc(&srv->d_active, (size_t)ctd_server::TICKS_IN_FLIGHT * max_active * sizeof(uint32_t));
    if (e == cudaSuccess)
        e = cudaMalloc(&srv->d_spans, (max_active + 1) * sizeof(BatchSpan));
    if (e == cudaSuccess)
        e = cudaMalloc(&srv->d_ctl, sizeof(BatchControl));
    if (e == cudaSuccess)
        e = cudaMalloc(&srv->d_bucket, 3ull * max_active * CLASS_BUCKETS * sizeof(uint32_t));
    if (e == cudaSuccess)
        e = cudaMallocHost(&srv->h_stage, max_active * sizeof(BatchJob));
    if (e == cudaSuccess)
        e = cudaMallocHost(&srv->h_active, (size_t)ctd_server::TICKS_IN_FLIGHT * max_active * sizeof(uint32_t));
    if (e != cudaSuccess) {
        ctd_serve_close(srv);
        return ctx_fail(ctx, e == cudaErrorMemoryAllocation ? CTD_ERR_OUT_OF_MEMORY : CTD_ERR_CUDA,
                        std::string("ctd_serve_open: ") + cudaGetErrorString(e));
    }
    for (uint32_t s = max_active; s-- > 0;)
        srv->free_slots.push_back(s);
    *out = srv;
    return CTD_OK;
}

void ctd_serve_close(ctd_server *srv)
{
    if (!srv)
        return;
    cudaSetDevice(ctx_device(srv->ctx));
    cudaStreamSynchronize(ctx_stream(srv->ctx));
    for (auto &j : srv->running) {
        cudaFree(j.d_counts);
        cudaFree(j.d_factors);
        free_job_host(j);
    }
    for (auto &kv : srv->done)
        free_job_host(kv.second);
    for (cudaEvent_t ev : srv->inflight)
        cudaEventDestroy(ev);
    cudaFree(srv->d_jobs);
    cudaFree(srv->d_active);
    cudaFree(srv->d_primes);
    cudaFree(srv->d_spans);
    cudaFree(srv->d_ctl);
    cudaFree(srv->d_codes);
    cudaFree(srv->d_items);
    cudaFree(srv->d_bucket);
    cudaFreeHost(srv->h_stage);
    cudaFreeHost(srv->h_active);
    delete srv;
}

int ctd_serve_submit(ctd_server *srv, const ctd_job *job, uint64_t *id)
{
    if (!srv || !job || !id)
        return CTD_ERR_INVALID_ARGUMENT;
    if (ctd_check_job(job) || job->f1 <= job->f0)
        return ctx_fail(srv->ctx, CTD_ERR_INVALID_ARGUMENT, "ctd_serve_submit: invalid job");
    ctd_server::Job j;
    j.id = srv->next_id++;
    j.job = *job;
    srv->adm.queue.push_back(j);
    *id = j.id;
    return CTD_OK;
}

int ctd_serve_status(ctd_server *srv, uint32_t *active, uint32_t *queued, uint64_t *memory_used)
{
    if (!srv)
        return CTD_ERR_INVALID_ARGUMENT;
    if (active)
        *active = srv->adm.active;
    if (queued)
        *queued = (uint32_t)srv->adm.queue.size();
    if (memory_used)
        *memory_used = srv->adm.used;
    return CTD_OK;
}

int ctd_serve_tick(ctd_server *srv, uint64_t *done_ids, uint32_t cap, uint32_t *ndone)
{
    if (!srv || !ndone || (cap && !done_ids))
        return CTD_ERR_INVALID_ARGUMENT;
    ctd_ctx *ctx = srv->ctx;
    *ndone = 0;
    CTX_TRY(cudaSetDevice(ctx_device(ctx)));
    cudaStream_t st = ctx_stream(ctx);
    std::string err;
    const uint64_t S = srv->seg;

    // 1. collect finished jobs whose results have arrived on the host
    for (size_t k = 0; k < srv->running.size();) {
        ctd_server::Job &j = srv->running[k];
        if (j.finishing && cudaEventQuery(j.done_event) == cudaSuccess) {
            srv->adm.release(job_bytes(j.job));
            srv->free_slots.push_back(j.slot);
            if (*ndone < cap)
                done_ids[*ndone] = j.id;
            ++*ndone;
            srv->done[j.id] = j;
            srv->running.erase(srv->running.begin() + (long)k);
        } else {
            ++k;
        }
    }
    cudaGetLastError();  // cudaEventQuery's "not ready" is not an error

    // 2. admission: slots and the memory budget, arrival order
    std::vector<ctd_server::Job> admitted;
    int arc = srv->adm.admit(
        [](const ctd_server::Job &j) { return job_bytes(j.job); },
        [&](ctd_server::Job &j, uint64_t) -> int {
            const uint64_t N = j.job.n1 - j.job.n0;
            cudaError_t e = cudaMallocAsync(&j.d_counts, N * sizeof(uint32_t), st);
            if (e == cudaSuccess)
                e = cudaMallocAsync(&j.d_factors, N * j.job.max_factors * sizeof(uint64_t), st);
            if (e != cudaSuccess) {
                if (j.d_counts)
                    cudaFreeAsync(j.d_counts, st);
                j.d_counts = nullptr;
                j.d_factors = nullptr;
                cudaGetLastError();
                err = std::string("job buffers: ") + cudaGetErrorString(e);
                return CTD_ERR_OUT_OF_MEMORY;
            }
            return CTD_OK;
        },
        [&](ctd_server::Job &j) { admitted.push_back(j); });
    for (ctd_server::Job &j : admitted) {
        const uint64_t N = j.job.n1 - j.job.n0;
        j.slot = srv->free_slots.back();
        srv->free_slots.pop_back();
        CTX_TRY(cudaMemsetAsync(j.d_counts, 0, N * sizeof(uint32_t), st));
        CTX_TRY(cudaMemsetAsync(j.d_factors, 0, N * j.job.max_factors * sizeof(uint64_t), st));
        BatchJob b = batch_job_of(ctx, j.job, j.d_counts, j.d_factors);
        if (j.job.f0 <= 2 && j.job.f1 > 2) {
            int rc = launch_mod2(b.view, st, err);
            if (rc)
                return ctx_fail(ctx, rc, err);
        }
        // segments: start where most running jobs covering this one are
        j.seg_first = b.f0 / srv->seg;
        j.seg_last = (b.f1 - 1) / srv->seg;
        j.segs_left = b.f0 < b.f1 ? j.seg_last - j.seg_first + 1 : 0;
        j.next_seg = j.seg_first;
        {
            std::map<uint64_t, uint32_t> votes;
            for (const ctd_server::Job &r : srv->running)
                if (r.segs_left && r.next_seg >= j.seg_first && r.next_seg <= j.seg_last)
                    ++votes[r.next_seg];
            uint32_t best = 0;
            for (auto &kv : votes)
                if (kv.second > best) {
                    best = kv.second;
                    j.next_seg = kv.first;
                }
        }
        srv->h_stage[j.slot] = b;
        CTX_TRY(cudaMemcpyAsync(srv->d_jobs + j.slot, srv->h_stage + j.slot, sizeof(BatchJob), cudaMemcpyHostToDevice,
                                st));
        srv->running.push_back(j);
    }
    if (arc && srv->running.empty())
        return ctx_fail(ctx, arc, err);  // nothing runs and the first queued job cannot be placed

    // 3. one tick: every running job advances over its next segment
    std::map<uint64_t, std::vector<uint32_t>> byseg;  // segment index -> running indices
    for (uint32_t k = 0; k < srv->running.size(); ++k) {
        const ctd_server::Job &j = srv->running[k];
        if (!j.finishing && j.segs_left)
            byseg[j.next_seg].push_back(k);
    }
    // a job's part of segment k: [max(f0, k S), min(f1, (k + 1) S))
    auto part_lo = [&](const ctd_server::Job &j, uint64_t k) { return std::max(srv->h_stage[j.slot].f0, k * S); };
    auto part_hi = [&](const ctd_server::Job &j, uint64_t k) {
        return k + 1 > ~0ull / S ? j.job.f1 : std::min(j.job.f1, (k + 1) * S);
    };
    if (!byseg.empty()) {
        // bounded lead over the GPU: wait for the tick before last
        while ((int)srv->inflight.size() >= ctd_server::TICKS_IN_FLIGHT) {
            CTX_TRY(cudaEventSynchronize(srv->inflight.front()));
            cudaEventDestroy(srv->inflight.front());
            srv->inflight.pop_front();
        }
        uint64_t primes_need = 0, class_need = 0, maxhi = 0;
        for (auto &kv : byseg) {
            const uint64_t slo = kv.first * S;
            primes_need = std::max(primes_need, prime_count_upper_bound(slo, slo + S));
            uint64_t ncls = 0;
            for (uint32_t k : kv.second) {
                const ctd_server::Job &j = srv->running[k];
                maxhi = std::max(maxhi, j.job.f1);
                if (srv->h_stage[j.slot].classified)
                    ncls += prime_count_upper_bound(part_lo(j, kv.first), part_hi(j, kv.first));
            }
            class_need = std::max(class_need, ncls);
        }
        if (primes_need > srv->primes_cap || class_need > srv->class_cap) {
            // regrow between ticks: everything queued so far must finish first
            CTX_TRY(cudaStreamSynchronize(st));
            if (primes_need > srv->primes_cap) {
                cudaFree(srv->d_primes);
                srv->d_primes = nullptr;
                srv->primes_cap = 0;
                CTX_TRY(cudaMalloc(&srv->d_primes, primes_need * sizeof(uint64_t)));
                srv->primes_cap = primes_need;
            }
            if (class_need > srv->class_cap) {
                cudaFree(srv->d_codes);
                cudaFree(srv->d_items);
                srv->d_codes = nullptr;
                srv->d_items = nullptr;
                srv->class_cap = 0;
                CTX_TRY(cudaMalloc(&srv->d_codes, class_need * sizeof(uint32_t)));
                CTX_TRY(cudaMalloc(&srv->d_items, class_need * sizeof(ClassItem)));
                srv->class_cap = class_need;
            }
        }
        int rc = sieve_prepare_base(ctx_workspace(ctx), maxhi, st, err);
        if (!rc)
            rc = sieve_prepare_windows(ctx_workspace(ctx), S, err);
        if (rc)
            return ctx_fail(ctx, rc, err);
        // this tick's active lists (slot numbers), in its own staging region
        const uint32_t region = (uint32_t)(srv->tick_count % ctd_server::TICKS_IN_FLIGHT) * srv->adm.max_active;
        uint32_t *h_act = srv->h_active + region;
        uint32_t *d_act = srv->d_active + region;
        uint32_t used = 0;
        for (auto &kv : byseg) {
            uint64_t lo = ~0ull, hi = 0;
            bool any_cls = false;
            const uint32_t first = used;
            std::vector<uint32_t> ks = kv.second;
            uint32_t gcount[BATCH_GROUPS];
            order_active(
                ks, gcount, [&](uint32_t x) { return srv->running[x].job.n1 - srv->running[x].job.n0; },
                [&](uint32_t x) { return srv->running[x].job.family; },
                [&](uint32_t x) {
                    const ctd_server::Job &j = srv->running[x];
                    return batch_group(j.job.family, srv->h_stage[j.slot].classified != 0);
                });
            for (uint32_t k : ks) {
                ctd_server::Job &j = srv->running[k];
                lo = std::min(lo, part_lo(j, kv.first));
                hi = std::max(hi, part_hi(j, kv.first));
                any_cls |= srv->h_stage[j.slot].classified != 0;
                h_act[used++] = j.slot;
                --j.segs_left;
                j.next_seg = j.next_seg == j.seg_last ? j.seg_first : j.next_seg + 1;
            }
            CTX_TRY(cudaMemcpyAsync(d_act + first, h_act + first, (used - first) * sizeof(uint32_t),
                                    cudaMemcpyHostToDevice, st));
            const uint64_t *d_count = nullptr;
            rc = sieve_odd_async(ctx_workspace(ctx), lo, hi, srv->d_primes, srv->primes_cap, &d_count, st, err);
            if (!rc) {
                BatchScratch bs;
                bs.spans = srv->d_spans;
                bs.ctl = srv->d_ctl;
                bs.codes = srv->d_codes;
                bs.items = srv->d_items;
                bs.class_cap = srv->class_cap;
                bs.bucket_count = srv->d_bucket;
                bs.bucket_base = srv->d_bucket + 2ull * (used - first) * CLASS_BUCKETS;
                rc = launch_batch(srv->d_jobs, d_act + first, gcount, any_cls, srv->d_primes, d_count, lo, hi,
                                  bs, ctx_sm_count(ctx), st, err);
            }
            if (rc)
                return ctx_fail(ctx, rc, err);
        }
        // jobs that reached the end of their range: results to the host
        for (ctd_server::Job &j : srv->running) {
            if (j.finishing || j.segs_left)
                continue;
            const uint64_t N = j.job.n1 - j.job.n0;
            CTX_TRY(cudaMallocHost(&j.h_counts, N * sizeof(uint32_t)));
            CTX_TRY(cudaMallocHost(&j.h_factors, N * j.job.max_factors * sizeof(uint64_t)));
            CTX_TRY(cudaMemcpyAsync(j.h_counts, j.d_counts, N * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
            CTX_TRY(cudaMemcpyAsync(j.h_factors, j.d_factors, N * j.job.max_factors * sizeof(uint64_t),
                                    cudaMemcpyDeviceToHost, st));
            CTX_TRY(cudaFreeAsync(j.d_counts, st));
            CTX_TRY(cudaFreeAsync(j.d_factors, st));
            j.d_counts = nullptr;
            j.d_factors = nullptr;
            CTX_TRY(cudaEventCreateWithFlags(&j.done_event, cudaEventDisableTiming));
            CTX_TRY(cudaEventRecord(j.done_event, st));
            j.finishing = true;
        }
        cudaEvent_t ev;
        CTX_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        CTX_TRY(cudaEventRecord(ev, st));
        srv->inflight.push_back(ev);
        ++srv->tick_count;
    } else if (!srv->running.empty()) {
        // nothing left to queue: wait for the oldest finishing job
        for (ctd_server::Job &j : srv->running)
            if (j.finishing) {
                CTX_TRY(cudaEventSynchronize(j.done_event));
                break;
            }
    }
    return CTD_OK;
}

int ctd_serve_fetch(ctd_server *srv, uint64_t id, uint32_t *counts, uint64_t *factors)
{
    if (!srv || !counts || !factors)
        return CTD_ERR_INVALID_ARGUMENT;
    auto it = srv->done.find(id);
    if (it == srv->done.end())
        return ctx_fail(srv->ctx, CTD_ERR_NOT_FOUND, "ctd_serve_fetch: job not finished or unknown");
    ctd_server::Job &j = it->second;
    const uint64_t N = j.job.n1 - j.job.n0;
    std::memcpy(counts, j.h_counts, N * sizeof(uint32_t));
    std::memcpy(factors, j.h_factors, N * j.job.max_factors * sizeof(uint64_t));
    free_job_host(j);
    srv->done.erase(it);
    return CTD_OK;
}

}  // extern "C"
