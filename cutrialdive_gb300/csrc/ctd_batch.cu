// ctd_batch.cu -- many jobs at once: the batched runner and the server.
//
// The reference runs one job per process (src/main.cpp:94-146) and one
// kernel launch per sieve segment (src/trial_factoring.cuh:437-488); it has
// no batching or serving layer.  Here:
//
// * ctd_batch_run walks the union of the jobs' prime ranges segment by
//   segment ("chunk-major"): each 2^k-aligned segment is sieved once and
//   consumed by every job whose range covers it, with one batched residue
//   launch per family present.  The whole schedule -- sieve, bounds and
//   residue kernels of every segment -- is captured once into a CUDA graph
//   and launched once; nothing waits on the host until the end.
// * ctd_serve_* keeps a set of active jobs with per-job prime cursors on the
//   device and advances all of them by one aligned segment per tick; jobs
//   submitted while others run are admitted at the next tick as slots and
//   the device-memory budget allow (continuous batching).
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

JobView view_of(ctd_ctx *ctx, const ctd_job &j, uint32_t *counts, uint64_t *factors)
{
    JobView v{};
    v.family = j.family;
    v.tiles = 1;
    ctd_tuning t{};
    v.variant = ctd_get_tuning(ctx, j.family, &t) == CTD_OK ? t.variant : CTD_VARIANT_AUTO;
    v.param = j.param;
    v.n0 = j.n0;
    v.n1 = j.n1;
    v.tile_len = j.n1 - j.n0;
    v.fb.counts = counts;
    v.fb.factors = factors;
    v.fb.max_factors = j.max_factors;
    return v;
}

// odd-prime range of a job after the prime 2 is handled separately
uint64_t odd_f0(const ctd_job &j) { return j.f0 <= 2 ? 3 : j.f0; }

struct Launch {  // one batched launch of a segment
    uint32_t family;
    uint32_t first;  // offset into the active-list array
    uint32_t count;
};

struct Segment {
    uint64_t lo, hi;
    std::vector<Launch> launches;
};

int grid_for_family(ctd_ctx *ctx, uint32_t family)
{
    int per_sm = batch_blocks_per_sm(family);
    return ctx_sm_count(ctx) * (per_sm > 0 ? per_sm : 1);
}

}  // namespace

struct ctd_server {
    ctd_ctx *ctx = nullptr;
    uint64_t budget = 0;
    uint64_t used = 0;
    uint32_t max_active = 0;
    uint64_t seg = 0;
    uint64_t next_id = 1;
    struct Job {
        uint64_t id;
        ctd_job job;
        uint32_t *d_counts = nullptr;
        uint64_t *d_factors = nullptr;
        uint64_t cursor = 0;  // next prime bound to process
        std::chrono::steady_clock::time_point submitted;
    };
    std::deque<Job> queue;           // submitted, not admitted
    std::vector<Job> active;
    std::map<uint64_t, std::pair<std::vector<uint32_t>, std::vector<uint64_t>>> done;
    // device scratch
    uint64_t *d_primes = nullptr;
    uint64_t primes_cap = 0;
    BatchJob *d_jobs = nullptr;
    uint32_t *d_active = nullptr;
    BatchSpan *d_spans = nullptr;
    uint32_t cap_jobs = 0;
};

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
    int rc = CTD_OK;

    // device factors buffers, one allocation
    std::vector<uint64_t> off(njobs + 1, 0);
    for (uint32_t i = 0; i < njobs; ++i)
        off[i + 1] = off[i] + job_bytes(jobs[i]);
    unsigned char *d_buf = nullptr;
    BatchJob *d_jobs = nullptr;
    uint32_t *d_active = nullptr;
    BatchSpan *d_spans = nullptr;
    uint64_t *d_primes = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<BatchJob> hjobs(njobs);
    std::vector<Segment> segs;
    std::vector<uint32_t> hactive;
    uint64_t lo = ~0ull, hi = 0, primes_cap = 0;
    uint32_t max_launch = 1;

    auto cleanup = [&]() {
        if (exec)
            cudaGraphExecDestroy(exec);
        if (graph)
            cudaGraphDestroy(graph);
        cudaFree(d_buf);
        cudaFree(d_jobs);
        cudaFree(d_active);
        cudaFree(d_spans);
        cudaFree(d_primes);
    };
#define BATCH_TRY(expr)                                                                                   \
    do {                                                                                                  \
        cudaError_t e_ = (expr);                                                                          \
        if (e_ != cudaSuccess) {                                                                          \
            cleanup();                                                                                    \
            return ctx_fail(ctx, e_ == cudaErrorMemoryAllocation ? CTD_ERR_OUT_OF_MEMORY : CTD_ERR_CUDA, \
                            std::string(#expr ": ") + cudaGetErrorString(e_));                            \
        }                                                                                                 \
    } while (0)

    BATCH_TRY(cudaMalloc(&d_buf, off[njobs]));
    for (uint32_t i = 0; i < njobs; ++i) {
        const ctd_job &j = jobs[i];
        const uint64_t N = j.n1 - j.n0;
        auto *dc = reinterpret_cast<uint32_t *>(d_buf + off[i]);
        auto *df = reinterpret_cast<uint64_t *>(d_buf + off[i] + counts_bytes(j));
        BATCH_TRY(cudaMemcpyAsync(dc, counts_inout[i], N * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
        BATCH_TRY(cudaMemcpyAsync(df, factors_inout[i], N * j.max_factors * sizeof(uint64_t),
                                  cudaMemcpyHostToDevice, st));
        hjobs[i].view = view_of(ctx, j, dc, df);
        hjobs[i].f0 = odd_f0(j);
        hjobs[i].f1 = j.f1;
        if (j.f0 <= 2 && j.f1 > 2) {  // the prime 2 for this job
            rc = launch_mod2(hjobs[i].view, st, err);
            if (rc) {
                cleanup();
                return ctx_fail(ctx, rc, err);
            }
        }
        if (hjobs[i].f0 < hjobs[i].f1) {
            lo = std::min(lo, hjobs[i].f0);
            hi = std::max(hi, hjobs[i].f1);
        }
    }
    BATCH_TRY(cudaMalloc(&d_jobs, njobs * sizeof(BatchJob)));
    BATCH_TRY(cudaMemcpyAsync(d_jobs, hjobs.data(), njobs * sizeof(BatchJob), cudaMemcpyHostToDevice, st));

    // chunk-major schedule over aligned segments
    if (lo < hi) {
        for (uint64_t k = lo / S; k * S < hi && k <= (~0ull / S); ++k) {
            Segment sg;
            sg.lo = std::max(k * S, lo);
            sg.hi = (k + 1 > ~0ull / S) ? hi : std::min((k + 1) * S, hi);
            std::map<uint32_t, std::vector<uint32_t>> byfam;
            for (uint32_t i = 0; i < njobs; ++i)
                if (hjobs[i].f0 < sg.hi && hjobs[i].f1 > sg.lo)
                    byfam[jobs[i].family].push_back(i);
            if (byfam.empty())
                continue;
            for (auto &kv : byfam) {
                // longest index range first (the kernel hands out items in this order)
                std::stable_sort(kv.second.begin(), kv.second.end(), [&](uint32_t x, uint32_t y) {
                    return jobs[x].n1 - jobs[x].n0 > jobs[y].n1 - jobs[y].n0;
                });
                for (size_t b = 0; b < kv.second.size(); b += MAX_ACTIVE_PER_LAUNCH) {
                    Launch l;
                    l.family = kv.first;
                    l.first = (uint32_t)hactive.size();
                    l.count = (uint32_t)std::min<size_t>(MAX_ACTIVE_PER_LAUNCH, kv.second.size() - b);
                    hactive.insert(hactive.end(), kv.second.begin() + b, kv.second.begin() + b + l.count);
                    max_launch = std::max(max_launch, l.count);
                    sg.launches.push_back(l);
                }
            }
            primes_cap = std::max(primes_cap, prime_count_upper_bound(sg.lo, sg.hi));
            segs.push_back(std::move(sg));
        }
    }
    if (!segs.empty()) {
        BATCH_TRY(cudaMalloc(&d_active, hactive.size() * sizeof(uint32_t)));
        BATCH_TRY(cudaMemcpyAsync(d_active, hactive.data(), hactive.size() * sizeof(uint32_t),
                                  cudaMemcpyHostToDevice, st));
        BATCH_TRY(cudaMalloc(&d_spans, (max_launch + 1) * sizeof(BatchSpan)));
        BATCH_TRY(cudaMalloc(&d_primes, primes_cap * sizeof(uint64_t)));
        rc = sieve_prepare_base(ctx_workspace(ctx), hi, st, err);
        if (!rc)
            rc = sieve_prepare_windows(ctx_workspace(ctx), S, err);
        if (rc) {
            cleanup();
            return ctx_fail(ctx, rc, err);
        }
        BATCH_TRY(cudaStreamSynchronize(st));
        std::vector<int> grids(CTD_PEANO + 1, 0);
        for (auto &sg : segs)
            for (auto &l : sg.launches)
                if (!grids[l.family])
                    grids[l.family] = grid_for_family(ctx, l.family);
        if (use_graph)
            BATCH_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        for (auto &sg : segs) {
            const uint64_t *d_count = nullptr;
            rc = sieve_odd_async(ctx_workspace(ctx), sg.lo, sg.hi, d_primes, primes_cap, &d_count, st, err);
            for (size_t li = 0; !rc && li < sg.launches.size(); ++li) {
                const Launch &l = sg.launches[li];
                rc = launch_batch(l.family, d_jobs, d_active + l.first, l.count, d_primes, d_count, sg.lo, sg.hi,
                                  d_spans, grids[l.family], st, err);
            }
            if (rc)
                break;
        }
        if (use_graph) {
            cudaError_t e = cudaStreamEndCapture(st, &graph);
            if (rc) {
                cleanup();
                return ctx_fail(ctx, rc, err);
            }
            BATCH_TRY(e);
            BATCH_TRY(cudaGraphInstantiate(&exec, graph, 0));
            BATCH_TRY(cudaGraphLaunch(exec, st));
        } else if (rc) {
            cleanup();
            return ctx_fail(ctx, rc, err);
        }
    }
    for (uint32_t i = 0; i < njobs; ++i) {
        const ctd_job &j = jobs[i];
        const uint64_t N = j.n1 - j.n0;
        BATCH_TRY(cudaMemcpyAsync(counts_inout[i], hjobs[i].view.fb.counts, N * sizeof(uint32_t),
                                  cudaMemcpyDeviceToHost, st));
        BATCH_TRY(cudaMemcpyAsync(factors_inout[i], hjobs[i].view.fb.factors, N * j.max_factors * sizeof(uint64_t),
                                  cudaMemcpyDeviceToHost, st));
    }
    BATCH_TRY(cudaStreamSynchronize(st));
    cleanup();
#undef BATCH_TRY
    return CTD_OK;
}

// ------------------------------------------------------------ the server

int ctd_serve_open(ctd_ctx *ctx, uint64_t memory_budget, uint32_t max_active, uint64_t segment_length,
                   ctd_server **out)
{
    if (!ctx || !out || !max_active)
        return ctx ? ctx_fail(ctx, CTD_ERR_INVALID_ARGUMENT, "ctd_serve_open: bad arguments")
                   : CTD_ERR_INVALID_ARGUMENT;
    auto *srv = new (std::nothrow) ctd_server();
    if (!srv)
        return CTD_ERR_OUT_OF_MEMORY;
    srv->ctx = ctx;
    srv->budget = memory_budget;
    srv->max_active = max_active;
    srv->seg = segment_length ? segment_length : (1ull << 30);
    *out = srv;
    return CTD_OK;
}

void ctd_serve_close(ctd_server *srv)
{
    if (!srv)
        return;
    cudaSetDevice(ctx_device(srv->ctx));
    cudaStreamSynchronize(ctx_stream(srv->ctx));
    for (auto &j : srv->active) {
        cudaFree(j.d_counts);
        cudaFree(j.d_factors);
    }
    cudaFree(srv->d_primes);
    cudaFree(srv->d_jobs);
    cudaFree(srv->d_active);
    cudaFree(srv->d_spans);
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
    j.submitted = std::chrono::steady_clock::now();
    srv->queue.push_back(j);
    *id = j.id;
    return CTD_OK;
}

int ctd_serve_status(ctd_server *srv, uint32_t *active, uint32_t *queued, uint64_t *memory_used)
{
    if (!srv)
        return CTD_ERR_INVALID_ARGUMENT;
    if (active)
        *active = (uint32_t)srv->active.size();
    if (queued)
        *queued = (uint32_t)srv->queue.size();
    if (memory_used)
        *memory_used = srv->used;
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
    // admission: slots and the memory budget, in arrival order
    while (!srv->queue.empty() && srv->active.size() < srv->max_active) {
        ctd_server::Job &q = srv->queue.front();
        const uint64_t bytes = job_bytes(q.job);
        if (srv->used + bytes > srv->budget && !srv->active.empty())
            break;
        const uint64_t N = q.job.n1 - q.job.n0;
        CTX_TRY(cudaMallocAsync(&q.d_counts, N * sizeof(uint32_t), st));
        CTX_TRY(cudaMallocAsync(&q.d_factors, N * q.job.max_factors * sizeof(uint64_t), st));
        CTX_TRY(cudaMemsetAsync(q.d_counts, 0, N * sizeof(uint32_t), st));
        CTX_TRY(cudaMemsetAsync(q.d_factors, 0, N * q.job.max_factors * sizeof(uint64_t), st));
        if (q.job.f0 <= 2 && q.job.f1 > 2) {
            int rc = launch_mod2(view_of(ctx, q.job, q.d_counts, q.d_factors), st, err);
            if (rc)
                return ctx_fail(ctx, rc, err);
        }
        q.cursor = odd_f0(q.job);
        srv->used += bytes;
        srv->active.push_back(q);
        srv->queue.pop_front();
    }
    if (srv->active.empty())
        return CTD_OK;
    // every active job advances over its current aligned segment; jobs on the
    // same segment share its sieve
    const uint64_t S = srv->seg;
    std::map<uint64_t, std::vector<uint32_t>> byseg;
    for (uint32_t i = 0; i < srv->active.size(); ++i) {
        auto &j = srv->active[i];
        if (j.cursor < j.job.f1)
            byseg[j.cursor / S].push_back(i);
    }
    const uint32_t na = (uint32_t)srv->active.size();
    if (na > srv->cap_jobs) {
        cudaFree(srv->d_jobs);
        cudaFree(srv->d_active);
        cudaFree(srv->d_spans);
        srv->d_jobs = nullptr;
        srv->d_active = nullptr;
        srv->d_spans = nullptr;
        srv->cap_jobs = 0;
        CTX_TRY(cudaMalloc(&srv->d_jobs, na * sizeof(BatchJob)));
        CTX_TRY(cudaMalloc(&srv->d_active, na * sizeof(uint32_t)));
        CTX_TRY(cudaMalloc(&srv->d_spans, (na + 1) * sizeof(BatchSpan)));
        srv->cap_jobs = na;
    }
    std::vector<BatchJob> hj(na);
    for (uint32_t i = 0; i < na; ++i) {
        auto &j = srv->active[i];
        hj[i].view = view_of(ctx, j.job, j.d_counts, j.d_factors);
        hj[i].f0 = odd_f0(j.job);
        hj[i].f1 = j.job.f1;
    }
    CTX_TRY(cudaMemcpyAsync(srv->d_jobs, hj.data(), na * sizeof(BatchJob), cudaMemcpyHostToDevice, st));
    // capacity for the primes of the largest segment group of this tick
    uint64_t primes_need = 0;
    for (auto &kv : byseg) {
        const uint64_t slo = kv.first * S;
        primes_need = std::max(primes_need, prime_count_upper_bound(slo, slo + S));
    }
    if (primes_need > srv->primes_cap) {
        cudaFree(srv->d_primes);
        srv->d_primes = nullptr;
        srv->primes_cap = 0;
        CTX_TRY(cudaMalloc(&srv->d_primes, primes_need * sizeof(uint64_t)));
        srv->primes_cap = primes_need;
    }
    uint64_t maxhi = 0;
    for (auto &j : srv->active)
        maxhi = std::max(maxhi, j.job.f1);
    int rc = sieve_prepare_base(ctx_workspace(ctx), maxhi, st, err);
    if (!rc)
        rc = sieve_prepare_windows(ctx_workspace(ctx), S, err);
    if (rc)
        return ctx_fail(ctx, rc, err);
    std::vector<uint32_t> order;  // active indices grouped by segment then family
    struct L { uint64_t lo, hi; uint32_t family, first, count; };
    std::vector<L> launches;
    for (auto &kv : byseg) {
        uint64_t lo = ~0ull, hi = 0;
        std::map<uint32_t, std::vector<uint32_t>> byfam;
        for (uint32_t i : kv.second) {
            auto &j = srv->active[i];
            lo = std::min(lo, j.cursor);
            hi = std::max(hi, std::min(j.job.f1, (kv.first + 1) * S));
            byfam[j.job.family].push_back(i);
        }
        for (auto &f : byfam) {
            // longest index range first (the kernel hands out items in this order)
            std::stable_sort(f.second.begin(), f.second.end(), [&](uint32_t x, uint32_t y) {
                const ctd_job &a = srv->active[x].job, &c = srv->active[y].job;
                return a.n1 - a.n0 > c.n1 - c.n0;
            });
            launches.push_back({lo, hi, f.first, (uint32_t)order.size(), (uint32_t)f.second.size()});
            order.insert(order.end(), f.second.begin(), f.second.end());
        }
    }
    CTX_TRY(cudaMemcpyAsync(srv->d_active, order.data(), order.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    // the launches of one segment follow its sieve; launches are grouped by segment
    uint64_t cur_lo = ~0ull, cur_hi = 0;
    const uint64_t *d_count = nullptr;
    for (auto &l : launches) {
        if (l.lo != cur_lo || l.hi != cur_hi) {
            rc = sieve_odd_async(ctx_workspace(ctx), l.lo, l.hi, srv->d_primes, srv->primes_cap, &d_count, st, err);
            if (rc)
                return ctx_fail(ctx, rc, err);
            cur_lo = l.lo;
            cur_hi = l.hi;
        }
        rc = launch_batch(l.family, srv->d_jobs, srv->d_active + l.first, l.count, srv->d_primes, d_count, l.lo, l.hi,
                          srv->d_spans, grid_for_family(ctx, l.family), st, err);
        if (rc)
            return ctx_fail(ctx, rc, err);
    }
    // advance cursors; finished jobs hand their results back to the host
    std::vector<ctd_server::Job> still;
    for (auto &j : srv->active) {
        const uint64_t seg_end = (j.cursor / S + 1) * S;
        const uint64_t upto = std::min(j.job.f1, seg_end);
        j.cursor = upto;
        if (j.cursor >= j.job.f1) {
            const uint64_t N = j.job.n1 - j.job.n0;
            auto &res = srv->done[j.id];
            res.first.resize(N);
            res.second.resize(N * j.job.max_factors);
            CTX_TRY(cudaMemcpyAsync(res.first.data(), j.d_counts, N * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
            CTX_TRY(cudaMemcpyAsync(res.second.data(), j.d_factors, N * j.job.max_factors * sizeof(uint64_t),
                                    cudaMemcpyDeviceToHost, st));
            CTX_TRY(cudaFreeAsync(j.d_counts, st));
            CTX_TRY(cudaFreeAsync(j.d_factors, st));
            srv->used -= job_bytes(j.job);
            if (*ndone < cap)
                done_ids[*ndone] = j.id;
            ++*ndone;
        } else {
            still.push_back(j);
        }
    }
    CTX_TRY(cudaStreamSynchronize(st));
    srv->active.swap(still);
    return CTD_OK;
}

int ctd_serve_fetch(ctd_server *srv, uint64_t id, uint32_t *counts, uint64_t *factors)
{
    if (!srv || !counts || !factors)
        return CTD_ERR_INVALID_ARGUMENT;
    auto it = srv->done.find(id);
    if (it == srv->done.end())
        return ctx_fail(srv->ctx, CTD_ERR_NOT_FOUND, "ctd_serve_fetch: job not finished or unknown");
    std::memcpy(counts, it->second.first.data(), it->second.first.size() * sizeof(uint32_t));
    std::memcpy(factors, it->second.second.data(), it->second.second.size() * sizeof(uint64_t));
    srv->done.erase(it);
    return CTD_OK;
}

}  // extern "C"
