// ctd_engine.cu -- the C ABI of libctd_gpu.so (include/ctd_gpu.h).
//
// A context owns one device, one stream, the sieve workspace and the
// device buffers of the job in flight.  ctd_run_plain is the device-side
// replacement of device_trial_factor (src/trial_factoring.cuh:334-513):
// the prime 2 first, then for each segment [fx, fy) of the prime range the
// device sieve writes the segment's primes into HBM and the family's
// residue kernel consumes them; the factors buffer stays on the device
// until the end (or a snapshot the caller asks for).
#include "ctd_internal.h"

#include <chrono>
#include <cstring>
#include <new>
#include <string>

using namespace ctd;

struct ctd_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    SieveWorkspace *ws = nullptr;
    std::string last_error;
    int grid_override = 0;
    int block_override = 0;
    int sm_count = 1;
    char name[256] = {0};
    uint64_t total_mem = 0;
    // device buffers reused across calls
    uint64_t *d_primes = nullptr;
    size_t primes_cap = 0;
    uint32_t *d_counts = nullptr;
    size_t counts_cap = 0;
    uint64_t *d_factors = nullptr;
    size_t factors_cap = 0;
};

namespace {

int fail(ctd_ctx *ctx, int code, const std::string &msg)
{
    if (ctx)
        ctx->last_error = msg;
    return code;
}

int cuda_fail(ctd_ctx *ctx, cudaError_t e, const char *what)
{
    return fail(ctx, e == cudaErrorMemoryAllocation ? CTD_ERR_OUT_OF_MEMORY : CTD_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}

#define CTX_CUDA(expr)                                 \
    do {                                               \
        cudaError_t e_ = (expr);                       \
        if (e_ != cudaSuccess)                         \
            return cuda_fail(ctx, e_, #expr);          \
    } while (0)

template <class T>
int ensure_buffer(ctd_ctx *ctx, T *&ptr, size_t &cap, size_t n)
{
    if (n <= cap && ptr)
        return CTD_OK;
    cudaFree(ptr);
    ptr = nullptr;
    cap = 0;
    cudaError_t e = cudaMalloc(&ptr, (n ? n : 1) * sizeof(T));
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "cudaMalloc");
    cap = n;
    return CTD_OK;
}

bool job_ok(const ctd_job *job)
{
    if (!job)
        return false;
    switch (job->family) {
    case CTD_MERSENNE:
    case CTD_FIBONACCI:
    case CTD_LUCAS:
    case CTD_TRIBONACCI:
    case CTD_PEANO: break;
    case CTD_PROTH:
    case CTD_RIESEL:
    case CTD_PROTH_FIXED_N:
    case CTD_RIESEL_FIXED_N:
        if (!job->param)
            return false;
        break;
    case CTD_SMARANDACHE:
        if (job->param < 2 || job->param > 64)
            return false;
        break;
    default: return false;
    }
    if (job->n1 <= job->n0 || job->max_factors == 0)
        return false;
    // counts and factors of the whole index range must be addressable
    const uint64_t N = job->n1 - job->n0;
    if (N > (1ull << 40) / job->max_factors)
        return false;
    return true;
}

int default_block(const ctd_ctx *ctx) { return ctx->block_override > 0 ? ctx->block_override : 256; }

int default_grid(ctd_ctx *ctx, uint32_t family, int block)
{
    if (ctx->grid_override > 0)
        return ctx->grid_override;
    // persistent grid: exactly the CTAs that are resident at once, so every
    // thread strides over the same number of work items and no CTA waits
    // for a second wave
    int per_sm = residue_blocks_per_sm(family, block);
    if (per_sm < 1)
        per_sm = 1;
    return ctx->sm_count * per_sm;
}

// index tiles per prime so that short prime lists still fill the GPU,
// keeping each tile long enough to amortize its jump
void choose_tiles(const ctd_ctx *ctx, uint64_t nprimes, uint64_t N, int grid, int block, uint32_t &tiles,
                  uint64_t &tile_len)
{
    tiles = 1;
    tile_len = N;
    const uint64_t threads = (uint64_t)grid * block;
    const uint64_t want = 8 * threads;
    if (nprimes >= want || N < 2 * 4096)
        return;
    uint64_t t = (want + nprimes - 1) / (nprimes ? nprimes : 1);
    uint64_t tmax = N / 4096;
    if (t > tmax)
        t = tmax;
    if (t < 1)
        t = 1;
    tile_len = (N + t - 1) / t;
    tiles = (uint32_t)((N + tile_len - 1) / tile_len);
    (void)ctx;
}

JobView make_view(const ctd_job *job, uint32_t *d_counts, uint64_t *d_factors)
{
    JobView v{};
    v.family = job->family;
    v.tiles = 1;
    v.param = job->param;
    v.n0 = job->n0;
    v.n1 = job->n1;
    v.tile_len = job->n1 - job->n0;
    v.fb.counts = d_counts;
    v.fb.factors = d_factors;
    v.fb.max_factors = job->max_factors;
    return v;
}

}  // namespace

namespace ctd {
int ctx_device(const ctd_ctx *ctx) { return ctx->device; }
int ctx_sm_count(const ctd_ctx *ctx) { return ctx->sm_count; }
cudaStream_t ctx_stream(const ctd_ctx *ctx) { return ctx->stream; }
SieveWorkspace *ctx_workspace(const ctd_ctx *ctx) { return ctx->ws; }
int ctx_fail(ctd_ctx *ctx, int code, const std::string &msg) { return fail(ctx, code, msg); }
}  // namespace ctd

extern "C" {

int ctd_abi_version(void) { return CTD_ABI_VERSION; }

uint64_t ctd_kernel_launches(void) { return kernel_launch_count(); }

const char *ctd_strerror(int status)
{
    switch (status) {
    case CTD_OK: return "ok";
    case CTD_ERR_INVALID_ARGUMENT: return "invalid argument";
    case CTD_ERR_CUDA: return "CUDA error";
    case CTD_ERR_OUT_OF_MEMORY: return "out of device memory";
    case CTD_ERR_ABORTED: return "aborted by callback";
    case CTD_ERR_TIMEOUT: return "wait limit expired";
    case CTD_ERR_CAPACITY: return "output buffer too small";
    case CTD_ERR_NOT_FOUND: return "not found";
    default: return "unknown status";
    }
}

int ctd_open(int device, ctd_ctx **out)
{
    if (!out)
        return CTD_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    ctd_ctx *ctx = new (std::nothrow) ctd_ctx();
    if (!ctx)
        return CTD_ERR_OUT_OF_MEMORY;
    ctx->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) {
        cudaDeviceProp prop;
        e = cudaGetDeviceProperties(&prop, device);
        if (e == cudaSuccess) {
            ctx->sm_count = prop.multiProcessorCount;
            std::strncpy(ctx->name, prop.name, sizeof(ctx->name) - 1);
            ctx->total_mem = prop.totalGlobalMem;
        }
    }
    if (e == cudaSuccess)
        e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        int code = e == cudaErrorMemoryAllocation ? CTD_ERR_OUT_OF_MEMORY : CTD_ERR_CUDA;
        delete ctx;
        return code;
    }
    ctx->ws = sieve_workspace_create();
    *out = ctx;
    return CTD_OK;
}

void ctd_close(ctd_ctx *ctx)
{
    if (!ctx)
        return;
    cudaSetDevice(ctx->device);
    if (ctx->stream)
        cudaStreamSynchronize(ctx->stream);
    sieve_workspace_destroy(ctx->ws);
    cudaFree(ctx->d_primes);
    cudaFree(ctx->d_counts);
    cudaFree(ctx->d_factors);
    if (ctx->stream)
        cudaStreamDestroy(ctx->stream);
    delete ctx;
}

const char *ctd_last_error(const ctd_ctx *ctx) { return ctx ? ctx->last_error.c_str() : "no context"; }

int ctd_device_info(ctd_ctx *ctx, char *name, size_t name_len, uint64_t *total_mem, int *sm_count)
{
    if (!ctx)
        return CTD_ERR_INVALID_ARGUMENT;
    if (name && name_len) {
        std::strncpy(name, ctx->name, name_len - 1);
        name[name_len - 1] = 0;
    }
    if (total_mem)
        *total_mem = ctx->total_mem;
    if (sm_count)
        *sm_count = ctx->sm_count;
    return CTD_OK;
}

int ctd_set_launch(ctd_ctx *ctx, int grid_size, int block_size)
{
    if (!ctx || grid_size < 0 || block_size < 0 || block_size > 1024 || (block_size % 32))
        return fail(ctx, CTD_ERR_INVALID_ARGUMENT, "invalid launch shape");
    ctx->grid_override = grid_size;
    ctx->block_override = block_size;
    return CTD_OK;
}

int ctd_check_job(const ctd_job *job) { return job_ok(job) ? CTD_OK : CTD_ERR_INVALID_ARGUMENT; }

int ctd_sieve_device(ctd_ctx *ctx, uint64_t lo, uint64_t hi, uint64_t *d_out, uint64_t capacity, uint64_t *count,
                     void *stream)
{
    if (!ctx || !count || (capacity && !d_out))
        return fail(ctx, CTD_ERR_INVALID_ARGUMENT, "ctd_sieve_device: bad arguments");
    CTX_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    std::string err;
    int rc = sieve_range(ctx->ws, lo, hi, d_out, capacity, count, st, err);
    if (rc)
        return fail(ctx, rc, err);
    if (*count > capacity)
        return fail(ctx, CTD_ERR_CAPACITY, "ctd_sieve_device: output capacity too small");
    return CTD_OK;
}

int ctd_sieve(ctd_ctx *ctx, uint64_t lo, uint64_t hi, uint64_t *out, uint64_t capacity, uint64_t *count)
{
    if (!ctx || !count || (capacity && !out))
        return fail(ctx, CTD_ERR_INVALID_ARGUMENT, "ctd_sieve: bad arguments");
    CTX_CUDA(cudaSetDevice(ctx->device));
    uint64_t bound = prime_count_upper_bound(lo, hi);
    uint64_t cap = capacity < bound ? capacity : bound;
    int rc = ensure_buffer(ctx, ctx->d_primes, ctx->primes_cap, cap);
    if (rc)
        return rc;
    std::string err;
    rc = sieve_range(ctx->ws, lo, hi, ctx->d_primes, cap, count, ctx->stream, err);
    if (rc)
        return fail(ctx, rc, err);
    uint64_t n = *count < cap ? *count : cap;
    if (n)
        CTX_CUDA(cudaMemcpyAsync(out, ctx->d_primes, n * sizeof(uint64_t), cudaMemcpyDeviceToHost, ctx->stream));
    CTX_CUDA(cudaStreamSynchronize(ctx->stream));
    if (*count > capacity)
        return fail(ctx, CTD_ERR_CAPACITY, "ctd_sieve: output capacity too small");
    return CTD_OK;
}

int ctd_residues_device(ctd_ctx *ctx, const ctd_job *job, const uint64_t *d_primes, uint64_t nprimes,
                        uint32_t *d_counts, uint64_t *d_factors, void *stream)
{
    if (!ctx || !job_ok(job) || !d_counts || !d_factors || (nprimes && !d_primes))
        return fail(ctx, CTD_ERR_INVALID_ARGUMENT, "ctd_residues_device: bad arguments");
    CTX_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    JobView v = make_view(job, d_counts, d_factors);
    const int block = default_block(ctx);
    const int grid = default_grid(ctx, job->family, block);
    choose_tiles(ctx, nprimes, job->n1 - job->n0, grid, block, v.tiles, v.tile_len);
    std::string err;
    int rc = launch_residues(v, d_primes, nprimes, grid, block, st, err);
    return rc ? fail(ctx, rc, err) : CTD_OK;
}

int ctd_mod2_device(ctd_ctx *ctx, const ctd_job *job, uint32_t *d_counts, uint64_t *d_factors, void *stream)
{
    if (!ctx || !job_ok(job) || !d_counts || !d_factors)
        return fail(ctx, CTD_ERR_INVALID_ARGUMENT, "ctd_mod2_device: bad arguments");
    CTX_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    std::string err;
    int rc = launch_mod2(make_view(job, d_counts, d_factors), st, err);
    return rc ? fail(ctx, rc, err) : CTD_OK;
}

int ctd_run_plain(ctd_ctx *ctx, const ctd_job *job, uint32_t *counts_inout, uint64_t *factors_inout,
                  uint64_t resume_after_prime, uint64_t segment_length, ctd_progress_cb cb, void *user)
{
    if (!ctx)
        return CTD_ERR_INVALID_ARGUMENT;
    if (!job_ok(job))
        return fail(ctx, CTD_ERR_INVALID_ARGUMENT, "invalid job (family, parameter or index range)");
    if (!counts_inout || !factors_inout)
        return fail(ctx, CTD_ERR_INVALID_ARGUMENT, "null factors buffer");
    if (job->f1 <= job->f0)
        return fail(ctx, CTD_ERR_INVALID_ARGUMENT, "empty prime range");
    CTX_CUDA(cudaSetDevice(ctx->device));
    const auto t_start = std::chrono::steady_clock::now();
    const uint64_t N = job->n1 - job->n0;
    const uint64_t NF = N * job->max_factors;
    int rc = ensure_buffer(ctx, ctx->d_counts, ctx->counts_cap, N);
    if (!rc)
        rc = ensure_buffer(ctx, ctx->d_factors, ctx->factors_cap, NF);
    if (rc)
        return rc;
    cudaStream_t st = ctx->stream;
    // the resume state (zeros for a fresh job) goes to the device once
    CTX_CUDA(cudaMemcpyAsync(ctx->d_counts, counts_inout, N * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    CTX_CUDA(cudaMemcpyAsync(ctx->d_factors, factors_inout, NF * sizeof(uint64_t), cudaMemcpyHostToDevice, st));
    JobView view = make_view(job, ctx->d_counts, ctx->d_factors);
    std::string err;

    uint64_t f0 = resume_after_prime ? resume_after_prime + 1 : job->f0;
    const uint64_t f1 = job->f1;
    if (f0 <= 2 && f1 > 2) {  // the prime 2 (src/trial_factoring.cuh:414-418)
        f0 = 3;
        rc = launch_mod2(view, st, err);
        if (rc)
            return fail(ctx, rc, err);
    }
    const uint64_t seg = segment_length ? segment_length : (1ull << 26);
    const int block = default_block(ctx);
    const int grid = default_grid(ctx, job->family, block);
    uint64_t last_prime = resume_after_prime;
    uint64_t primes_done = 0;
    for (uint64_t fx = f0, fy = (f1 - f0 > seg) ? f0 + seg : f1; fx < f1;
         fx = fy, fy = (f1 - fy > seg) ? fy + seg : f1) {
        const uint64_t bound = prime_count_upper_bound(fx, fy);
        rc = ensure_buffer(ctx, ctx->d_primes, ctx->primes_cap, bound);
        if (rc)
            return rc;
        uint64_t np = 0;
        rc = sieve_range(ctx->ws, fx, fy, ctx->d_primes, ctx->primes_cap, &np, st, err);
        if (rc)
            return fail(ctx, rc, err);
        if (np > ctx->primes_cap)
            return fail(ctx, CTD_ERR_CAPACITY, "prime count above its bound");
        if (np) {
            choose_tiles(ctx, np, N, grid, block, view.tiles, view.tile_len);
            rc = launch_residues(view, ctx->d_primes, np, grid, block, st, err);
            if (rc)
                return fail(ctx, rc, err);
            uint64_t lp = 0;
            CTX_CUDA(cudaMemcpyAsync(&lp, ctx->d_primes + np - 1, sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
            CTX_CUDA(cudaStreamSynchronize(st));
            last_prime = lp;
            primes_done += np;
        } else {
            CTX_CUDA(cudaStreamSynchronize(st));
        }
        if (cb) {
            ctd_progress prog;
            prog.segment_end = fy;
            prog.last_prime = last_prime;
            prog.primes_done = primes_done;
            prog.elapsed_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
            int want = cb(user, &prog, 0);
            if (want == CTD_CB_SNAPSHOT) {
                CTX_CUDA(cudaMemcpyAsync(counts_inout, ctx->d_counts, N * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                         st));
                CTX_CUDA(cudaMemcpyAsync(factors_inout, ctx->d_factors, NF * sizeof(uint64_t),
                                         cudaMemcpyDeviceToHost, st));
                CTX_CUDA(cudaStreamSynchronize(st));
                want = cb(user, &prog, 1);
            }
            if (want == CTD_CB_ABORT)
                return fail(ctx, CTD_ERR_ABORTED, "aborted by progress callback");
        }
        if (fy == f1)
            break;
    }
    CTX_CUDA(cudaMemcpyAsync(counts_inout, ctx->d_counts, N * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    CTX_CUDA(cudaMemcpyAsync(factors_inout, ctx->d_factors, NF * sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
    CTX_CUDA(cudaStreamSynchronize(st));
    return CTD_OK;
}

}  // extern "C"
