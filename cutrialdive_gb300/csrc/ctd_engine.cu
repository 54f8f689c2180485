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
    ResidueScratch *rs = nullptr;
    BatchCache *batch = nullptr;
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
    // the occupied slots of a factors buffer packed for the way back to the
    // host (pack_occupied): device records, their length, pinned host copy
    uint64_t *d_pack = nullptr;
    size_t pack_cap = 0;
    unsigned long long *d_pack_words = nullptr;
    size_t pack_words_cap = 0;
    uint64_t *h_pack = nullptr;
    size_t h_pack_cap = 0;
    // per-family launch and tiling parameters (ctd_set_tuning / ctd_autotune)
    ctd_tuning tuning[10] = {};
    bool tuned[10] = {};
    // per family and prime width (bit length of the primes, 0..64): what
    // ctd_autotune measured or ctd_set_tuning_for set; wins over the family
    // entry above for primes of that width
    ctd_tuning wtuning[10][65] = {};
    bool wtuned[10][65] = {};
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

// ---- the factors buffer across the host link
// A buffer holds max_factors slots a term and a few thousand hits a
// segment: a call moves the counts and only the occupied slots.  A fresh
// buffer (every count zero, so every slot zero) is cleared on the device
// instead of copied; on the way back each term with hits becomes a record
// {term, count, its min(count, max_factors) slots} in a packed device
// buffer (record order is arrival order: the host places each by its term).
__global__ void pack_occupied(const uint32_t *__restrict__ counts, const uint64_t *__restrict__ factors, uint64_t n,
                              uint32_t maxf, uint64_t *__restrict__ pack, unsigned long long *__restrict__ words)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint32_t c = counts[i];
        if (!c)
            continue;
        const uint32_t k = c < maxf ? c : maxf;
        const unsigned long long at = atomicAdd(words, (unsigned long long)k + 2);
        pack[at] = i;
        pack[at + 1] = c;
        for (uint32_t j = 0; j < k; ++j)
            pack[at + 2 + j] = factors[i * maxf + j];
    }
}

bool all_zero(const uint32_t *a, uint64_t n)
{
    for (uint64_t i = 0; i < n; ++i)
        if (a[i])
            return false;
    return true;
}

// the resume state to the device: cleared there when it is all zeros
int factors_to_device(ctd_ctx *ctx, const uint32_t *counts, const uint64_t *factors, uint64_t n, uint32_t maxf,
                      cudaStream_t st)
{
    if (all_zero(counts, n)) {
        CTX_CUDA(cudaMemsetAsync(ctx->d_counts, 0, n * sizeof(uint32_t), st));
        CTX_CUDA(cudaMemsetAsync(ctx->d_factors, 0, n * maxf * sizeof(uint64_t), st));
        return CTD_OK;
    }
    CTX_CUDA(cudaMemcpyAsync(ctx->d_counts, counts, n * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    CTX_CUDA(cudaMemcpyAsync(ctx->d_factors, factors, n * maxf * sizeof(uint64_t), cudaMemcpyHostToDevice, st));
    return CTD_OK;
}

// the result to the host: the counts, then the occupied slots as records
// (the whole factors array when the records would not be much smaller);
// the host slots past a term's count keep their zeros
int factors_to_host(ctd_ctx *ctx, uint32_t *counts, uint64_t *factors, uint64_t n, uint32_t maxf, cudaStream_t st)
{
    const uint64_t nf = n * maxf;
    int rc = ensure_buffer(ctx, ctx->d_pack, ctx->pack_cap, nf + 2 * n);
    if (!rc)
        rc = ensure_buffer(ctx, ctx->d_pack_words, ctx->pack_words_cap, 1);
    if (rc)
        return rc;
    CTX_CUDA(cudaMemcpyAsync(counts, ctx->d_counts, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    CTX_CUDA(cudaMemsetAsync(ctx->d_pack_words, 0, sizeof(unsigned long long), st));
    const uint64_t want = (n + 255) / 256;
    const int grid = (int)(want < (uint64_t)ctx->sm_count * 4 ? (want ? want : 1) : (uint64_t)ctx->sm_count * 4);
    pack_occupied<<<grid, 256, 0, st>>>(ctx->d_counts, ctx->d_factors, n, maxf, ctx->d_pack, ctx->d_pack_words);
    CTX_CUDA(cudaGetLastError());
    note_kernel_launch();
    unsigned long long words = 0;
    CTX_CUDA(cudaMemcpyAsync(&words, ctx->d_pack_words, sizeof(words), cudaMemcpyDeviceToHost, st));
    CTX_CUDA(cudaStreamSynchronize(st));
    if (words * 2 > nf) {
        CTX_CUDA(cudaMemcpyAsync(factors, ctx->d_factors, nf * sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
        CTX_CUDA(cudaStreamSynchronize(st));
        return CTD_OK;
    }
    if (words > ctx->h_pack_cap) {
        cudaFreeHost(ctx->h_pack);
        ctx->h_pack = nullptr;
        ctx->h_pack_cap = 0;
        const size_t cap = words < 4096 ? 4096 : 2 * words;
        CTX_CUDA(cudaMallocHost(&ctx->h_pack, cap * sizeof(uint64_t)));
        ctx->h_pack_cap = cap;
    }
    if (words) {
        CTX_CUDA(cudaMemcpyAsync(ctx->h_pack, ctx->d_pack, words * sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
        CTX_CUDA(cudaStreamSynchronize(st));
    }
    for (uint64_t at = 0; at < words;) {
        const uint64_t i = ctx->h_pack[at];
        const uint64_t c = ctx->h_pack[at + 1];
        const uint64_t k = c < maxf ? c : maxf;
        std::memcpy(factors + i * maxf, ctx->h_pack + at + 2, k * sizeof(uint64_t));
        at += k + 2;
    }
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

// slot of a family in the tuning tables (the nine num_seq_id families, then PEANO)
int tuning_slot(uint32_t family) { return family < 9 ? (int)family : 9; }

constexpr uint32_t DEFAULT_ITEMS_PER_THREAD = 8;
constexpr uint32_t DEFAULT_MIN_TILE = 4096;
constexpr uint32_t DEFAULT_SEGMENT_LOG2 = 26;

int bit_length(uint64_t x) { return x ? 64 - __builtin_clzll(x) : 0; }

// the entry in force for `family` at primes of `bits` bits: the width entry,
// else the family entry, else none (defaults)
const ctd_tuning *tuning_of(const ctd_ctx *ctx, uint32_t family, int bits)
{
    const int k = tuning_slot(family);
    if (bits >= 0 && bits <= 64 && ctx->wtuned[k][bits])
        return &ctx->wtuning[k][bits];
    return ctx->tuned[k] ? &ctx->tuning[k] : nullptr;
}

int default_block(const ctd_ctx *ctx, uint32_t family, int bits)
{
    if (ctx->block_override > 0)
        return ctx->block_override;
    const ctd_tuning *t = tuning_of(ctx, family, bits);
    return t && t->block_size > 0 ? t->block_size : 256;
}

// CTAs of `family` at `block` threads in the persistent grid: the resident
// maximum, or fewer when the tuning says so
int grid_for(const ctd_ctx *ctx, uint32_t family, int block, int ctas_per_sm)
{
    int per_sm = residue_blocks_per_sm(family, block);
    if (per_sm < 1)
        per_sm = 1;
    if (ctas_per_sm > 0 && ctas_per_sm < per_sm)
        per_sm = ctas_per_sm;
    return ctx->sm_count * per_sm;
}

int default_grid(ctd_ctx *ctx, uint32_t family, int block, int bits)
{
    if (ctx->grid_override > 0)
        return ctx->grid_override;
    // persistent grid: exactly the CTAs that are resident at once, so every
    // thread strides over the same number of work items and no CTA waits
    // for a second wave
    const ctd_tuning *t = tuning_of(ctx, family, bits);
    return grid_for(ctx, family, block, t ? t->ctas_per_sm : 0);
}

// index tiles per prime so that short prime lists still fill the GPU,
// keeping each tile long enough to amortize its jump
void tiles_for(uint64_t nprimes, uint64_t N, int grid, int block, uint32_t items_per_thread, uint32_t min_tile,
               uint32_t &tiles, uint64_t &tile_len)
{
    tiles = 1;
    tile_len = N;
    const uint64_t threads = (uint64_t)grid * block;
    const uint64_t want = (uint64_t)items_per_thread * threads;
    if (nprimes >= want || N < 2 * (uint64_t)min_tile)
        return;
    uint64_t t = (want + nprimes - 1) / (nprimes ? nprimes : 1);
    uint64_t tmax = N / min_tile;
    if (t > tmax)
        t = tmax;
    if (t < 1)
        t = 1;
    tile_len = (N + t - 1) / t;
    tiles = (uint32_t)((N + tile_len - 1) / tile_len);
}

void choose_tiles(const ctd_ctx *ctx, uint32_t family, int bits, uint64_t nprimes, uint64_t N, int grid, int block,
                  uint32_t &tiles, uint64_t &tile_len)
{
    const ctd_tuning *t = tuning_of(ctx, family, bits);
    tiles_for(nprimes, N, grid, block, t && t->items_per_thread ? t->items_per_thread : DEFAULT_ITEMS_PER_THREAD,
              t && t->min_tile ? t->min_tile : DEFAULT_MIN_TILE, tiles, tile_len);
}

uint32_t variant_of(const ctd_ctx *ctx, uint32_t family, int bits)
{
    const ctd_tuning *t = tuning_of(ctx, family, bits);
    return t ? t->variant : CTD_VARIANT_AUTO;
}

uint32_t classify_min_of(const ctd_ctx *ctx, uint32_t family, int bits)
{
    const ctd_tuning *t = tuning_of(ctx, family, bits);
    return t && t->classify_min ? t->classify_min : DEFAULT_CLASSIFY_MIN;
}

uint32_t refine_q_of(const ctd_ctx *ctx, uint32_t family, int bits)
{
    const ctd_tuning *t = tuning_of(ctx, family, bits);
    return t ? t->refine_q : 0;
}

uint64_t default_segment(const ctd_ctx *ctx, uint32_t family, int bits)
{
    const ctd_tuning *t = tuning_of(ctx, family, bits);
    return 1ull << (t && t->segment_log2 ? t->segment_log2 : DEFAULT_SEGMENT_LOG2);
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
BatchCache *&ctx_batch_cache(ctd_ctx *ctx) { return ctx->batch; }
ctd_tuning ctx_tuning(ctd_ctx *ctx, uint32_t family, uint64_t first_prime)
{
    ctd_tuning t{};
    ctd_get_tuning_for(ctx, family, (uint32_t)bit_length(first_prime < 3 ? 3 : first_prime), &t);
    return t;
}
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
    // device tables of the residue kernels, uploaded before any launch or
    // graph capture on this device
    std::string terr;
    int trc = prepare_residue_tables(device, terr);
    if (trc == CTD_OK)
        trc = noalloc_prepare(device, terr);
    if (trc != CTD_OK) {
        cudaStreamDestroy(ctx->stream);
        delete ctx;
        return trc;
    }
    ctx->ws = sieve_workspace_create();
    ctx->rs = residue_scratch_create(device, ctx->sm_count);
    if (!ctx->ws || !ctx->rs) {
        sieve_workspace_destroy(ctx->ws);
        residue_scratch_destroy(ctx->rs);
        cudaStreamDestroy(ctx->stream);
        delete ctx;
        return CTD_ERR_OUT_OF_MEMORY;
    }
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
    residue_scratch_destroy(ctx->rs);
    batch_cache_destroy(ctx->batch);
    cudaFree(ctx->d_primes);
    cudaFree(ctx->d_counts);
    cudaFree(ctx->d_factors);
    cudaFree(ctx->d_pack);
    cudaFree(ctx->d_pack_words);
    cudaFreeHost(ctx->h_pack);
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

int ctd_get_tuning(ctd_ctx *ctx, uint32_t family, ctd_tuning *out) { return ctd_get_tuning_for(ctx, family, 0, out); }

int ctd_get_tuning_for(ctd_ctx *ctx, uint32_t family, uint32_t prime_bits, ctd_tuning *out)
{
    if (!ctx || !out || prime_bits > 64)
        return CTD_ERR_INVALID_ARGUMENT;
    const ctd_tuning *t = tuning_of(ctx, family, prime_bits ? (int)prime_bits : -1);
    if (t) {
        *out = *t;
        return CTD_OK;
    }
    *out = ctd_tuning{};
    out->block_size = 256;
    out->ctas_per_sm = residue_blocks_per_sm(family, 256);
    out->items_per_thread = DEFAULT_ITEMS_PER_THREAD;
    out->min_tile = DEFAULT_MIN_TILE;
    out->segment_log2 = DEFAULT_SEGMENT_LOG2;
    return CTD_OK;
}

int ctd_set_tuning(ctd_ctx *ctx, uint32_t family, const ctd_tuning *t) { return ctd_set_tuning_for(ctx, family, 0, t); }

int ctd_set_tuning_for(ctd_ctx *ctx, uint32_t family, uint32_t prime_bits, const ctd_tuning *t)
{
    if (!ctx || prime_bits > 64)
        return CTD_ERR_INVALID_ARGUMENT;
    const int k = tuning_slot(family);
    if (!t) {
        if (prime_bits)
            ctx->wtuned[k][prime_bits] = false;
        else
            ctx->tuned[k] = false;
        return CTD_OK;
    }
    if (t->block_size < 32 || t->block_size > 256 || (t->block_size % 32) || t->ctas_per_sm < 0 ||
        t->items_per_thread == 0 || t->min_tile == 0 || (t->segment_log2 && (t->segment_log2 < 20 || t->segment_log2 > 40)) ||
        t->variant > CTD_VARIANT_MONTGOMERY)
        return fail(ctx, CTD_ERR_INVALID_ARGUMENT,
                    "ctd_set_tuning: block_size 32..256 (multiple of 32), ctas_per_sm >= 0, items_per_thread and "
                    "min_tile > 0, segment_log2 0 or 20..40, variant 0..2");
    if (prime_bits) {
        ctx->wtuning[k][prime_bits] = *t;
        ctx->wtuned[k][prime_bits] = true;
    } else {
        ctx->tuning[k] = *t;
        ctx->tuned[k] = true;
    }
    return CTD_OK;
}

int ctd_autotune(ctd_ctx *ctx, const ctd_job *job, double budget_s, ctd_tuning *best)
{
    if (!ctx || !best || !job_ok(job) || job->f1 <= job->f0 || !(budget_s > 0))
        return fail(ctx, CTD_ERR_INVALID_ARGUMENT, "ctd_autotune: bad arguments");
    CTX_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    const auto t0 = std::chrono::steady_clock::now();
    auto elapsed = [&] { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); };
    // the sample: the job's first prime segment (odd primes only); the
    // result is kept for the family at this prime width
    const uint64_t fx = job->f0 < 3 ? 3 : job->f0;
    const int bits = bit_length(fx);
    ctd_tuning cur{};
    ctd_get_tuning_for(ctx, job->family, (uint32_t)bits, &cur);
    const uint64_t seg = 1ull << (cur.segment_log2 ? cur.segment_log2 : DEFAULT_SEGMENT_LOG2);
    const uint64_t fy = job->f1 - fx > seg ? fx + seg : job->f1;
    if (fx >= fy) {
        *best = cur;
        return CTD_OK;
    }
    const uint64_t N = job->n1 - job->n0;
    int rc = ensure_buffer(ctx, ctx->d_primes, ctx->primes_cap, prime_count_upper_bound(fx, fy));
    if (!rc)
        rc = ensure_buffer(ctx, ctx->d_counts, ctx->counts_cap, N);
    if (!rc)
        rc = ensure_buffer(ctx, ctx->d_factors, ctx->factors_cap, N * job->max_factors);
    if (rc)
        return rc;
    std::string err;
    uint64_t np = 0;
    rc = sieve_range(ctx->ws, fx, fy, ctx->d_primes, ctx->primes_cap, &np, st, err);
    if (rc)
        return fail(ctx, rc, err);
    if (!np) {
        *best = cur;
        return CTD_OK;
    }
    cudaEvent_t ea, eb;
    CTX_CUDA(cudaEventCreate(&ea));
    CTX_CUDA(cudaEventCreate(&eb));
    JobView view = make_view(job, ctx->d_counts, ctx->d_factors);
    // milliseconds of one residue launch over `n` sample primes (best of two
    // after a warm-up); the counts are cleared so no term overflows
    auto time_config = [&](const ctd_tuning &c, uint64_t n, float &ms) -> int {
        const int grid = grid_for(ctx, job->family, c.block_size, c.ctas_per_sm);
        tiles_for(n, N, grid, c.block_size, c.items_per_thread, c.min_tile, view.tiles, view.tile_len);
        view.variant = c.variant;
        view.classify_min = c.classify_min ? c.classify_min : DEFAULT_CLASSIFY_MIN;
        view.refine_q = c.refine_q;
        ms = 1e30f;
        for (int r = 0; r < 3; ++r) {
            if (cudaMemsetAsync(ctx->d_counts, 0, N * sizeof(uint32_t), st) != cudaSuccess)
                return CTD_ERR_CUDA;
            cudaEventRecord(ea, st);
            int e = launch_residues(view, ctx->d_primes, n, grid, c.block_size, st, err, ctx->rs);
            if (e)
                return e;
            cudaEventRecord(eb, st);
            if (cudaEventSynchronize(eb) != cudaSuccess)
                return CTD_ERR_CUDA;
            float t = 0;
            cudaEventElapsedTime(&t, ea, eb);
            if (r && t < ms)
                ms = t;
        }
        return CTD_OK;
    };
    auto try_config = [&](const ctd_tuning &t, ctd_tuning &winner, float &best_ms) -> int {
        float ms = 0;
        const int e = time_config(t, np, ms);
        if (!e && ms < best_ms) {
            best_ms = ms;
            winner = t;
        }
        return e;
    };
    ctd_tuning base = cur;
    base.block_size = 256;
    base.ctas_per_sm = 0;
    base.variant = CTD_VARIANT_AUTO;
    float best_ms = 0;
    rc = time_config(base, np, best_ms);
    // keep one trial near a sixth of the budget: a prefix of the sample primes
    if (!rc && best_ms * 1e-3 * 3 > budget_s / 6) {
        const double f = (budget_s / 6) / (best_ms * 1e-3 * 3);
        const uint64_t floor_n = (uint64_t)ctx->sm_count * 256 * 8;
        uint64_t n2 = (uint64_t)(np * f);
        np = n2 > floor_n ? n2 : (floor_n < np ? floor_n : np);
        rc = time_config(base, np, best_ms);
    }
    ctd_tuning winner = base;
    const uint32_t fam = job->family;
    // power-residue classes (doubling families): always, or never; then the
    // rare primes of their refinement: all (up to 127, the starting entry),
    // none, up to 31
    if (!rc && (fam == CTD_PROTH || fam == CTD_RIESEL || fam == CTD_MERSENNE)) {
        for (uint32_t cm : {1u, 0xffffffffu}) {
            if (elapsed() >= budget_s)
                break;
            ctd_tuning t = winner;
            t.classify_min = cm;
            rc = try_config(t, winner, best_ms);
            if (rc)
                break;
        }
        for (uint32_t rq : {1u, 31u}) {
            if (rc || elapsed() >= budget_s || winner.classify_min == 0xffffffffu)
                break;
            ctd_tuning t = winner;
            t.refine_q = rq;
            rc = try_config(t, winner, best_ms);
        }
    }
    // launch shape: block size and resident CTAs per SM
    const int blocks[] = {256, 128, 64};
    for (int bi = 0; !rc && bi < 3 && elapsed() < budget_s; ++bi) {
        const int occ = residue_blocks_per_sm(fam, blocks[bi]);
        const int cands[] = {occ, occ - 1, occ / 2, (occ * 3) / 4};
        for (int ci = 0; !rc && ci < 4 && elapsed() < budget_s; ++ci) {
            const int c = cands[ci];
            if (c < 1 || (blocks[bi] == 256 && c == occ))
                continue;
            ctd_tuning t = winner;
            t.block_size = blocks[bi];
            t.ctas_per_sm = c;
            rc = try_config(t, winner, best_ms);
        }
    }
    // tiling: only where it changes the split of this sample
    const uint32_t items[] = {2, 4, 8, 16, 32};
    const uint32_t tiles_min[] = {1024, 2048, 4096, 8192, 16384};
    const int wgrid = grid_for(ctx, fam, winner.block_size, winner.ctas_per_sm);
    uint32_t seen_tiles[32];
    int nseen = 0;
    {
        uint32_t tt;
        uint64_t tl;
        tiles_for(np, N, wgrid, winner.block_size, winner.items_per_thread, winner.min_tile, tt, tl);
        seen_tiles[nseen++] = tt;
    }
    for (int i = 0; !rc && i < 5 && elapsed() < budget_s; ++i)
        for (int j = 0; !rc && j < 5 && elapsed() < budget_s; ++j) {
            ctd_tuning t = winner;
            t.items_per_thread = items[i];
            t.min_tile = tiles_min[j];
            uint32_t tt;
            uint64_t tl;
            tiles_for(np, N, wgrid, t.block_size, t.items_per_thread, t.min_tile, tt, tl);
            bool dup = false;
            for (int k = 0; k < nseen; ++k)
                dup |= seen_tiles[k] == tt;
            if (dup || nseen >= 32)
                continue;
            seen_tiles[nseen++] = tt;
            rc = try_config(t, winner, best_ms);
        }
    // step form: the term-by-term walk against the blocks (doubling, fixed-n),
    // and the Smarandache step variants
    const bool has_walk = fam == CTD_PROTH || fam == CTD_RIESEL || fam == CTD_MERSENNE ||
                          fam == CTD_PROTH_FIXED_N || fam == CTD_RIESEL_FIXED_N || fam == CTD_SMARANDACHE;
    for (uint32_t v = CTD_VARIANT_WALK; !rc && has_walk && v <= CTD_VARIANT_MONTGOMERY && elapsed() < budget_s; ++v) {
        if (v == CTD_VARIANT_MONTGOMERY && fam != CTD_SMARANDACHE)
            break;
        ctd_tuning t = winner;
        t.variant = v;
        rc = try_config(t, winner, best_ms);
    }
    // segment length: one whole segment (device sieve + residue launch) per
    // candidate, compared per prime; the plain path walks the job in segments
    // of the winner's length
    if (!rc && elapsed() < budget_s) {
        double best_per_prime = 0;
        uint32_t best_log2 = winner.segment_log2 ? winner.segment_log2 : DEFAULT_SEGMENT_LOG2;
        for (uint32_t lg : {26u, 28u, 30u}) {
            if (elapsed() >= budget_s)
                break;
            const uint64_t sy = job->f1 - fx > (1ull << lg) ? fx + (1ull << lg) : job->f1;
            if (ensure_buffer(ctx, ctx->d_primes, ctx->primes_cap, prime_count_upper_bound(fx, sy)))
                break;
            const int grid = grid_for(ctx, fam, winner.block_size, winner.ctas_per_sm);
            view.variant = winner.variant;
            view.classify_min = winner.classify_min ? winner.classify_min : DEFAULT_CLASSIFY_MIN;
            view.refine_q = winner.refine_q;
            uint64_t n = 0;
            float t = 0;
            if (cudaMemsetAsync(ctx->d_counts, 0, N * sizeof(uint32_t), st) != cudaSuccess)
                break;
            cudaEventRecord(ea, st);
            rc = sieve_range(ctx->ws, fx, sy, ctx->d_primes, ctx->primes_cap, &n, st, err);
            if (!rc && n) {
                tiles_for(n, N, grid, winner.block_size, winner.items_per_thread, winner.min_tile, view.tiles,
                          view.tile_len);
                rc = launch_residues(view, ctx->d_primes, n, grid, winner.block_size, st, err, ctx->rs);
            }
            cudaEventRecord(eb, st);
            if (rc || cudaEventSynchronize(eb) != cudaSuccess)
                break;
            cudaEventElapsedTime(&t, ea, eb);
            const double per_prime = n ? t / (double)n : 1e30;
            if (!best_per_prime || per_prime < best_per_prime) {
                best_per_prime = per_prime;
                best_log2 = lg;
            }
            if (sy == job->f1)
                break;  // the job has no longer segment to offer
        }
        winner.segment_log2 = best_log2;
    }
    cudaEventDestroy(ea);
    cudaEventDestroy(eb);
    if (rc)
        return fail(ctx, rc, err.empty() ? std::string("ctd_autotune: CUDA error") : err);
    const int k = tuning_slot(fam);
    ctx->wtuning[k][bits] = winner;
    ctx->wtuned[k][bits] = true;
    *best = winner;
    return CTD_OK;
}

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
    // the width of the list's primes: the job's prime range start (the
    // list holds primes of [f0, f1))
    const int bits = bit_length(job->f0 < 3 ? 3 : job->f0);
    JobView v = make_view(job, d_counts, d_factors);
    v.variant = variant_of(ctx, job->family, bits);
    v.classify_min = classify_min_of(ctx, job->family, bits);
    v.refine_q = refine_q_of(ctx, job->family, bits);
    const int block = default_block(ctx, job->family, bits);
    const int grid = default_grid(ctx, job->family, block, bits);
    choose_tiles(ctx, job->family, bits, nprimes, job->n1 - job->n0, grid, block, v.tiles, v.tile_len);
    std::string err;
    int rc = launch_residues(v, d_primes, nprimes, grid, block, st, err, ctx->rs);
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
    rc = factors_to_device(ctx, counts_inout, factors_inout, N, job->max_factors, st);
    if (rc)
        return rc;
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
    // tuning by prime width: the job's first prime sets the segment length,
    // each segment's first prime its launch shape and step forms
    const uint64_t seg = segment_length ? segment_length : default_segment(ctx, job->family, bit_length(f0));
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
            const int bits = bit_length(fx);
            const int block = default_block(ctx, job->family, bits);
            const int grid = default_grid(ctx, job->family, block, bits);
            view.variant = variant_of(ctx, job->family, bits);
            view.classify_min = classify_min_of(ctx, job->family, bits);
            view.refine_q = refine_q_of(ctx, job->family, bits);
            choose_tiles(ctx, job->family, bits, np, N, grid, block, view.tiles, view.tile_len);
            rc = launch_residues(view, ctx->d_primes, np, grid, block, st, err, ctx->rs);
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
    return factors_to_host(ctx, counts_inout, factors_inout, N, job->max_factors, st);
}

}  // extern "C"
