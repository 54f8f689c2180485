// ctd_sieve.cu -- device segmented sieve of Eratosthenes.
//
// Replaces the reference's host siever (src/siever.hpp:179-237: primesieve
// on `threads` host workers) and the synchronous host-to-device copy of each
// segment's primes (src/prime_data.hpp:166-196).  Primes are produced on the
// GPU and written straight into an HBM chunk, ascending, as u64.
//
// Layout: odd numbers only, one bit each.  A window is WIN_WORDS 32-bit words
// (2^19 odd numbers, a 2^20-wide range) held in shared memory.
//   pass 1  sieve_windows: each CTA clears a window, crosses off multiples
//           of every odd base prime p (p^2 below the window end) with
//           shared-memory atomics, writes the prime bitmap to global memory
//           and its popcount;
//   pass 2  scan_counts: exclusive scan of the window counts (one CTA);
//   pass 3  compact: each CTA re-reads a window's bitmap and writes its
//           primes at the window's offset, ordered by a block scan per round.
// Base primes (all odd p <= sqrt(hi)) come from the same kernels: the odd
// primes below 2^16 from a one-CTA sieve, the rest by sieving [3, sqrt(hi)].
#include "ctd_internal.h"

#include <algorithm>
#include <cmath>
#include <vector>

namespace ctd {

namespace {

constexpr uint32_t WIN_WORDS = 16384;                       // 64 KiB of shared memory
constexpr uint64_t WIN_ODD = 32ull * WIN_WORDS;             // odd numbers per window
constexpr int SIEVE_THREADS = 512;
constexpr uint32_t SMALL_PRIMES = 256;                      // crossed off cooperatively by the CTA
constexpr uint32_t LEVEL0_LIMIT = 65536;                    // level-0 base primes: odd p < 2^16

#define CUDA_TRY(expr)                                                      \
    do {                                                                    \
        cudaError_t e_ = (expr);                                            \
        if (e_ != cudaSuccess) {                                            \
            err = std::string(#expr ": ") + cudaGetErrorString(e_);         \
            return e_ == cudaErrorMemoryAllocation ? CTD_ERR_OUT_OF_MEMORY  \
                                                   : CTD_ERR_CUDA;          \
        }                                                                   \
    } while (0)

// index (in odd steps from wlo) of the first odd multiple of p that is
// >= max(p^2, wlo)
__device__ __forceinline__ uint64_t first_index(uint32_t p, uint64_t wlo)
{
    uint64_t pp = (uint64_t)p * p;
    uint64_t m;
    if (pp >= wlo) {
        m = pp;
    } else {
        uint64_t r = wlo % p;
        m = r ? wlo + (p - r) : wlo;
        if (!(m & 1))
            m += p;
    }
    return (m - wlo) >> 1;
}

// The wheel: the odd primes 3..31, whose multiples take most of a
// window's crossings (sum of 1/q = 1.06 of about 2.3 for all base primes).
// Their multiples in a word of 32 odd numbers are a fixed bit pattern
// shifted to the word's phase, so each word gets them by shifts and ORs
// written once, not by shared-memory atomics bit by bit.
constexpr int WHEEL = 10;
__host__ __device__ constexpr uint32_t wheel_q(int k)
{
    return k < 5 ? (k < 3 ? 3 + 2 * k : (k == 3 ? 11 : 13)) : (k < 8 ? (k == 5 ? 17 : (k == 6 ? 19 : 23)) : (k == 8 ? 29 : 31));
}

// bits 0, q, 2q, ... of a 32-bit word
__host__ __device__ constexpr uint32_t wheel_pattern(uint32_t q)
{
    uint32_t m = 0;
    for (uint32_t b = 0; b < 32; b += q)
        m |= 1u << b;
    return m;
}

__global__ void __launch_bounds__(SIEVE_THREADS) sieve_windows(uint64_t lo_odd, uint64_t nodd, uint32_t nwin,
                                                               const uint32_t *__restrict__ base, uint32_t nbase,
                                                               uint32_t *__restrict__ bits, uint32_t *__restrict__ wcount)
{
    extern __shared__ uint32_t sm[];
    __shared__ uint32_t warp_sums[SIEVE_THREADS / 32];
    const uint32_t tid = threadIdx.x, bd = blockDim.x;
    for (uint32_t w = blockIdx.x; w < nwin; w += gridDim.x) {
        const uint64_t off = (uint64_t)w * WIN_ODD;
        const uint64_t wlo = lo_odd + 2 * off;
        const uint64_t len = (nodd - off) < WIN_ODD ? (nodd - off) : WIN_ODD;
        const uint64_t whi = wlo + 2 * len;
        {
            // bit b of word i is the odd number wlo + 2 (32 i + b); it is a
            // multiple of q iff its odd index g = (value - 1) / 2 is
            // (q - 1) / 2 mod q, so in word i the multiples start at bit
            // ph = ((q - 1) / 2 - g(i, 0)) mod q, and moving on by bd words
            // lowers ph by 32 bd mod q
            const uint64_t g0 = (wlo - 1) / 2 + 32ull * tid;
            uint32_t ph[WHEEL], step[WHEEL];
#pragma unroll
            for (int k = 0; k < WHEEL; ++k) {
                const uint32_t q = wheel_q(k);
                const uint32_t gm = (uint32_t)(g0 % q);
                const uint32_t h = (q - 1) / 2;
                ph[k] = h >= gm ? h - gm : h + q - gm;
                step[k] = (32u * bd) % q;
            }
            for (uint32_t i = tid; i < WIN_WORDS; i += bd) {
                uint32_t v = 0;
#pragma unroll
                for (int k = 0; k < WHEEL; ++k) {
                    const uint32_t q = wheel_q(k);
                    v |= wheel_pattern(q) << ph[k];
                    ph[k] = ph[k] >= step[k] ? ph[k] - step[k] : ph[k] + q - step[k];
                }
                sm[i] = v;
            }
        }
        __syncthreads();
        if (tid == 0 && wlo <= wheel_q(WHEEL - 1)) {
            // the wheel primes themselves are not composite
            for (int k = 0; k < WHEEL; ++k) {
                const uint64_t q = wheel_q(k);
                if (q >= wlo && q < whi) {
                    const uint64_t j = (q - wlo) >> 1;
                    sm[j >> 5] &= ~(1u << (j & 31));
                }
            }
        }
        __syncthreads();
        // small primes past the wheel: the whole CTA strides over each
        // prime's multiples (base[] starts with the wheel primes 3..31)
        const uint32_t nsmall = nbase < SMALL_PRIMES ? nbase : SMALL_PRIMES;
        for (uint32_t k = WHEEL; k < nsmall; ++k) {
            const uint32_t p = base[k];
            if ((uint64_t)p * p >= whi)
                break;
            const uint64_t j0 = first_index(p, wlo);
            for (uint64_t j = j0 + (uint64_t)tid * p; j < len; j += (uint64_t)bd * p)
                atomicOr(&sm[j >> 5], 1u << (j & 31));
        }
        // larger primes: one prime per thread
        for (uint32_t k = nsmall + tid; k < nbase; k += bd) {
            const uint32_t p = base[k];
            if ((uint64_t)p * p >= whi)
                break;
            for (uint64_t j = first_index(p, wlo); j < len; j += p)
                atomicOr(&sm[j >> 5], 1u << (j & 31));
        }
        __syncthreads();
        uint32_t cnt = 0;
        uint32_t *out = bits + (uint64_t)w * WIN_WORDS;
        for (uint32_t i = tid; i < WIN_WORDS; i += bd) {
            uint32_t v = ~sm[i];
            const uint64_t j = (uint64_t)i * 32;
            if (j + 32 > len)
                v = (j >= len) ? 0u : (v & ((1u << (uint32_t)(len - j)) - 1u));
            out[i] = v;
            cnt += __popc(v);
        }
        // block reduction of the window's prime count
        for (int o = 16; o; o >>= 1)
            cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
        if ((tid & 31) == 0)
            warp_sums[tid >> 5] = cnt;
        __syncthreads();
        if (tid == 0) {
            uint32_t s = 0;
            for (uint32_t i = 0; i < bd / 32; ++i)
                s += warp_sums[i];
            wcount[w] = s;
        }
        __syncthreads();
    }
}

// exclusive scan of window counts into 64-bit offsets; offsets[nwin] = total
__global__ void __launch_bounds__(1024) scan_counts(const uint32_t *__restrict__ wcount, uint32_t nwin,
                                                    uint64_t *__restrict__ offsets)
{
    __shared__ uint64_t warp_sums[32];
    __shared__ uint64_t carry;
    const uint32_t tid = threadIdx.x;
    if (tid == 0)
        carry = 0;
    __syncthreads();
    for (uint32_t base = 0; base < nwin; base += blockDim.x) {
        const uint32_t i = base + tid;
        uint64_t v = i < nwin ? wcount[i] : 0;
        uint64_t x = v;
        for (int o = 1; o < 32; o <<= 1) {
            uint64_t y = __shfl_up_sync(0xffffffffu, x, o);
            if ((tid & 31) >= (uint32_t)o)
                x += y;
        }
        if ((tid & 31) == 31)
            warp_sums[tid >> 5] = x;
        __syncthreads();
        if (tid < 32) {
            uint64_t s = (tid < blockDim.x / 32) ? warp_sums[tid] : 0;
            for (int o = 1; o < 32; o <<= 1) {
                uint64_t y = __shfl_up_sync(0xffffffffu, s, o);
                if (tid >= (uint32_t)o)
                    s += y;
            }
            warp_sums[tid] = s;  // inclusive scan of warp totals
        }
        __syncthreads();
        const uint64_t warp_prefix = (tid >> 5) ? warp_sums[(tid >> 5) - 1] : 0;
        if (i < nwin)
            offsets[i] = carry + warp_prefix + x - v;
        __syncthreads();
        if (tid == 0)
            carry += warp_sums[blockDim.x / 32 - 1];
        __syncthreads();
    }
    if (tid == 0)
        offsets[nwin] = carry;
}

template <class T>
__global__ void __launch_bounds__(SIEVE_THREADS) compact_windows(uint64_t lo_odd, uint32_t nwin,
                                                                 const uint32_t *__restrict__ bits,
                                                                 const uint64_t *__restrict__ offsets,
                                                                 T *__restrict__ out, uint64_t capacity,
                                                                 uint64_t out_base)
{
    __shared__ uint32_t warp_sums[SIEVE_THREADS / 32];
    const uint32_t tid = threadIdx.x, bd = blockDim.x, lane = tid & 31, warp = tid >> 5;
    for (uint32_t w = blockIdx.x; w < nwin; w += gridDim.x) {
        const uint64_t wlo = lo_odd + 2 * (uint64_t)w * WIN_ODD;
        uint64_t run = out_base + offsets[w];
        const uint32_t *wb = bits + (uint64_t)w * WIN_WORDS;
        for (uint32_t r = 0; r < WIN_WORDS; r += bd) {
            const uint32_t i = r + tid;
            uint32_t v = i < WIN_WORDS ? wb[i] : 0u;
            uint32_t c = __popc(v), x = c;
            for (int o = 1; o < 32; o <<= 1) {
                uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= (uint32_t)o)
                    x += y;
            }
            if (lane == 31)
                warp_sums[warp] = x;
            __syncthreads();
            uint32_t before = 0, total = 0;
            for (uint32_t k = 0; k < bd / 32; ++k) {
                uint32_t s = warp_sums[k];
                if (k < warp)
                    before += s;
                total += s;
            }
            uint64_t pos = run + before + x - c;
            while (v) {
                const uint32_t b = __ffs(v) - 1;
                v &= v - 1;
                if (pos < capacity)
                    out[pos] = (T)(wlo + 2 * ((uint64_t)i * 32 + b));
                ++pos;
            }
            run += total;
            __syncthreads();
        }
    }
}

// odd primes below 2^16 by one CTA: cross off multiples of every odd k < 256
__global__ void __launch_bounds__(1024) level0_primes(uint32_t *__restrict__ out, uint32_t *__restrict__ count)
{
    constexpr uint32_t NW = LEVEL0_LIMIT / 64;  // odd numbers 1,3,..,65535 -> 32768 bits
    __shared__ uint32_t sm[NW];
    __shared__ uint32_t warp_sums[32];
    const uint32_t tid = threadIdx.x;
    for (uint32_t i = tid; i < NW; i += blockDim.x)
        sm[i] = 0;
    __syncthreads();
    if (tid == 0)
        atomicOr(&sm[0], 1u);  // 1 is not prime
    for (uint32_t k = 3 + 2 * tid; k < 256; k += 2 * blockDim.x)
        for (uint32_t m = k * k; m < LEVEL0_LIMIT; m += 2 * k)
            atomicOr(&sm[(m >> 1) >> 5], 1u << ((m >> 1) & 31));
    __syncthreads();
    // ordered compaction, one word per thread (NW = 1024 = blockDim)
    uint32_t v = tid < NW ? ~sm[tid] : 0u;
    if (tid == 0)
        v &= ~1u;  // drop 1 (already marked) -- keep explicit
    uint32_t c = __popc(v), x = c;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if ((tid & 31) >= (uint32_t)o)
            x += y;
    }
    if ((tid & 31) == 31)
        warp_sums[tid >> 5] = x;
    __syncthreads();
    uint32_t before = 0, total = 0;
    for (uint32_t k = 0; k < blockDim.x / 32; ++k) {
        if (k < (tid >> 5))
            before += warp_sums[k];
        total += warp_sums[k];
    }
    uint32_t pos = before + x - c;
    while (v) {
        uint32_t b = __ffs(v) - 1;
        v &= v - 1;
        out[pos++] = 2 * (tid * 32 + b) + 1;
    }
    if (tid == 0)
        *count = total;
}

uint64_t isqrt64(uint64_t x)
{
    uint64_t r = (uint64_t)std::sqrt((long double)x);
    while (r * r > x)
        --r;
    while ((r + 1) <= 0xffffffffull && (r + 1) * (r + 1) <= x)
        ++r;
    return r;
}

}  // namespace

struct SieveWorkspace {
    // base primes (odd, ascending) covering [3, base_limit]
    uint32_t *d_base = nullptr;
    uint32_t nbase = 0;
    uint64_t base_limit = 0;
    size_t base_cap = 0;
    // per-range scratch
    uint32_t *d_bits = nullptr;
    size_t bits_cap = 0;  // windows
    uint32_t *d_wcount = nullptr;
    uint64_t *d_offsets = nullptr;
    size_t win_cap = 0;
    uint64_t *h_total = nullptr;  // pinned
    int sm_count = 0;
};

SieveWorkspace *sieve_workspace_create()
{
    auto *ws = new SieveWorkspace();
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&ws->sm_count, cudaDevAttrMultiProcessorCount, dev);
    if (ws->sm_count <= 0)
        ws->sm_count = 1;
    return ws;
}

void sieve_workspace_destroy(SieveWorkspace *ws)
{
    if (!ws)
        return;
    cudaFree(ws->d_base);
    cudaFree(ws->d_bits);
    cudaFree(ws->d_wcount);
    cudaFree(ws->d_offsets);
    cudaFreeHost(ws->h_total);
    delete ws;
}

static int ensure_windows(SieveWorkspace *ws, uint64_t nwin, std::string &err)
{
    if (nwin > ws->win_cap) {
        cudaFree(ws->d_bits);
        cudaFree(ws->d_wcount);
        cudaFree(ws->d_offsets);
        ws->d_bits = nullptr;
        ws->d_wcount = nullptr;
        ws->d_offsets = nullptr;
        ws->win_cap = 0;
        CUDA_TRY(cudaMalloc(&ws->d_bits, nwin * WIN_WORDS * sizeof(uint32_t)));
        CUDA_TRY(cudaMalloc(&ws->d_wcount, nwin * sizeof(uint32_t)));
        CUDA_TRY(cudaMalloc(&ws->d_offsets, (nwin + 1) * sizeof(uint64_t)));
        ws->win_cap = nwin;
    }
    if (!ws->h_total)
        CUDA_TRY(cudaMallocHost(&ws->h_total, sizeof(uint64_t)));
    return CTD_OK;
}

static int grid_for(const SieveWorkspace *ws, uint64_t nwin)
{
    uint64_t g = (uint64_t)ws->sm_count * 3;  // three 64 KiB windows fit an SM
    return (int)(nwin < g ? nwin : g);
}

// odd primes in [lo_odd, lo_odd + 2*nodd) into out[out_base ...], counts in ws
template <class T>
static int sieve_odd(SieveWorkspace *ws, uint64_t lo_odd, uint64_t nodd, const uint32_t *d_base, uint32_t nbase,
                     T *d_out, uint64_t capacity, uint64_t out_base, uint64_t *count, cudaStream_t st,
                     std::string &err)
{
    *count = 0;
    if (!nodd)
        return CTD_OK;
    const uint64_t nwin = (nodd + WIN_ODD - 1) / WIN_ODD;
    if (nwin > 0xffffffffull) {
        err = "sieve range too large";
        return CTD_ERR_INVALID_ARGUMENT;
    }
    int rc = ensure_windows(ws, nwin, err);
    if (rc)
        return rc;
    const size_t smem = WIN_WORDS * sizeof(uint32_t);
    // a function attribute belongs to the current device: set it on every
    // call (a host-side call, no stream work), so a context on any device
    // launches with it
    CUDA_TRY(cudaFuncSetAttribute(sieve_windows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int grid = grid_for(ws, nwin);
    sieve_windows<<<grid, SIEVE_THREADS, smem, st>>>(lo_odd, nodd, (uint32_t)nwin, d_base, nbase, ws->d_bits,
                                                    ws->d_wcount);
    CUDA_TRY(cudaGetLastError());
    note_kernel_launch();
    scan_counts<<<1, 1024, 0, st>>>(ws->d_wcount, (uint32_t)nwin, ws->d_offsets);
    CUDA_TRY(cudaGetLastError());
    note_kernel_launch();
    compact_windows<T><<<grid, SIEVE_THREADS, 0, st>>>(lo_odd, (uint32_t)nwin, ws->d_bits, ws->d_offsets, d_out,
                                                       capacity, out_base);
    CUDA_TRY(cudaGetLastError());
    note_kernel_launch();
    CUDA_TRY(cudaMemcpyAsync(ws->h_total, ws->d_offsets + nwin, sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    *count = *ws->h_total;
    return CTD_OK;
}

// make sure base primes cover every odd p <= limit
static int ensure_base(SieveWorkspace *ws, uint64_t limit, cudaStream_t st, std::string &err)
{
    if (ws->base_limit >= limit && ws->d_base)
        return CTD_OK;
    if (!ws->d_base) {
        ws->base_cap = 8192;
        CUDA_TRY(cudaMalloc(&ws->d_base, ws->base_cap * sizeof(uint32_t)));
        uint32_t *d_cnt = nullptr;
        CUDA_TRY(cudaMalloc(&d_cnt, sizeof(uint32_t)));
        level0_primes<<<1, 1024, 0, st>>>(ws->d_base, d_cnt);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) {
            note_kernel_launch();
            uint32_t n = 0;
            e = cudaMemcpyAsync(&n, d_cnt, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess)
                e = cudaStreamSynchronize(st);
            ws->nbase = n;
        }
        cudaFree(d_cnt);
        if (e != cudaSuccess) {
            err = std::string("level-0 sieve: ") + cudaGetErrorString(e);
            return CTD_ERR_CUDA;
        }
        ws->base_limit = LEVEL0_LIMIT - 1;
    }
    if (ws->base_limit >= limit)
        return CTD_OK;
    // extend: odd primes in (base_limit, new_limit] sieved with the level-0 primes
    uint64_t new_limit = limit;
    if (new_limit > 0xffffffffull)
        new_limit = 0xffffffffull;
    // round up generously so later ranges rarely need another extension
    uint64_t grow = ws->base_limit * 2;
    if (new_limit < grow)
        new_limit = grow < 0xffffffffull ? grow : 0xffffffffull;
    const uint64_t lo_odd = (ws->base_limit + 1) | 1;
    const uint64_t nodd = new_limit >= lo_odd ? (new_limit - lo_odd) / 2 + 1 : 0;
    const uint64_t need = ws->nbase + prime_count_upper_bound(lo_odd, new_limit + 1) + 64;
    if (need > ws->base_cap) {
        uint32_t *nb = nullptr;
        CUDA_TRY(cudaMalloc(&nb, need * sizeof(uint32_t)));
        CUDA_TRY(cudaMemcpyAsync(nb, ws->d_base, ws->nbase * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        cudaFree(ws->d_base);
        ws->d_base = nb;
        ws->base_cap = need;
    }
    // level-0 primes (p < 2^16) suffice for any new_limit < 2^32
    uint32_t nlevel0 = 0;
    {
        // the level-0 prefix: all primes below 2^16 are the first entries
        nlevel0 = ws->nbase;  // base_limit >= 2^16 - 1 holds the level-0 list at the front
        // only primes < 2^16 are needed; they are a prefix of d_base
        // (6541 odd primes below 2^16)
        if (nlevel0 > 6541)
            nlevel0 = 6541;
    }
    uint64_t cnt = 0;
    int rc = sieve_odd<uint32_t>(ws, lo_odd, nodd, ws->d_base, nlevel0, ws->d_base, ws->base_cap, ws->nbase, &cnt,
                                 st, err);
    if (rc)
        return rc;
    ws->nbase += (uint32_t)cnt;
    ws->base_limit = new_limit;
    return CTD_OK;
}

uint64_t prime_count_upper_bound(uint64_t lo, uint64_t hi)
{
    if (hi <= lo)
        return 0;
    const double y = (double)(hi - lo);
    double bound = y;  // trivial
    if (y >= 3) {
        // Montgomery-Vaughan: pi(x + y) - pi(x) <= 2y / ln y for y > 1
        bound = std::min(bound, 2.0 * y / std::log(y));
    }
    if (hi > 17) {
        // Rosser-Schoenfeld / Dusart: x/ln x <= pi(x) (x >= 17), pi(x) < 1.25506 x / ln x (x > 1)
        const double up = 1.25506 * (double)hi / std::log((double)hi);
        const double low = lo >= 17 ? (double)lo / std::log((double)lo) : 0.0;
        bound = std::min(bound, up - low);
    }
    return (uint64_t)bound + 64;
}

// ------------------------------------------------ launch-only variant
// For the batched engine: base primes and window scratch are prepared once,
// then each segment is three kernel launches with the prime count left in
// device memory -- no allocation and no host wait, so a whole schedule of
// segments can be captured in one CUDA graph.
int sieve_prepare_base(SieveWorkspace *ws, uint64_t hi, cudaStream_t st, std::string &err)
{
    if (hi < 3)
        return CTD_OK;
    return ensure_base(ws, isqrt64(hi - 1), st, err);
}

int sieve_prepare_windows(SieveWorkspace *ws, uint64_t max_width, std::string &err)
{
    const uint64_t nwin = (max_width / 2 + 1 + WIN_ODD - 1) / WIN_ODD + 1;
    int rc = ensure_windows(ws, nwin, err);
    if (rc)
        return rc;
    const size_t smem = WIN_WORDS * sizeof(uint32_t);
    CUDA_TRY(cudaFuncSetAttribute(sieve_windows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    return CTD_OK;
}

uint64_t sieve_state_key(const SieveWorkspace *ws)
{
    // FNV-1a over what sieve_odd_async's launches take besides the range
    const uint64_t parts[] = {(uint64_t)(uintptr_t)ws->d_base, ws->nbase, (uint64_t)(uintptr_t)ws->d_bits,
                              (uint64_t)(uintptr_t)ws->d_wcount, (uint64_t)(uintptr_t)ws->d_offsets,
                              (uint64_t)ws->sm_count};
    uint64_t h = 1469598103934665603ull;
    for (uint64_t x : parts)
        for (int b = 0; b < 8; ++b) {
            h ^= (x >> (8 * b)) & 0xff;
            h *= 1099511628211ull;
        }
    return h;
}

int sieve_odd_async(SieveWorkspace *ws, uint64_t lo, uint64_t hi, uint64_t *d_out, uint64_t capacity,
                    const uint64_t **count_out, cudaStream_t st, std::string &err)
{
    const uint64_t lo_odd = lo < 3 ? 3 : (lo | 1);
    const uint64_t nodd = lo_odd < hi ? (hi - lo_odd + 1) / 2 : 0;
    const uint64_t nwin = nodd ? (nodd + WIN_ODD - 1) / WIN_ODD : 0;
    if (nwin > ws->win_cap || !ws->d_base) {
        err = "sieve scratch not prepared for this segment";
        return CTD_ERR_INVALID_ARGUMENT;
    }
    *count_out = ws->d_offsets + nwin;
    if (!nwin) {  // empty: a zero count
        CUDA_TRY(cudaMemsetAsync(ws->d_offsets, 0, sizeof(uint64_t), st));
        return CTD_OK;
    }
    const size_t smem = WIN_WORDS * sizeof(uint32_t);
    const int grid = grid_for(ws, nwin);
    sieve_windows<<<grid, SIEVE_THREADS, smem, st>>>(lo_odd, nodd, (uint32_t)nwin, ws->d_base, ws->nbase, ws->d_bits,
                                                    ws->d_wcount);
    CUDA_TRY(cudaGetLastError());
    scan_counts<<<1, 1024, 0, st>>>(ws->d_wcount, (uint32_t)nwin, ws->d_offsets);
    CUDA_TRY(cudaGetLastError());
    compact_windows<uint64_t><<<grid, SIEVE_THREADS, 0, st>>>(lo_odd, (uint32_t)nwin, ws->d_bits, ws->d_offsets,
                                                              d_out, capacity, 0);
    CUDA_TRY(cudaGetLastError());
    note_kernel_launch();
    note_kernel_launch();
    note_kernel_launch();
    return CTD_OK;
}

// ----------------------------------------------- fixed-scratch variant
// The same three-pass sieve over scratch the caller provides (no device
// allocation, no cached state): base primes are recomputed on every call
// into `sc.base`, whose unused tail is filled with 0xffffffff so the kernels'
// "p^2 beyond the window" test stops at the real list.
uint64_t sieve_scratch_windows(uint64_t lo, uint64_t hi)
{
    const uint64_t lo_odd = lo < 3 ? 3 : (lo | 1);
    if (lo_odd >= hi)
        return 0;
    const uint64_t nodd = (hi - lo_odd + 1) / 2;
    return (nodd + WIN_ODD - 1) / WIN_ODD;
}

uint64_t sieve_scratch_base_windows(uint64_t limit)
{
    return limit < LEVEL0_LIMIT ? 0 : (limit - LEVEL0_LIMIT) / (2 * WIN_ODD) + 1;
}

int sieve_range_scratch(const SieveScratch &sc, int sm_count, uint64_t lo, uint64_t hi, uint64_t *d_out,
                        uint64_t capacity, uint64_t *count, cudaStream_t st, std::string &err)
{
    *count = 0;
    if (hi <= lo)
        return CTD_OK;
    const size_t smem = WIN_WORDS * sizeof(uint32_t);
    CUDA_TRY(cudaFuncSetAttribute(sieve_windows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    uint64_t out_base = 0;
    if (lo <= 2 && hi > 2) {
        if (capacity > 0) {  // the u64 value 2, little-endian
            CUDA_TRY(cudaMemsetAsync(d_out, 0, sizeof(uint64_t), st));
            CUDA_TRY(cudaMemsetAsync(d_out, 2, 1, st));
        }
        out_base = 1;
    }
    const uint64_t lo_odd = lo < 3 ? 3 : (lo | 1);
    if (lo_odd >= hi) {
        *count = out_base;
        return CTD_OK;
    }
    // base primes: level 0 (odd p < 2^16), then (2^16, sqrt(hi)] from them
    const uint64_t limit = isqrt64(hi - 1);
    CUDA_TRY(cudaMemsetAsync(sc.base, 0xff, sc.base_cap * sizeof(uint32_t), st));
    level0_primes<<<1, 1024, 0, st>>>(sc.base, sc.level0_count);
    CUDA_TRY(cudaGetLastError());
    note_kernel_launch();
    const uint32_t nlevel0 = 6541;  // odd primes below 2^16
    const uint64_t bwin = sieve_scratch_base_windows(limit);
    if (bwin) {
        const uint64_t b_lo = LEVEL0_LIMIT + 1;
        const uint64_t b_nodd = (limit - b_lo) / 2 + 1;
        const int grid = (int)std::min<uint64_t>(bwin, (uint64_t)sm_count * 3);
        sieve_windows<<<grid, SIEVE_THREADS, smem, st>>>(b_lo, b_nodd, (uint32_t)bwin, sc.base, nlevel0, sc.bits,
                                                         sc.wcount);
        CUDA_TRY(cudaGetLastError());
        scan_counts<<<1, 1024, 0, st>>>(sc.wcount, (uint32_t)bwin, sc.offsets);
        CUDA_TRY(cudaGetLastError());
        compact_windows<uint32_t><<<grid, SIEVE_THREADS, 0, st>>>(b_lo, (uint32_t)bwin, sc.bits, sc.offsets, sc.base,
                                                                  sc.base_cap - 1, nlevel0);
        CUDA_TRY(cudaGetLastError());
        note_kernel_launch();
        note_kernel_launch();
        note_kernel_launch();
    }
    // the range itself, against every base prime (the sentinel tail stops the scan)
    const uint64_t nodd = (hi - lo_odd + 1) / 2;
    const uint64_t nwin = (nodd + WIN_ODD - 1) / WIN_ODD;
    const int grid = (int)std::min<uint64_t>(nwin, (uint64_t)sm_count * 3);
    sieve_windows<<<grid, SIEVE_THREADS, smem, st>>>(lo_odd, nodd, (uint32_t)nwin, sc.base, sc.base_cap, sc.bits,
                                                     sc.wcount);
    CUDA_TRY(cudaGetLastError());
    scan_counts<<<1, 1024, 0, st>>>(sc.wcount, (uint32_t)nwin, sc.offsets);
    CUDA_TRY(cudaGetLastError());
    compact_windows<uint64_t><<<grid, SIEVE_THREADS, 0, st>>>(lo_odd, (uint32_t)nwin, sc.bits, sc.offsets, d_out,
                                                              capacity, out_base);
    CUDA_TRY(cudaGetLastError());
    note_kernel_launch();
    note_kernel_launch();
    note_kernel_launch();
    uint64_t total = 0;
    CUDA_TRY(cudaMemcpyAsync(&total, sc.offsets + nwin, sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    *count = out_base + total;
    return CTD_OK;
}

int sieve_range(SieveWorkspace *ws, uint64_t lo, uint64_t hi, uint64_t *d_out, uint64_t capacity, uint64_t *count,
                cudaStream_t st, std::string &err)
{
    *count = 0;
    if (hi <= lo)
        return CTD_OK;
    uint64_t total = 0;
    if (lo <= 2 && hi > 2) {
        if (capacity > 0) {
            const uint64_t two = 2;
            CUDA_TRY(cudaMemcpyAsync(d_out, &two, sizeof(two), cudaMemcpyHostToDevice, st));
            CUDA_TRY(cudaStreamSynchronize(st));
        }
        total = 1;
    }
    const uint64_t lo_odd = lo < 3 ? 3 : (lo | 1);
    if (lo_odd < hi) {
        const uint64_t nodd = (hi - lo_odd + 1) / 2;
        const uint64_t limit = isqrt64(hi - 1);
        int rc = ensure_base(ws, limit, st, err);
        if (rc)
            return rc;
        // base primes p with p <= limit: count them on the host side once
        // (the list is ascending; the kernels stop at p^2 >= window end)
        uint64_t cnt = 0;
        rc = sieve_odd<uint64_t>(ws, lo_odd, nodd, ws->d_base, ws->nbase, d_out, capacity, total, &cnt, st, err);
        if (rc)
            return rc;
        total += cnt;
    }
    *count = total;
    return CTD_OK;
}

}  // namespace ctd
