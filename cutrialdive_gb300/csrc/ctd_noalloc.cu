// ctd_noalloc.cu -- the device sieve for callers that cannot allocate.
//
// Some callers of this library may not call cudaMalloc at all: a serving
// process that reserves its whole device-memory budget at start-up and
// admits work against that fixed budget (a hidden allocation would break its
// accounting or fail under memory pressure), or a host application whose
// GPU memory is owned by its own pool allocator and which forbids libraries
// from allocating behind its back.  ctd_sieve_device (ctd_engine.cu) grows
// its scratch with cudaMalloc as ranges grow; ctd_sieve_device_noalloc below
// runs the same kernels over a fixed scratch area that lives in this file as
// a static __device__ array, so it never allocates device memory.
//
// Limits: hi - lo <= CTD_NOALLOC_SIEVE_MAX_RANGE (2^26) and
// hi <= CTD_NOALLOC_SIEVE_MAX_HI (2^48, so every base prime is below 2^24).
// The array (about 8.6 MiB) is placed on a GPU when a context opens on it
// (ctd_open looks up its address) and stays there until the process exits.
// Every call uses the same array and it keeps the previous call's contents;
// each call rewrites everything it reads, and calls that overlap on the GPU
// (different streams or threads at the same time) race on it.
#include "ctd_internal.h"

#include <mutex>

namespace ctd {
namespace {

constexpr uint64_t MAX_RANGE = CTD_NOALLOC_SIEVE_MAX_RANGE;
constexpr uint64_t MAX_HI = CTD_NOALLOC_SIEVE_MAX_HI;
// windows of the range itself (+1 when the range straddles a window edge)
// and of the base primes in (2^16, 2^24]
constexpr uint64_t RANGE_WINDOWS = MAX_RANGE / SIEVE_WIN_RANGE + 1;
constexpr uint64_t BASE_WINDOWS = ((1ull << 24) - 65536) / SIEVE_WIN_RANGE + 1;
constexpr uint64_t WINDOWS = RANGE_WINDOWS > BASE_WINDOWS ? RANGE_WINDOWS : BASE_WINDOWS;
constexpr uint64_t BASE_CAP = 1100000;  // pi(2^24) = 1077871

constexpr uint64_t align256(uint64_t x) { return (x + 255) & ~uint64_t{255}; }
constexpr uint64_t OFF_BITS = 0;
constexpr uint64_t OFF_WCOUNT = align256(OFF_BITS + WINDOWS * SIEVE_WIN_WORDS * 4);
constexpr uint64_t OFF_OFFSETS = align256(OFF_WCOUNT + WINDOWS * 4);
constexpr uint64_t OFF_BASE = align256(OFF_OFFSETS + (WINDOWS + 1) * 8);
constexpr uint64_t OFF_LEVEL0 = align256(OFF_BASE + BASE_CAP * 4);
constexpr uint64_t SCRATCH_BYTES = align256(OFF_LEVEL0 + 4);

// the scratch; host code only ever uses its device address from
// cudaGetSymbolAddress (the name itself is a host-side stand-in)
static __device__ __align__(256) unsigned char g_sieve_scratch[SCRATCH_BYTES];

constexpr int MAX_DEVICES = 64;
std::mutex g_setup_mutex;
unsigned char *g_scratch_addr[MAX_DEVICES] = {};

// once per device, with that device current: the array's device address
int scratch_for_device(int device, unsigned char **addr, std::string &err)
{
    if (device < 0 || device >= MAX_DEVICES) {
        err = "device index out of range";
        return CTD_ERR_INVALID_ARGUMENT;
    }
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[device]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_sieve_scratch);
        if (e != cudaSuccess || !p) {
            err = std::string("cudaGetSymbolAddress(sieve scratch): ") + cudaGetErrorString(e);
            return CTD_ERR_CUDA;
        }
        g_scratch_addr[device] = static_cast<unsigned char *>(p);
    }
    *addr = g_scratch_addr[device];
    return CTD_OK;
}

}  // namespace

// Called by ctd_open on its device: the lookup loads this file's module,
// and with it the array, onto the device when the context opens.  Under
// CUDA's lazy module loading the array would otherwise arrive with the
// first allocation-free call -- possibly after the caller has reserved all
// of the device's memory for itself.
int noalloc_prepare(int device, std::string &err)
{
    unsigned char *addr = nullptr;
    return scratch_for_device(device, &addr, err);
}

}  // namespace ctd

using namespace ctd;

extern "C" int ctd_sieve_device_noalloc(ctd_ctx *ctx, uint64_t lo, uint64_t hi, uint64_t *d_out, uint64_t capacity,
                                        uint64_t *count, void *stream)
{
    if (!ctx || !count || (capacity && !d_out))
        return ctx ? ctx_fail(ctx, CTD_ERR_INVALID_ARGUMENT, "ctd_sieve_device_noalloc: bad arguments")
                   : CTD_ERR_INVALID_ARGUMENT;
    *count = 0;
    if (hi > lo && hi - lo > MAX_RANGE)
        return ctx_fail(ctx, CTD_ERR_INVALID_ARGUMENT,
                        "ctd_sieve_device_noalloc: range wider than CTD_NOALLOC_SIEVE_MAX_RANGE (2^26)");
    if (hi > MAX_HI)
        return ctx_fail(ctx, CTD_ERR_INVALID_ARGUMENT,
                        "ctd_sieve_device_noalloc: upper bound above CTD_NOALLOC_SIEVE_MAX_HI (2^48)");
    const int device = ctx_device(ctx);
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess)
        return ctx_fail(ctx, CTD_ERR_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
    std::string err;
    unsigned char *base = nullptr;
    int rc = scratch_for_device(device, &base, err);
    if (rc)
        return ctx_fail(ctx, rc, err);
    SieveScratch sc;
    sc.bits = reinterpret_cast<uint32_t *>(base + OFF_BITS);
    sc.wcount = reinterpret_cast<uint32_t *>(base + OFF_WCOUNT);
    sc.offsets = reinterpret_cast<uint64_t *>(base + OFF_OFFSETS);
    sc.base = reinterpret_cast<uint32_t *>(base + OFF_BASE);
    sc.base_cap = BASE_CAP;
    sc.level0_count = reinterpret_cast<uint32_t *>(base + OFF_LEVEL0);
    sc.max_windows = WINDOWS;
    if (sieve_scratch_windows(lo, hi) > WINDOWS)
        return ctx_fail(ctx, CTD_ERR_INVALID_ARGUMENT, "ctd_sieve_device_noalloc: range needs too many windows");
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx_stream(ctx);
    rc = sieve_range_scratch(sc, ctx_sm_count(ctx), lo, hi, d_out, capacity, count, st, err);
    if (rc)
        return ctx_fail(ctx, rc, err);
    if (*count > capacity)
        return ctx_fail(ctx, CTD_ERR_CAPACITY, "ctd_sieve_device_noalloc: output capacity too small");
    return CTD_OK;
}
