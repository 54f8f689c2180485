// ctd_internal.h -- internal C++ interface between the C-ABI layer
// (ctd_engine.cu), the device sieve (ctd_sieve.cu) and the residue kernels
// (ctd_residue.cu).  Not installed; the public boundary is include/ctd_gpu.h.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "../../include/ctd_gpu.h"

namespace ctd {

// Family ids: the numbering of the reference's num_seq_id
// (src/num_seq_id.hpp:16-26); PEANO is its test-only S(n) = n sequence
// (tests/peano.hpp:127-137).
enum Family : uint32_t {
    MERSENNE = CTD_MERSENNE,
    PROTH = CTD_PROTH,
    RIESEL = CTD_RIESEL,
    SMARANDACHE = CTD_SMARANDACHE,
    FIBONACCI = CTD_FIBONACCI,
    LUCAS = CTD_LUCAS,
    PROTH_FIXED_N = CTD_PROTH_FIXED_N,
    RIESEL_FIXED_N = CTD_RIESEL_FIXED_N,
    TRIBONACCI = CTD_TRIBONACCI,
    PEANO = CTD_PEANO,
};

// Device view of one job's factors buffer, in the reference layout
// (src/factors_buffer.hpp:77-86): counts[N], factors[N * max_factors],
// slot order = arrival order.
struct FactorsView {
    uint32_t *counts;
    uint64_t *factors;
    uint32_t max_factors;
};

// What a residue launch needs to know about its job.
struct JobView {
    uint32_t family;
    uint32_t tiles;      // index tiles per prime (>= 1)
    uint32_t variant;    // step form (CTD_VARIANT_*)
    uint32_t classify_min;  // doubling families: index ranges this long or longer walk power-residue classes
    uint32_t refine_q;   // largest rare prime whose character refines the classes (0: 61; < 11: none)
    uint32_t pad;
    uint64_t param;      // k, n or base
    uint64_t n0, n1;     // index range of the factors buffer
    uint64_t tile_len;   // indices per tile (last tile may be shorter)
    FactorsView fb;
};

// Status word written by kernels that can fail on the device (bounded
// waits, capacity checks); 0 = ok.
struct DeviceStatus {
    uint32_t code;
    uint32_t detail;
};

// ---------------------------------------------------------------- sieve
// Primes in [lo, hi) (ascending) written to d_out; *count receives the
// number of primes (the list is truncated at `capacity`).  Scratch is the
// sieve's own (SieveWorkspace); all work is queued on `stream`, which is
// synchronized once to read the count.
struct SieveWorkspace;
SieveWorkspace *sieve_workspace_create();
void sieve_workspace_destroy(SieveWorkspace *ws);
int sieve_range(SieveWorkspace *ws, uint64_t lo, uint64_t hi, uint64_t *d_out, uint64_t capacity,
                uint64_t *count, cudaStream_t stream, std::string &err);
// Upper bound on the number of primes in [lo, hi) (for buffer sizing).
uint64_t prime_count_upper_bound(uint64_t lo, uint64_t hi);

// Geometry of a sieve window: 16384 words of 32 odd numbers (a 2^20-wide range).
constexpr uint64_t SIEVE_WIN_WORDS = 16384;
constexpr uint64_t SIEVE_WIN_RANGE = 2 * 32 * SIEVE_WIN_WORDS;
constexpr uint32_t SIEVE_LEVEL0_ODD_PRIMES = 6541;  // odd primes below 2^16

// Scratch for the fixed-scratch sieve (sieve_range_scratch): device pointers
// the caller owns; bits/wcount/offsets hold `max_windows` windows.
struct SieveScratch {
    uint32_t *bits;
    uint32_t *wcount;
    uint64_t *offsets;
    uint32_t *base;
    uint64_t base_cap;
    uint32_t *level0_count;
    uint64_t max_windows;
};
// Windows the fixed-scratch sieve needs for [lo, hi), and for the base primes
// up to `limit` above 2^16.
uint64_t sieve_scratch_windows(uint64_t lo, uint64_t hi);
uint64_t sieve_scratch_base_windows(uint64_t limit);
// Primes in [lo, hi) using only `sc` as scratch: no allocation, no state
// kept between calls (base primes recomputed).  Synchronizes `stream` once
// to read the count.
int sieve_range_scratch(const SieveScratch &sc, int sm_count, uint64_t lo, uint64_t hi, uint64_t *d_out,
                        uint64_t capacity, uint64_t *count, cudaStream_t stream, std::string &err);
// Looks up the allocation-free sieve's static scratch on `device` (the
// current device), which places it there; called when a context opens.
int noalloc_prepare(int device, std::string &err);

// -------------------------------------------------------------- residues
// Scratch of the classified doubling launches (Proth, Riesel, Mersenne over
// long index ranges): per prime its power-residue class, then the primes
// regrouped by class so a warp's lanes walk classes of equal length.  Owned
// by a context; grown on demand (never during a graph capture).
// classes: the divisors of 2^3 * 3 * 5 * 7, ranked by size
// classes ranked by M: the 32 divisors of 840, then M above 840 by half
// octaves (M < 2^16)
constexpr uint32_t CLASS_BUCKETS = 48;
struct ClassCounters {
    uint32_t count[CLASS_BUCKETS];  // primes per class
    uint32_t fill[CLASS_BUCKETS];   // regroup cursors
    unsigned long long next;        // walk work counter
    uint32_t nrefine;               // primes listed for the rare-prime refinement
    uint32_t nlisted[8];            // primes the screen left for classification, by divisibility pattern
    uint32_t wide;                  // a prime of the launch is 2^40 or above
    uint32_t nnine;                 // primes listed for the 9th-power character
};
// a prime with its class code (M << 16 | r)
struct ClassItem {
    uint64_t p;
    uint32_t code;
    uint32_t pad;
};
struct ResidueScratch {
    int device = 0;
    int sm_count = 1;
    uint32_t *codes = nullptr;
    ClassItem *items = nullptr;
    uint32_t *refine = nullptr;  // indices of the primes to refine
    uint8_t *refine_q = nullptr; // and their rare q
    uint32_t *listed = nullptr;  // indices of the primes to classify: 8 lists of cap, by pattern
    uint32_t *nine = nullptr;    // indices of the primes for the 9th-power character
    uint64_t cap = 0;  // primes
    ClassCounters *counters = nullptr;
};
ResidueScratch *residue_scratch_create(int device, int sm_count);
void residue_scratch_destroy(ResidueScratch *rs);
// default length from which the doubling families walk power-residue classes
constexpr uint32_t DEFAULT_CLASSIFY_MIN = 8192;
// Uploads the residue kernels' per-device tables (the trial-division primes
// of the Fibonacci/Lucas rank-of-apparition path) to `device`, the current
// device, once per process and device.
int prepare_residue_tables(int device, std::string &err);
// Odd primes only.  Launches the family's residue kernel over
// nprimes x view.tiles work items; with `scratch`, the doubling families'
// long ranges go through the classified launches (classify, regroup, walk).
int launch_residues(const JobView &view, const uint64_t *d_primes, uint64_t nprimes, int grid, int block,
                    cudaStream_t stream, std::string &err, ResidueScratch *scratch = nullptr);
// One job of a batched launch: its view (factors buffer, index range,
// tiles), its odd-prime range [f0, f1) and whether it walks power-residue
// classes (doubling families over long ranges).
// `cursor` is the job's progress on the device: each segment's bounds
// kernel moves it to the end of the job's part of the segment (the server
// may take a job's segments in rotated order, see ctd_batch.cu, so it
// records the last segment done, not a bound below which all are done).
struct BatchJob {
    JobView view;
    uint64_t f0, f1;
    uint64_t cursor;
    uint32_t classified;
    uint32_t pad;
};
// Per active job of a batched segment: its primes [pbeg, pend) in the
// segment's list, its offset in the class buffers, its (prime, tile) units
// and the exclusive prefix of warp items (entry nactive holds the totals).
struct BatchSpan {
    uint64_t pbeg, pend;
    uint64_t coff;
    uint64_t units;
    uint64_t warp_prefix;
};
// Walk groups of a batched segment, by the code and resources their walks
// need: the doubling families over power-residue classes and over every
// term (both with the target filter in shared memory), Smarandache (the
// multiply pipe) and the rest.  A segment's active list is group-major.
constexpr int BATCH_GROUPS = 4;
constexpr int BATCH_CLASSES = 0, BATCH_DOUBLING = 1, BATCH_MULTIPLY = 2, BATCH_OTHER = 3;
inline int batch_group(uint32_t family, bool classified)
{
    if (family == CTD_PROTH || family == CTD_RIESEL || family == CTD_MERSENNE)
        return classified ? BATCH_CLASSES : BATCH_DOUBLING;
    return family == CTD_SMARANDACHE ? BATCH_MULTIPLY : BATCH_OTHER;
}
struct BatchControl {
    uint64_t nclass;                        // (classified job, prime) pairs
    uint64_t total_warps[BATCH_GROUPS];     // warp items of each group's walk
    unsigned long long next[BATCH_GROUPS];  // the walks' work counters
    unsigned long long nlisted;             // pairs the quadratic screen left for classification
    unsigned long long nrefine;             // pairs listed for the rare-prime refinement
};
// Device scratch of one batched segment (sized by the caller):
// spans[nactive + 1], codes/items[class pairs], bucket_count[2 * nactive *
// CLASS_BUCKETS] (counts, then regroup cursors), bucket_base[nactive *
// CLASS_BUCKETS].  The screen's and the refinement's pair lists (8 bytes a
// pair each) live in the items buffer (16 bytes a pair), which holds nothing
// until the regroup that follows them.
struct BatchScratch {
    BatchSpan *spans;
    BatchControl *ctl;
    uint32_t *codes;
    ClassItem *items;
    uint64_t class_cap;  // pairs the codes and items buffers hold
    uint32_t *bucket_count;
    uint32_t *bucket_base;
};
// The kernels of one batched segment over the primes of [lo, hi) in
// d_primes (count read from *d_count on the device): bounds, classes (when
// any active job is classified), plan, regroup and one walk launch per walk
// group present; the active list d_active is group-major with gcount[g]
// jobs in group g.  Nothing waits on the host.  Each active job's device
// cursor moves to the end of its part of [lo, hi).
int launch_batch(BatchJob *d_jobs, const uint32_t *d_active, const uint32_t gcount[BATCH_GROUPS], bool any_classified,
                 const uint64_t *d_primes, const uint64_t *d_count, uint64_t lo, uint64_t hi,
                 const BatchScratch &bs, int sm_count, cudaStream_t stream, std::string &err);
// Odd primes of [lo, hi) into d_out without waiting on the host; the count
// is left at *count_out (device memory, owned by the workspace).  Base primes
// must already cover sqrt(hi) (sieve_prepare_base).
int sieve_prepare_base(SieveWorkspace *ws, uint64_t hi, cudaStream_t stream, std::string &err);
int sieve_prepare_windows(SieveWorkspace *ws, uint64_t max_width, std::string &err);
int sieve_odd_async(SieveWorkspace *ws, uint64_t lo, uint64_t hi, uint64_t *d_out, uint64_t capacity,
                    const uint64_t **count_out, cudaStream_t stream, std::string &err);
// Changes whenever sieve_odd_async's launches would take other arguments
// for the same range (base primes extended, scratch regrown): part of the
// key under which a captured schedule may be replayed.
uint64_t sieve_state_key(const SieveWorkspace *ws);

// Resident CTAs per SM of the family's residue kernel at `block` threads
// (0 if the query fails); the persistent grid is SMs x this.
int residue_blocks_per_sm(uint32_t family, int block);
// The prime 2: the reference's serial mod-2 pass (src/trial_factoring.cuh:139-154).
int launch_mod2(const JobView &view, cudaStream_t stream, std::string &err);
// Number of kernel launches issued by this process so far (diagnostics).
uint64_t kernel_launch_count();
void note_kernel_launch();
// counts n launches at once (the kernels of a replayed graph)
void note_kernel_launches(uint64_t n);

// Device buffers and the captured schedule of ctd_batch_run, kept by a
// context across calls (ctd_batch.cu).
struct BatchCache;
void batch_cache_destroy(BatchCache *bc);

// Context accessors for entry points defined outside ctd_engine.cu.
int ctx_device(const ctd_ctx *ctx);
int ctx_sm_count(const ctd_ctx *ctx);
cudaStream_t ctx_stream(const ctd_ctx *ctx);
SieveWorkspace *ctx_workspace(const ctd_ctx *ctx);
BatchCache *&ctx_batch_cache(ctd_ctx *ctx);
// the launch/tiling parameters in force for a family at primes of
// first_prime's width (defaults when untuned)
ctd_tuning ctx_tuning(ctd_ctx *ctx, uint32_t family, uint64_t first_prime);
int ctx_fail(ctd_ctx *ctx, int code, const std::string &msg);

}  // namespace ctd
