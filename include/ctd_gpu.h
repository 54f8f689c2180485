/*
 * ctd_gpu.h -- C ABI of libctd_gpu.so, the GB300 (sm_103a) trial-factoring
 * engine for recurrence-defined integer sequences.
 *
 * Plain pointers and sizes only; no C++ or CUDA types cross this boundary
 * (streams are passed as opaque `void *`, 0 meaning the context's own
 * stream).  Every call returns an int status: CTD_OK (0) or a negative
 * CTD_ERR_* code; ctd_last_error() gives the message of the last failure on
 * a context.  No call throws.
 *
 * Each entry point names the reference interface it replaces (paths within
 * the cutrialdive project).
 */
#ifndef CTD_GPU_H
#define CTD_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CTD_ABI_VERSION 1

/* ---- status codes ---- */
#define CTD_OK 0
#define CTD_ERR_INVALID_ARGUMENT (-1) /* bad job/range/pointer (reference: std::invalid_argument / runtime_error) */
#define CTD_ERR_CUDA (-2)             /* a CUDA runtime call failed */
#define CTD_ERR_OUT_OF_MEMORY (-3)    /* device allocation failed or a budget was exceeded */
#define CTD_ERR_ABORTED (-4)          /* a progress callback asked to stop */
#define CTD_ERR_TIMEOUT (-5)          /* a bounded device or host wait expired */
#define CTD_ERR_CAPACITY (-6)         /* an output buffer is too small */
#define CTD_ERR_NOT_FOUND (-7)        /* unknown job/request id */

/* ---- sequence families: the numbering of num_seq_id (src/num_seq_id.hpp:16-26),
 *      which the checkpoint file stores (src/checkpoint.cpp:186,213-216) ---- */
#define CTD_MERSENNE 0
#define CTD_PROTH 1
#define CTD_RIESEL 2
#define CTD_SMARANDACHE 3
#define CTD_FIBONACCI 4
#define CTD_LUCAS 5
#define CTD_PROTH_FIXED_N 6
#define CTD_RIESEL_FIXED_N 7
#define CTD_TRIBONACCI 8
/* S(n) = n, the reference's test-only sequence (tests/peano.hpp:127-137) */
#define CTD_PEANO 256

/*
 * One trial-factoring job: the terms S(n), n in [n0, n1), of `family`
 * (parameter `param`: k for proth/riesel, n for the fixed-n families, the
 * base 2..64 for smarandache, unused otherwise) by every prime p in
 * [f0, f1).  The device-side replacement of the template instantiation
 * trial_factor<Seq>(trial_factoring_context&&, args...)
 * (src/trial_factoring_impl.hpp:369-441) with its trial_factoring_options
 * (src/trial_factoring_options.hpp:15-31).
 */
typedef struct ctd_job {
    uint32_t family;
    uint32_t max_factors; /* factors stored per term (--max-factors-per-number, default 32) */
    uint64_t param;
    uint64_t n0, n1;
    uint64_t f0, f1;
} ctd_job;

/* Progress report after each completed prime segment. */
typedef struct ctd_progress {
    uint64_t segment_end;   /* upper bound fy of the segment just completed */
    uint64_t last_prime;    /* largest prime processed so far, 0 if none */
    uint64_t primes_done;   /* odd primes processed by this call so far */
    double elapsed_s;       /* wall time since the call started */
} ctd_progress;

/* Return values of a progress callback. */
#define CTD_CB_CONTINUE 0
#define CTD_CB_SNAPSHOT 1 /* copy the factors buffer into the caller's arrays, then call back with snapshot=1 */
#define CTD_CB_ABORT 2

/* Called on the calling thread between segments (never while a kernel of
 * this call runs).  With snapshot=1 the caller's counts/factors arrays hold
 * the state after `prog->last_prime`: what the reference checkpoints
 * (src/trial_factoring.cuh:453-465). */
typedef int (*ctd_progress_cb)(void *user, const ctd_progress *prog, int snapshot);

typedef struct ctd_ctx ctd_ctx;

/* ---- library ---- */
int ctd_abi_version(void);
const char *ctd_strerror(int status);
/* Number of kernels this process has launched through the library. */
uint64_t ctd_kernel_launches(void);

/* Opens a context on `device`.  Replaces cudaSetDevice + device property and
 * occupancy queries of device_trial_factor (src/trial_factoring.cuh:342-380). */
int ctd_open(int device, ctd_ctx **out);
void ctd_close(ctd_ctx *ctx);
const char *ctd_last_error(const ctd_ctx *ctx);
/* Device name / memory / SM count (src/trial_factoring.cuh:241-252). */
int ctd_device_info(ctd_ctx *ctx, char *name, size_t name_len, uint64_t *total_mem, int *sm_count);
/* Override the residue kernel's launch shape (--grid-size / --block-size,
 * src/trial_factoring.cuh:280-286); 0 restores the default. */
int ctd_set_launch(ctd_ctx *ctx, int grid_size, int block_size);

/* Launch and tiling parameters of one family's residue kernel (the
 * reference derives grid and block from occupancy queries and picks a
 * divisor batch size by segment end, src/trial_factoring.cuh:275-331,472-481;
 * here they are measured per family by ctd_autotune). */
typedef struct ctd_tuning {
    int32_t block_size;        /* threads per CTA: 32..256, a multiple of 32 */
    int32_t ctas_per_sm;       /* CTAs per SM of the persistent grid; 0 = as many as fit */
    uint32_t items_per_thread; /* below this many (prime, tile) items per resident thread, index ranges are tiled */
    uint32_t min_tile;         /* shortest index tile (each tile starts with an O(log n) jump) */
    uint32_t segment_log2;     /* default prime-segment width of ctd_run_plain, log2; 0 = 26 */
    uint32_t variant;          /* step form, CTD_VARIANT_* (results never depend on it) */
    uint32_t classify_min;     /* Proth/Riesel/Mersenne: index ranges at least this long walk only the
                                  power-residue class of their zeros; 0 = 8192 */
    uint32_t refine_q;         /* power-residue classes: the largest prime q (11..127) whose q-th power character
                                  narrows them for the primes p with q | p - 1; 0 = 127, below 11 = none
                                  (the 9th-power character too) */
} ctd_tuning;

/* Step forms a tuning can select.  AUTO: the fastest measured form for the
 * family and prime width.  WALK: the term-by-term walk (doubling families:
 * no baby-step blocks and no power-residue classes; fixed-n families: the
 * walk instead of the closed-form solve; Fibonacci/Lucas: no rank of
 * apparition; Smarandache: the 64-bit Shoup step instead of the 32-bit
 * Barrett step).  MONTGOMERY: Smarandache steps in Montgomery form (the
 * general path).  Families without such a choice ignore it. */
#define CTD_VARIANT_AUTO 0
#define CTD_VARIANT_WALK 1
#define CTD_VARIANT_MONTGOMERY 2

/* The parameters in force for `family` (defaults until tuned or set). */
int ctd_get_tuning(ctd_ctx *ctx, uint32_t family, ctd_tuning *out);
/* Sets them for every prime width; NULL restores the defaults.
 * ctd_set_launch overrides still win. */
int ctd_set_tuning(ctd_ctx *ctx, uint32_t family, const ctd_tuning *t);
/* The same keyed by prime width: the parameters in force for primes of
 * `prime_bits` bits (1..64; 0 = the family entry).  A width entry wins over
 * the family entry for segments whose first prime has that width; NULL
 * clears it. */
int ctd_get_tuning_for(ctd_ctx *ctx, uint32_t family, uint32_t prime_bits, ctd_tuning *out);
int ctd_set_tuning_for(ctd_ctx *ctx, uint32_t family, uint32_t prime_bits, const ctd_tuning *t);
/* Autotuner: times candidate launch shapes, tilings, step forms, power-residue
 * classes on or off (doubling families) and the segment length (2^26, 2^28,
 * 2^30) of the job's family on the job's own first prime segment (its index
 * range, a sample of its primes) for about `budget_s` seconds, keeps the
 * fastest in the context for that family at the width of the job's first
 * prime -- ctd_run_plain, ctd_residues_device, ctd_batch_run and the server
 * use it there -- and returns it in *best.  Results never depend on the
 * tuning, only the speed. */
int ctd_autotune(ctd_ctx *ctx, const ctd_job *job, double budget_s, ctd_tuning *best);

/* Validates a job like the reference's dispatch and range checks
 * (src/num_seq_dispatch.hpp:120-170, src/trial_factoring_impl.hpp:380-387):
 * CTD_OK, or CTD_ERR_INVALID_ARGUMENT. */
int ctd_check_job(const ctd_job *job);

/*
 * Runs one job end to end on the device: the prime 2, then odd primes
 * segment by segment (device sieve -> residue kernel), results merged into
 * the caller-owned host factors buffer.  Replaces device_trial_factor
 * (src/trial_factoring.cuh:334-513) and the kernels it launches
 * (trial_div_by_2 :139-154, trial_div_by_odd_primes :156-228), including the
 * host siever and its H2D prime copy (src/siever.hpp:179-237,
 * src/prime_data.hpp:166-196).
 *
 * counts_inout[n1-n0] and factors_inout[(n1-n0)*max_factors] use the
 * reference factors_buffer layout (src/factors_buffer.hpp:77-86); on entry
 * they hold the resume state (zeros for a fresh job; slots past a term's
 * count must be zero), on return the result (slot order is arrival order:
 * sort per term before printing, as src/factors_buffer.hpp:123-138 does).
 * A term with more prime factors in range than max_factors keeps the
 * max_factors smallest and its count exceeds max_factors: the CPU engine's
 * result; the reference's device push keeps whichever arrive first and both
 * report the excess (src/factors_buffer.hpp:62-75).  Primes p <= resume_after_prime are
 * skipped (src/trial_factoring.cuh:404).  segment_length 0 = the tuned
 * length for the job's family and first prime width (2^26 untuned).  Across
 * the host link the call moves only what it must: an all-zero resume state
 * is cleared on the device instead of uploaded, and the counts come back
 * with the occupied slots only (the host slots past a count stay zero).
 */
int ctd_run_plain(ctd_ctx *ctx, const ctd_job *job, uint32_t *counts_inout, uint64_t *factors_inout,
                  uint64_t resume_after_prime, uint64_t segment_length, ctd_progress_cb cb, void *user);

/*
 * Primes in [lo, hi), ascending, from the device sieve, into a host array.
 * *count receives the number of primes in the range; if it exceeds
 * `capacity` the array holds the first `capacity` and CTD_ERR_CAPACITY is
 * returned.  Replaces siever_impl::sieve (src/siever.hpp:179-237, primes in
 * [start, end)).
 */
int ctd_sieve(ctd_ctx *ctx, uint64_t lo, uint64_t hi, uint64_t *out, uint64_t capacity, uint64_t *count);

/* ---- device-resident forms (inputs and outputs in device memory) ---- */

/* ctd_sieve into device memory, queued on `stream`. */
int ctd_sieve_device(ctd_ctx *ctx, uint64_t lo, uint64_t hi, uint64_t *d_out, uint64_t capacity,
                     uint64_t *count, void *stream);

/* The residue kernel over an explicit list of odd primes in device memory,
 * pushing hits into a device factors buffer (slots past a term's count
 * zero, as for ctd_run_plain).  The unit that
 * trial_div_by_odd_primes<Seq, 1, ...> implements (src/trial_factoring.cuh:156-228).
 * Asynchronous on `stream`; the launches use the context's scratch (work
 * counter, class buffers), so calls on one context must not overlap on
 * different streams.  The class buffers of the Proth, Riesel and Mersenne
 * launches (about 61 bytes per prime of the largest list, kept by the
 * context) are allocated on first need; where the device cannot give them,
 * the call walks every term instead, with the same results. */
int ctd_residues_device(ctd_ctx *ctx, const ctd_job *job, const uint64_t *d_primes, uint64_t nprimes,
                        uint32_t *d_counts, uint64_t *d_factors, void *stream);

/* The prime-2 pass into a device factors buffer (src/trial_factoring.cuh:139-154). */
int ctd_mod2_device(ctd_ctx *ctx, const ctd_job *job, uint32_t *d_counts, uint64_t *d_factors, void *stream);

/* ---- many jobs ----
 * No counterpart in the reference (one job per process there,
 * src/main.cpp:94-146); built from the same per-job semantics as
 * ctd_run_plain, so each job's factors buffer comes out exactly as a
 * ctd_run_plain of that job alone would leave it (slot order aside). */

/* Runs `njobs` jobs together: the union of their prime ranges is walked in
 * aligned segments of `segment_length` (0 = 2^30); each segment is sieved
 * once on the device and consumed by every job covering it in one
 * persistent walk launch over (job, 32 primes, index tile) work items of
 * all families.  With use_graph != 0 the whole schedule is captured into a
 * CUDA graph and launched once; the context keeps the instantiated graph
 * and its device buffers, so a later call with the same schedule replays it
 * and one with the same shape updates it in place (ctd_batch_graph_stats
 * counts each).  counts_inout[i] / factors_inout[i] are job i's host
 * factors buffers (resume state in, results out). */
int ctd_batch_run(ctd_ctx *ctx, const ctd_job *jobs, uint32_t njobs, uint32_t *const *counts_inout,
                  uint64_t *const *factors_inout, uint64_t segment_length, int use_graph);
/* Graphs instantiated, updated in place and replayed by ctd_batch_run on this context. */
int ctd_batch_graph_stats(ctd_ctx *ctx, uint64_t *instantiations, uint64_t *updates, uint64_t *replays);

/* Continuous-batching server.  Submitted jobs queue; each ctd_serve_tick
 * collects the jobs whose results have arrived on the host, admits queued
 * jobs (arrival order) while fewer than max_active run and their device
 * buffers fit memory_budget (a job larger than the budget runs alone), and
 * queues one more tick of work without waiting for the previous ticks (at
 * most two ahead of the GPU): every running job advances over its next
 * aligned prime segment, jobs in the same segment sharing its sieve and one
 * walk launch.  Progress cursors live in the server's device job table and
 * are moved by the kernels.  ctd_serve_fetch returns (and releases) a
 * finished job's factors buffer. */
typedef struct ctd_server ctd_server;
int ctd_serve_open(ctd_ctx *ctx, uint64_t memory_budget, uint32_t max_active, uint64_t segment_length,
                   ctd_server **out);
void ctd_serve_close(ctd_server *srv);
int ctd_serve_submit(ctd_server *srv, const ctd_job *job, uint64_t *id);
int ctd_serve_tick(ctd_server *srv, uint64_t *done_ids, uint32_t cap, uint32_t *ndone);
int ctd_serve_fetch(ctd_server *srv, uint64_t id, uint32_t *counts, uint64_t *factors);
int ctd_serve_status(ctd_server *srv, uint32_t *active, uint32_t *queued, uint64_t *memory_used);

/* ---- allocation-free device sieve ----
 * No counterpart in the reference.  For callers that may not allocate device
 * memory -- a process that reserves its whole memory budget at start-up and
 * admits work against it, or a host whose pool allocator owns all GPU
 * memory -- this is ctd_sieve_device without any cudaMalloc/cudaFree: its
 * scratch is a fixed array of about 8.6 MiB compiled into the library.
 * ctd_open places it on the context's device (it looks up the array's
 * address, which loads it even under CUDA's lazy module loading), and it
 * stays there until the process exits: reserve device memory after
 * ctd_open, not before.  Limits:
 * hi - lo <= CTD_NOALLOC_SIEVE_MAX_RANGE and hi <= CTD_NOALLOC_SIEVE_MAX_HI;
 * larger requests return CTD_ERR_INVALID_ARGUMENT (message in
 * ctd_last_error).  Output as ctd_sieve_device: primes in [lo, hi) ascending
 * in the caller's d_out, *count the number of primes (synchronizes the
 * stream to read it).  Calls only read the address ctd_open looked up, so
 * none of them does set-up work.  All calls
 * share the array: calls that overlap on the GPU (concurrent streams or
 * threads) race and must be serialized by the caller. */
#define CTD_NOALLOC_SIEVE_MAX_RANGE (1ull << 26)
#define CTD_NOALLOC_SIEVE_MAX_HI (1ull << 48)
int ctd_sieve_device_noalloc(ctd_ctx *ctx, uint64_t lo, uint64_t hi, uint64_t *d_out, uint64_t capacity,
                             uint64_t *count, void *stream);

#ifdef __cplusplus
}
#endif
#endif
