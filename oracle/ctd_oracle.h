/*
 * ctd_oracle.h -- CPU restatement of cutrialdive's trial-factoring hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker for the CUDA
 * path and the timed CPU baseline; the product (libctd_gpu.so and the
 * cutrialdive CLI) never links, loads or calls it.  Only tests/, the smoke
 * check in __graft_entry__.py and the cpu_baseline / reference legs of
 * bench.py use it.
 *
 * Parity pinning: every function below cites the reference file:line it
 * restates (paths relative to the cutrialdive project root).  The oracle is
 * checked against the reference's own golden vectors (tests/test_modular.cpp,
 * tests/<family>_tests.cpp, src/autotests.cpp) and against factor files produced by
 * the reference's own CPU engine built from its sources (oracle/build_ref.sh).
 */
#ifndef CTD_ORACLE_H
#define CTD_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Family ids: the numbering of num_seq_id (src/num_seq_id.hpp:16-26).
 * CTDO_PEANO is the reference's test-only sequence S(n) = n
 * (tests/peano.hpp:127-137); it has no --num-seq name. */
enum {
    CTDO_MERSENNE = 0,
    CTDO_PROTH = 1,
    CTDO_RIESEL = 2,
    CTDO_SMARANDACHE = 3,
    CTDO_FIBONACCI = 4,
    CTDO_LUCAS = 5,
    CTDO_PROTH_FIXED_N = 6,
    CTDO_RIESEL_FIXED_N = 7,
    CTDO_TRIBONACCI = 8,
    CTDO_PEANO = 256
};

/* ---- L1 modular arithmetic (src/modular_arithmetic_detail.hpp) ---- */
uint64_t ctdo_mu64(uint64_t p);
void ctdo_mu128(uint64_t p, uint64_t out_hi_lo[2]);
void ctdo_mul128hi(const uint64_t a_hi_lo[2], const uint64_t b_hi_lo[2], uint64_t out_hi_lo[2]);
uint64_t ctdo_mulmod(uint64_t a, uint64_t b, uint64_t d);
uint64_t ctdo_modpow(uint64_t a, uint64_t e, uint64_t d);
uint64_t ctdo_reciprocal(uint64_t d_normalized);
uint64_t ctdo_mod2by1(uint64_t u1, uint64_t u0, uint64_t d, uint64_t rnd);
uint64_t ctdo_modnby1(const uint64_t *limbs, uint64_t nlimbs, uint64_t d);

/* ---- prime generation: primes in [lo, hi), ascending ----
 * Restates the contract the engine gets from its siever with >= 2 threads
 * (src/siever.hpp:179-237).  Returns the number of primes; writes at most
 * `cap` of them to `out` (out may be NULL to count only). */
uint64_t ctdo_sieve(uint64_t lo, uint64_t hi, uint64_t *out, uint64_t cap);

/* ---- sequence plugins (src/number_sequences/) ---- */
typedef struct ctdo_state {
    uint64_t r;      /* S(n) mod p: the residue the engine propagates */
    uint64_t s[3];   /* per-family state (make_state) */
} ctdo_state;

/* 0 if (family, param) is accepted by the reference's dispatch
 * (src/num_seq_dispatch.hpp:120-170 and the plugin constructors), else -1. */
int ctdo_check_seq(uint32_t family, uint64_t param);
uint64_t ctdo_value_mod_2(uint32_t family, uint64_t param, uint64_t n);
uint64_t ctdo_next_value_mod_2(uint32_t family, uint64_t param, uint64_t r, uint64_t n);
/* Residue and state at index n0 for odd prime p.  For Smarandache `sm_limbs`
 * holds Sm_b(n0) (little-endian u64 limbs) and is reduced like the
 * reference's InitializeFromValue path; other families ignore it. */
void ctdo_init(uint32_t family, uint64_t param, uint64_t n0, uint64_t p,
               const uint64_t *sm_limbs, uint64_t sm_nlimbs, ctdo_state *st);
/* One propagation step: S(n) mod p -> S(n+1) mod p. */
void ctdo_step(uint32_t family, uint64_t param, uint64_t n, uint64_t p, ctdo_state *st);

/* Sm_b(n) as little-endian u64 limbs, built from its definition (the
 * concatenation of 1..n in base b, tests/smarandache_tests.cpp:22-35).
 * Returns the limb count; writes at most `cap` limbs (out may be NULL). */
uint64_t ctdo_smarandache_limbs(uint64_t base, uint64_t n, uint64_t *out, uint64_t cap);

/* ---- engine: restates host_trial_factor (src/trial_factoring_impl.hpp:278-366)
 * and trial_factorer::process_chunk (:193-248) ----
 * counts[n1-n0] / factors[(n1-n0)*max_factors] use the factors_buffer layout
 * (src/factors_buffer.hpp:77-86); they hold the resume state on entry (zeros
 * for a fresh job).  Primes p <= resume_after_prime are skipped.
 * Returns 0, or -1 for an invalid sequence / range. */
typedef struct ctdo_job {
    uint32_t family;
    uint32_t max_factors;
    uint64_t param;
    uint64_t n0, n1;
    uint64_t f0, f1;
} ctdo_job;

int ctdo_trial_factor(const ctdo_job *job, uint32_t *counts, uint64_t *factors,
                      uint64_t resume_after_prime, uint64_t segment_length, int threads);

/* Same loop over an explicit prime list (odd primes only), no sieve and no
 * mod-2 pass: the unit the GPU residue kernel implements. */
int ctdo_residues(const ctdo_job *job, const uint64_t *primes, uint64_t nprimes,
                  uint32_t *counts, uint64_t *factors, int threads);

#ifdef __cplusplus
}
#endif
#endif
