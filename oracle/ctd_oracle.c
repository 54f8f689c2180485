/*
 * ctd_oracle.c -- CPU restatement of cutrialdive's trial-factoring hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see ctd_oracle.h).  The product never links this
 * file; it is the checker the CUDA path is compared with and the timed CPU
 * baseline.  Each function cites the reference file:line it restates; paths
 * are relative to the cutrialdive project root.
 */
#include "ctd_oracle.h"

#include <pthread.h>
#include <stdlib.h>
#include <string.h>

typedef unsigned __int128 u128;

/* ======================================================================
 * L1 modular arithmetic -- src/modular_arithmetic_detail.hpp
 * ====================================================================== */

/* mu64 = floor((2^64 - 1) / p)  (modular_arithmetic_detail.hpp:249-253) */
uint64_t ctdo_mu64(uint64_t p) { return UINT64_MAX / p; }

/* mu128 = floor((2^128 - 1) / p)  (modular_arithmetic_detail.hpp:255-259) */
static u128 mu128(uint64_t p) { return (~(u128)0) / p; }

void ctdo_mu128(uint64_t p, uint64_t out[2])
{
    u128 m = mu128(p);
    out[0] = (uint64_t)(m >> 64);
    out[1] = (uint64_t)m;
}

/* floor(a * b / 2^128) from 64-bit halves (modular_arithmetic_detail.hpp:266-289):
 * the low product only contributes its high half and its carries. */
static u128 mul128hi(u128 a, u128 b)
{
    uint64_t a0 = (uint64_t)a, a1 = (uint64_t)(a >> 64);
    uint64_t b0 = (uint64_t)b, b1 = (uint64_t)(b >> 64);
    u128 mid = ((u128)a0 * b0) >> 64;
    u128 lmid = mid + (u128)a0 * b1;
    unsigned carry = lmid < mid;
    mid = lmid + (u128)a1 * b0;
    carry = carry || (mid < lmid);
    return (u128)a1 * b1 + (mid >> 64) + ((u128)carry << 64);
}

void ctdo_mul128hi(const uint64_t a[2], const uint64_t b[2], uint64_t out[2])
{
    u128 r = mul128hi(((u128)a[0] << 64) | a[1], ((u128)b[0] << 64) | b[1]);
    out[0] = (uint64_t)(r >> 64);
    out[1] = (uint64_t)r;
}

/* a mod d by the 64-bit Barrett multiplier (modular_arithmetic_detail.hpp:335-340) */
static uint64_t bmod(uint64_t a, uint64_t d, uint64_t m64)
{
    uint64_t q = (uint64_t)(((u128)a * m64) >> 64);
    uint64_t r = a - q * d;
    return r >= d ? r - d : r;
}

typedef struct { uint64_t d, m64; u128 m128; } mu_t;

static mu_t make_mu(uint64_t d)
{
    mu_t m;
    m.d = d;
    m.m64 = ctdo_mu64(d);
    m.m128 = mu128(d);
    return m;
}

/* a * b mod d: 64-bit Barrett when the product fits 64 bits, else the
 * 128-bit multiplier (modular_arithmetic_detail.hpp:349-355). */
static uint64_t mulmod(uint64_t a, uint64_t b, const mu_t *mu)
{
    u128 ab = (u128)a * b;
    u128 q = (ab >> 64) ? mul128hi(ab, mu->m128) : ((ab * mu->m64) >> 64);
    u128 r = ab - q * mu->d;
    return (uint64_t)(r >= mu->d ? r - mu->d : r);
}

uint64_t ctdo_mulmod(uint64_t a, uint64_t b, uint64_t d)
{
    mu_t mu = make_mu(d);
    return mulmod(a, b, &mu);
}

/* (modular_arithmetic_detail.hpp:376-403) */
static inline uint64_t doublemod(uint64_t a, uint64_t d) { return a < d - a ? a << 1 : a - (d - a); }
static inline uint64_t submod(uint64_t a, uint64_t b, uint64_t d) { return a >= b ? a - b : d - (b - a); }
static inline uint64_t addmod(uint64_t a, uint64_t b, uint64_t d) { return a < d - b ? a + b : a - (d - b); }

/* left-to-right square-and-multiply over the bits of e (modular_arithmetic_detail.hpp:413-424) */
static uint64_t modpow(uint64_t a, uint64_t e, const mu_t *mu)
{
    uint64_t r = 1;
    uint64_t m = (a < mu->d) ? a : bmod(a, mu->d, mu->m64);
    for (; e; e >>= 1) {
        if (e & 1)
            r = mulmod(r, m, mu);
        m = mulmod(m, m, mu);
    }
    return r;
}

uint64_t ctdo_modpow(uint64_t a, uint64_t e, uint64_t d)
{
    mu_t mu = make_mu(d);
    return modpow(a, e, &mu);
}

/* floor((2^128 - 1) / d) - 2^64 for normalized d (top bit set)
 * (modular_arithmetic_detail.hpp:155-177, host branch). */
uint64_t ctdo_reciprocal(uint64_t d)
{
    return (uint64_t)((((u128)(UINT64_MAX - d)) << 64 | UINT64_MAX) / d);
}

/* (u1*2^64 + u0) mod d for normalized d and u1 < d, using the precomputed
 * reciprocal: Moller & Granlund 2011, "Improved division by invariant
 * integers", algorithm 4 (modular_arithmetic_detail.hpp:181-211). */
uint64_t ctdo_mod2by1(uint64_t u1, uint64_t u0, uint64_t d, uint64_t rnd)
{
    u128 q = (u128)u1 * rnd;
    q += ((u128)u1 << 64) | u0;
    uint64_t q1 = (uint64_t)(q >> 64) + 1;
    uint64_t q0 = (uint64_t)q;
    uint64_t r = u0 - q1 * d;
    if (r > q0)
        r += d;
    if (r >= d)
        r -= d;
    return r;
}

/* N mod d for a little-endian limb array, reduced limb by limb against the
 * normalized divisor, then mod d (modular_arithmetic_detail.hpp:213-232). */
uint64_t ctdo_modnby1(const uint64_t *n, uint64_t nlen, uint64_t d)
{
    if (!nlen)
        return 0;
    unsigned s = (unsigned)__builtin_clzll(d);
    uint64_t nd = d << s;
    uint64_t rnd = ctdo_reciprocal(nd);
    uint64_t r = 0;
    for (uint64_t j = nlen; j-- > 0;)
        r = ctdo_mod2by1(r, n[j], nd, rnd);
    return r % d;
}

/* ======================================================================
 * Primes in [lo, hi) -- the siever contract (src/siever.hpp:179-237,
 * primes ascending, hi excluded when the siever runs >= 2 threads).
 * ====================================================================== */

static int is_prime_u64(uint64_t n)
{
    /* deterministic Miller-Rabin for 64-bit n: the first twelve primes as
     * witnesses are sufficient below 3.3e24 */
    static const uint64_t witnesses[] = {2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37};
    if (n < 2)
        return 0;
    for (int i = 0; i < 12; ++i) {
        if (n == witnesses[i])
            return 1;
        if (n % witnesses[i] == 0)
            return 0;
    }
    uint64_t d = n - 1;
    int s = 0;
    while (!(d & 1)) {
        d >>= 1;
        ++s;
    }
    mu_t mu = make_mu(n);
    for (int i = 0; i < 12; ++i) {
        uint64_t x = modpow(witnesses[i], d, &mu);
        if (x == 1 || x == n - 1)
            continue;
        int composite = 1;
        for (int k = 1; k < s; ++k) {
            x = mulmod(x, x, &mu);
            if (x == n - 1) {
                composite = 0;
                break;
            }
        }
        if (composite)
            return 0;
    }
    return 1;
}

static uint64_t isqrt_u64(uint64_t x)
{
    uint64_t r = (uint64_t)__builtin_sqrtl((long double)x);
    while (r * r > x)
        --r;
    while ((r + 1) * (r + 1) <= x && (r + 1) * (r + 1) > r * r)
        ++r;
    return r;
}

/* odd primes < limit (limit small) by the plain sieve of Eratosthenes */
static uint32_t *odd_primes_below(uint32_t limit, uint32_t *count)
{
    uint8_t *comp = calloc(limit + 1, 1);
    uint32_t cap = 1024, n = 0;
    uint32_t *ps = malloc(cap * sizeof(uint32_t));
    for (uint64_t i = 3; i < limit; i += 2) {
        if (comp[i])
            continue;
        if (n == cap) {
            cap *= 2;
            ps = realloc(ps, cap * sizeof(uint32_t));
        }
        ps[n++] = (uint32_t)i;
        for (uint64_t j = i * i; j < limit; j += 2 * i)
            comp[j] = 1;
    }
    free(comp);
    *count = n;
    return ps;
}

#define EMIT(v)                          \
    do {                                 \
        if (out && cnt < cap)            \
            out[cnt] = (v);              \
        ++cnt;                           \
    } while (0)

uint64_t ctdo_sieve(uint64_t lo, uint64_t hi, uint64_t *out, uint64_t cap)
{
    uint64_t cnt = 0;
    if (hi <= lo)
        return 0;
    if (lo <= 2 && hi > 2)
        EMIT(2);
    uint64_t start = lo < 3 ? 3 : (lo | 1);
    if (start >= hi)
        return cnt;
    uint64_t limit = isqrt_u64(hi - 1) + 1; /* base primes p with p*p <= hi-1 */
    if (limit > (1u << 26)) {
        /* huge values with a tiny window: test each odd candidate */
        for (uint64_t v = start; v < hi && v >= start; v += 2)
            if (is_prime_u64(v))
                EMIT(v);
        return cnt;
    }
    uint32_t nbase;
    uint32_t *base = odd_primes_below((uint32_t)limit + 1, &nbase);
    const uint64_t W = 1u << 18; /* odd numbers per window */
    uint8_t *comp = malloc(W);
    for (uint64_t wlo = start; wlo < hi; wlo += 2 * W) {
        uint64_t span = (hi - wlo + 1) / 2; /* odd numbers left in [wlo, hi) */
        uint64_t len = span < W ? span : W;
        memset(comp, 0, len);
        uint64_t whi = wlo + 2 * len; /* exclusive */
        for (uint32_t i = 0; i < nbase; ++i) {
            uint64_t p = base[i];
            if (p * p >= whi)
                break;
            uint64_t m = p * p;
            if (m < wlo) {
                uint64_t r = wlo % p;
                m = r ? wlo + (p - r) : wlo;
                if (!(m & 1))
                    m += p;
            }
            for (uint64_t j = (m - wlo) / 2; j < len; j += p)
                comp[j] = 1;
        }
        for (uint64_t j = 0; j < len; ++j) {
            uint64_t v = wlo + 2 * j;
            if (!comp[j] && v > 1)
                EMIT(v);
        }
        if (whi < wlo)
            break;
    }
    free(comp);
    free(base);
    return cnt;
}

/* ======================================================================
 * Sequence plugins -- src/number_sequences/
 * ====================================================================== */

int ctdo_check_seq(uint32_t family, uint64_t param)
{
    switch (family) {
    case CTDO_MERSENNE:
    case CTDO_FIBONACCI:
    case CTDO_LUCAS:
    case CTDO_TRIBONACCI:
    case CTDO_PEANO:
        return 0;
    case CTDO_PROTH:
    case CTDO_RIESEL: /* k must be non-zero (riesel_proth.hpp:133-141) */
    case CTDO_PROTH_FIXED_N:
    case CTDO_RIESEL_FIXED_N: /* n must be non-zero (riesel_proth_fixed_n.hpp:73-79) */
        return param ? 0 : -1;
    case CTDO_SMARANDACHE: /* bases 2..64 (num_seq_dispatch.hpp:47-115) */
        return (param >= 2 && param <= 64) ? 0 : -1;
    default:
        return -1;
    }
}

static int is_pow2(uint64_t b) { return !(b & (b - 1)); }

uint64_t ctdo_value_mod_2(uint32_t family, uint64_t param, uint64_t n)
{
    switch (family) {
    case CTDO_MERSENNE: /* mersenne.hpp:248-254 */
        return n > 0;
    case CTDO_PROTH:
    case CTDO_RIESEL: /* riesel_proth.hpp:74-81 */
        return n > 0 ? 1 : ((param & 1) ^ 1);
    case CTDO_SMARANDACHE: /* smarandache.hpp:83-95 */
        if (!(param & 1))
            return n & 1;
        return (n & 3) && ((n & 3) != 3);
    case CTDO_FIBONACCI:
    case CTDO_LUCAS: /* fibonacci.hpp:230-235, lucas.hpp:380-385 */
        return n % 3 == 0 ? 0 : 1;
    case CTDO_PROTH_FIXED_N:
    case CTDO_RIESEL_FIXED_N: /* riesel_proth_fixed_n.hpp:117-122 */
        return 1;
    case CTDO_TRIBONACCI: /* tribonacci.hpp:553-557 */
        return (n & 3) >> 1;
    case CTDO_PEANO: /* tests/peano.hpp value_mod(n, 2) */
        return n & 1;
    }
    return 0;
}

uint64_t ctdo_next_value_mod_2(uint32_t family, uint64_t param, uint64_t r, uint64_t n)
{
    switch (family) {
    case CTDO_MERSENNE:
    case CTDO_PROTH:
    case CTDO_RIESEL:
    case CTDO_PROTH_FIXED_N:
    case CTDO_RIESEL_FIXED_N:
        return 1; /* mersenne.hpp:277-286, riesel_proth.hpp:83-88, riesel_proth_fixed_n.hpp:135-140 */
    case CTDO_SMARANDACHE: /* smarandache.hpp:97-112 */
        if (!(param & 1))
            return (n & 1) ^ 1;
        return r ^ (n & 1) ^ 1;
    case CTDO_FIBONACCI:
    case CTDO_LUCAS: /* fibonacci.hpp:237-242 */
        return (n + 1) % 3 == 0 ? 0 : 1;
    case CTDO_TRIBONACCI: /* tribonacci.hpp:559-564 */
        return ((n + 1) & 3) >> 1;
    case CTDO_PEANO: /* tests/peano.hpp next_value_mod(r, n, 2) */
        return r + 1 == 2 ? 0 : r + 1;
    }
    return 0;
}

/* Number of base-b digits of m (smarandache.hpp:124,142 via
 * modular_arithmetic_detail.hpp:306-326). */
static uint64_t digits_in_base(uint64_t b, uint64_t m)
{
    uint64_t res = 1;
    while (m /= b)
        ++res;
    return res;
}

/* b^(digits of n+1) (smarandache.hpp:160-198) */
static uint64_t sm_multiplier(uint64_t b, uint64_t n)
{
    uint64_t m = n + 1, result = b;
    while (m /= b)
        result *= b;
    return result;
}

/* Fibonacci make_state: (F(n-1), F(n)) mod d by doubling over the bits of
 * n-1; n <= 1 leaves previous = 0 (fibonacci.hpp:245-269). */
static void fib_state(uint64_t n, const mu_t *mu, uint64_t *prev, uint64_t *cur)
{
    uint64_t d = mu->d;
    if (n <= 1) {
        *prev = 0;
        *cur = n;
        return;
    }
    n -= 1;
    uint64_t f0 = 0, f1 = 1;
    for (uint64_t m = (uint64_t)1 << (63 - __builtin_clzll(n)); m; m >>= 1) {
        if (m & n) {
            uint64_t t0 = mulmod(submod(doublemod(f1, d), f0, d), f0, mu);
            f0 = addmod(mulmod(f1, f1, mu), mulmod(f0, f0, mu), d);
            f1 = addmod(f0, t0, d);
        } else {
            uint64_t t0 = f0;
            f0 = mulmod(submod(doublemod(f1, d), f0, d), f0, mu);
            f1 = addmod(mulmod(f1, f1, mu), mulmod(t0, t0, mu), d);
        }
    }
    *prev = f0;
    *cur = f1;
}

/* Tribonacci (T(n), T(n+1), T(n+2)) mod d by the doubling identities of
 * tribonacci_at (tribonacci.hpp:513-551). */
static void trib_state(uint64_t n, const mu_t *mu, uint64_t *t0, uint64_t *t1, uint64_t *t2)
{
    uint64_t d = mu->d;
    uint64_t vn = 0, vn1 = 0, vn2 = 1 % d;
    if (n) {
        for (uint64_t m = (uint64_t)1 << (63 - __builtin_clzll(n)); m; m >>= 1) {
            uint64_t sq_vn = mulmod(vn, vn, mu);
            uint64_t sq_vn1 = mulmod(vn1, vn1, mu);
            uint64_t two_vn1_vn = mulmod(doublemod(vn1, d), vn, mu);
            uint64_t tvn = submod(submod(addmod(mulmod(doublemod(vn2, d), vn, mu), sq_vn1, d), two_vn1_vn, d), sq_vn, d);
            uint64_t tvn1 = submod(addmod(sq_vn, mulmod(doublemod(vn2, d), vn1, mu), d), sq_vn1, d);
            vn2 = addmod(addmod(two_vn1_vn, mulmod(vn2, vn2, mu), d), sq_vn1, d);
            vn = tvn;
            vn1 = tvn1;
            if (m & n) {
                uint64_t vn3 = addmod(addmod(vn, vn1, d), vn2, d);
                vn = vn1;
                vn1 = vn2;
                vn2 = vn3;
            }
        }
    }
    *t0 = vn;
    *t1 = vn1;
    *t2 = vn2;
}

void ctdo_init(uint32_t family, uint64_t param, uint64_t n0, uint64_t p,
               const uint64_t *sm_limbs, uint64_t sm_nlimbs, ctdo_state *st)
{
    mu_t mu = make_mu(p);
    uint64_t r;
    memset(st, 0, sizeof(*st));
    switch (family) {
    case CTDO_MERSENNE: /* mersenne.hpp:256-275 */
        if (n0 <= 1) {
            st->r = (n0 == 0 || p == 1) ? 0 : 1;
            return;
        }
        r = modpow(2, n0, &mu);
        st->r = r ? r - 1 : p - 1;
        return;
    case CTDO_PROTH:
    case CTDO_RIESEL: /* riesel_proth.hpp:90-101 */
        r = mulmod(modpow(2, n0, &mu), param, &mu);
        if (family == CTDO_PROTH)
            st->r = (r == p - 1) ? 0 : r + 1;
        else
            st->r = r ? r - 1 : p - 1;
        return;
    case CTDO_SMARANDACHE: /* InitializeFromValue: Sm_b(n0) mod p
                              (src/trial_factoring_impl.hpp:216-218, src/hgint.hpp:270-274) */
        st->r = 0;
        for (uint64_t j = sm_nlimbs; j-- > 0;)
            st->r = (uint64_t)((((u128)st->r) << 64 | sm_limbs[j]) % p);
        return;
    case CTDO_FIBONACCI: /* fibonacci.hpp:245-277 */
        fib_state(n0, &mu, &st->s[0], &st->s[1]);
        st->r = st->s[1];
        return;
    case CTDO_LUCAS: { /* lucas.hpp:394-412: L(n-1) = 2F(n) - F(n-1), L(n) = F(n) + 2F(n-1) */
        uint64_t fnm1, fn;
        fib_state(n0, &mu, &fnm1, &fn);
        st->s[0] = submod(doublemod(fn, p), fnm1, p);
        st->s[1] = addmod(fn, doublemod(fnm1, p), p);
        st->r = st->s[1];
        return;
    }
    case CTDO_PROTH_FIXED_N:
    case CTDO_RIESEL_FIXED_N: /* riesel_proth_fixed_n.hpp:88-94,124-133: index n0 is k */
        st->s[0] = modpow(2, param, &mu);
        r = bmod(n0, p, mu.m64);
        r = mulmod(r, st->s[0], &mu);
        if (family == CTDO_PROTH_FIXED_N)
            st->r = (r == p - 1) ? 0 : r + 1;
        else
            st->r = !r ? p - 1 : r - 1;
        return;
    case CTDO_TRIBONACCI: /* tribonacci.hpp:566-580 */
        trib_state(n0, &mu, &st->s[0], &st->s[1], &st->s[2]);
        st->r = st->s[0];
        return;
    case CTDO_PEANO: /* tests/peano.hpp value_mod */
        st->r = n0 % p;
        return;
    }
}

/* One step with the Barrett multipliers of p precomputed (the reference
 * computes them once per prime, src/trial_factoring_impl.hpp:201). */
static inline __attribute__((always_inline)) void step_impl(uint32_t family, uint64_t param, uint64_t n,
                                                            const mu_t *mu, ctdo_state *st)
{
    const uint64_t p = mu->d;
    uint64_t r = st->r;
    switch (family) {
    case CTDO_MERSENNE: /* M(n+1) = 2M(n) + 1 (mersenne.hpp:289-303) */
        if (r < p - r) {
            uint64_t v = (r << 1) + 1;
            st->r = v == p ? 0 : v;
        } else {
            st->r = r - (p - r) + 1;
        }
        return;
    case CTDO_PROTH:
    case CTDO_RIESEL: /* S(n+1) = 2S(n) -+ 1 (riesel_proth.hpp:103-115) */
        r = (r < p - r) ? r << 1 : r - (p - r);
        if (family == CTDO_PROTH)
            st->r = r ? r - 1 : p - 1;
        else
            st->r = (r == p - 1) ? 0 : r + 1;
        return;
    case CTDO_SMARANDACHE: { /* Sm(n+1) = Sm(n) * b^len(n+1) + n + 1 (smarandache.hpp:131-158) */
        /* s[0] caches b^len(n+1) (or the shift for power-of-2 bases) and s[1]
         * the next power of b, where len(n+1) grows; the reference gets the
         * same multiplier from compute_multiplier(n) each step */
        if (!st->s[1] || n + 1 >= st->s[1]) {
            uint64_t M = sm_multiplier(param, n);
            st->s[1] = M;
            st->s[0] = is_pow2(param) ? digits_in_base(param, n + 1) * (63 - __builtin_clzll(param)) : M;
        }
        u128 a;
        if (is_pow2(param))
            a = ((u128)r << st->s[0]) + n + 1;
        else
            a = (u128)r * st->s[0] + n + 1;
        u128 q = (a >> 64) ? mul128hi(a, mu->m128) : ((a * mu->m64) >> 64);
        u128 rr = a - q * p;
        st->r = (uint64_t)(rr >= p ? rr - p : rr);
        return;
    }
    case CTDO_FIBONACCI:
    case CTDO_LUCAS: /* fibonacci.hpp:279-285 */
        st->r = addmod(r, st->s[0], p);
        st->s[0] = r;
        return;
    case CTDO_PROTH_FIXED_N:
    case CTDO_RIESEL_FIXED_N: /* S(k+1) = S(k) + 2^n (riesel_proth_fixed_n.hpp:142-151) */
        st->r = (r >= p - st->s[0]) ? r - (p - st->s[0]) : r + st->s[0];
        return;
    case CTDO_TRIBONACCI: { /* tribonacci.hpp:582-590 */
        uint64_t t3 = addmod(addmod(st->s[0], st->s[1], p), st->s[2], p);
        st->s[0] = st->s[1];
        st->s[1] = st->s[2];
        st->s[2] = t3;
        st->r = st->s[0];
        return;
    }
    case CTDO_PEANO: /* tests/peano.hpp next_value_mod */
        st->r = (r + 1 == p) ? 0 : r + 1;
        return;
    }
}

void ctdo_step(uint32_t family, uint64_t param, uint64_t n, uint64_t p, ctdo_state *st)
{
    mu_t mu = make_mu(p);
    step_impl(family, param, n, &mu, st);
}

uint64_t ctdo_smarandache_limbs(uint64_t base, uint64_t n, uint64_t *out, uint64_t cap)
{
    /* v = v * b^len(i) + i for i = 1..n, several i folded per pass while the
     * multiplier and addend fit 64 bits */
    uint64_t nl = 0, alloc = 16;
    uint64_t *v = calloc(alloc, sizeof(uint64_t));
    uint64_t i = 1;
    while (i <= n) {
        uint64_t mul = 1, add = 0;
        while (i <= n) {
            uint64_t pw = sm_multiplier(base, i - 1); /* b^len(i) */
            u128 nm = (u128)mul * pw;
            u128 na = (u128)add * pw + i;
            if ((nm >> 64) || (na >> 64))
                break;
            mul = (uint64_t)nm;
            add = (uint64_t)na;
            ++i;
        }
        uint64_t carry = add;
        for (uint64_t j = 0; j < nl; ++j) {
            u128 t = (u128)v[j] * mul + carry;
            v[j] = (uint64_t)t;
            carry = (uint64_t)(t >> 64);
        }
        if (carry) {
            if (nl == alloc) {
                alloc *= 2;
                v = realloc(v, alloc * sizeof(uint64_t));
            }
            v[nl++] = carry;
        }
    }
    if (out)
        for (uint64_t j = 0; j < nl && j < cap; ++j)
            out[j] = v[j];
    free(v);
    return nl;
}

/* ======================================================================
 * Engine -- src/trial_factoring_impl.hpp
 * ====================================================================== */

/* factors_buffer::push_factor (src/factors_buffer.hpp:110-121): atomic
 * increment of the count, store only while below the per-index capacity */
static inline void push_factor(uint32_t *counts, uint64_t *factors, uint32_t maxf,
                               uint64_t idx, uint64_t p)
{
    uint32_t pos = __atomic_fetch_add(&counts[idx], 1u, __ATOMIC_RELAXED);
    if (pos < maxf)
        factors[idx * maxf + pos] = p;
}

typedef struct {
    const ctdo_job *job;
    const uint64_t *primes;
    uint64_t nprimes;
    uint64_t next; /* shared cursor, advanced atomically */
    uint32_t *counts;
    uint64_t *factors;
    const uint64_t *sm_limbs;
    uint64_t sm_nlimbs;
} work_t;

/* trial_factorer::process_chunk (src/trial_factoring_impl.hpp:193-248),
 * instantiated per family like the reference's templates */
#define PROCESS_FAMILY(FAM)                                                                   \
    case FAM:                                                                                 \
        for (uint64_t i = i0; i < i1; ++i) {                                                  \
            uint64_t p = w->primes[i];                                                        \
            mu_t mu = make_mu(p);                                                             \
            ctdo_state st;                                                                    \
            ctdo_init(FAM, job->param, job->n0, p, w->sm_limbs, w->sm_nlimbs, &st);           \
            if (!st.r)                                                                        \
                push_factor(w->counts, w->factors, job->max_factors, 0, p);                   \
            for (uint64_t n = job->n0, ne = job->n1 - 1; n < ne; ++n) {                       \
                step_impl(FAM, job->param, n, &mu, &st);                                      \
                if (!st.r)                                                                    \
                    push_factor(w->counts, w->factors, job->max_factors, n + 1 - job->n0, p); \
            }                                                                                 \
        }                                                                                     \
        break;

static void process_primes(work_t *w, uint64_t i0, uint64_t i1)
{
    const ctdo_job *job = w->job;
    switch (job->family) {
        PROCESS_FAMILY(CTDO_MERSENNE)
        PROCESS_FAMILY(CTDO_PROTH)
        PROCESS_FAMILY(CTDO_RIESEL)
        PROCESS_FAMILY(CTDO_SMARANDACHE)
        PROCESS_FAMILY(CTDO_FIBONACCI)
        PROCESS_FAMILY(CTDO_LUCAS)
        PROCESS_FAMILY(CTDO_PROTH_FIXED_N)
        PROCESS_FAMILY(CTDO_RIESEL_FIXED_N)
        PROCESS_FAMILY(CTDO_TRIBONACCI)
        PROCESS_FAMILY(CTDO_PEANO)
    }
}

static void *worker(void *arg)
{
    work_t *w = arg;
    const uint64_t chunk = 64;
    for (;;) {
        uint64_t i0 = __atomic_fetch_add(&w->next, chunk, __ATOMIC_RELAXED);
        if (i0 >= w->nprimes)
            break;
        uint64_t i1 = i0 + chunk < w->nprimes ? i0 + chunk : w->nprimes;
        process_primes(w, i0, i1);
    }
    return NULL;
}

static void run_parallel(work_t *w, int threads)
{
    if (threads <= 1 || w->nprimes < 256) {
        process_primes(w, 0, w->nprimes);
        return;
    }
    pthread_t *tid = malloc(sizeof(pthread_t) * (size_t)threads);
    int started = 0;
    for (int t = 0; t < threads; ++t)
        if (pthread_create(&tid[t], NULL, worker, w) == 0)
            ++started;
    if (!started)
        worker(w);
    for (int t = 0; t < started; ++t)
        pthread_join(tid[t], NULL);
    free(tid);
}

static int job_valid(const ctdo_job *job)
{
    if (ctdo_check_seq(job->family, job->param))
        return 0;
    return job->n1 > job->n0 && job->max_factors > 0;
}

static uint64_t *smarandache_init_limbs(const ctdo_job *job, uint64_t *nl)
{
    *nl = 0;
    if (job->family != CTDO_SMARANDACHE)
        return NULL;
    uint64_t n = ctdo_smarandache_limbs(job->param, job->n0, NULL, 0);
    uint64_t *l = malloc((n ? n : 1) * sizeof(uint64_t));
    ctdo_smarandache_limbs(job->param, job->n0, l, n);
    *nl = n;
    return l;
}

int ctdo_residues(const ctdo_job *job, const uint64_t *primes, uint64_t nprimes,
                  uint32_t *counts, uint64_t *factors, int threads)
{
    if (!job_valid(job))
        return -1;
    work_t w;
    memset(&w, 0, sizeof(w));
    w.job = job;
    w.primes = primes;
    w.nprimes = nprimes;
    w.counts = counts;
    w.factors = factors;
    w.sm_limbs = smarandache_init_limbs(job, &w.sm_nlimbs);
    run_parallel(&w, threads);
    free((void *)w.sm_limbs);
    return 0;
}

/* host_trial_factor (src/trial_factoring_impl.hpp:278-366): the prime 2 in
 * its own pass (:312-325), then odd primes segment by segment (:338-357). */
int ctdo_trial_factor(const ctdo_job *job, uint32_t *counts, uint64_t *factors,
                      uint64_t resume_after_prime, uint64_t segment_length, int threads)
{
    if (!job_valid(job) || job->f1 <= job->f0)
        return -1;
    const uint64_t n0 = job->n0, n1 = job->n1;
    uint64_t f0 = resume_after_prime ? resume_after_prime + 1 : job->f0;
    const uint64_t f1 = job->f1;
    if (!segment_length)
        segment_length = (uint64_t)1 << 26;
    if (f0 <= 2 && f1 > 2) {
        f0 = 3;
        uint64_t r = ctdo_value_mod_2(job->family, job->param, n0);
        if (!r)
            push_factor(counts, factors, job->max_factors, 0, 2);
        for (uint64_t n = n0; n < n1 - 1; ++n) {
            r = ctdo_next_value_mod_2(job->family, job->param, r, n);
            if (!r)
                push_factor(counts, factors, job->max_factors, n + 1 - n0, 2);
        }
    }
    uint64_t nl;
    uint64_t *limbs = smarandache_init_limbs(job, &nl);
    uint64_t cap = 0;
    uint64_t *primes = NULL;
    for (uint64_t fx = f0, fy = (f1 - f0 > segment_length) ? f0 + segment_length : f1; fx < f1;
         fx = fy, fy = (f1 - fy > segment_length) ? fy + segment_length : f1) {
        uint64_t np = ctdo_sieve(fx, fy, NULL, 0);
        if (np > cap) {
            cap = np;
            primes = realloc(primes, cap * sizeof(uint64_t));
        }
        ctdo_sieve(fx, fy, primes, np);
        work_t w;
        memset(&w, 0, sizeof(w));
        w.job = job;
        w.primes = primes;
        w.nprimes = np;
        w.counts = counts;
        w.factors = factors;
        w.sm_limbs = limbs;
        w.sm_nlimbs = nl;
        run_parallel(&w, threads);
    }
    free(primes);
    free(limbs);
    return 0;
}
