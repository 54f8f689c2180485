// ctd_powres.cuh -- power-residue classes of the doubling families.
//
// Proth k*2^n+1, Riesel k*2^n-1 and Mersenne 2^n-1 have a zero mod an odd
// prime p at n exactly when w(n) = 2^-n = wt (mod p), wt = -k, k or 1 (the
// baby-step walks of ctd_residue.cu walk w).  For every prime q dividing
// p - 1, raising both sides to e = (p - 1)/q maps them into the q-th roots
// of unity:  z^n = y  with  z = 2^-e,  y = wt^e.
//   * z = 1: every n gives 1, so either y = 1 (no condition) or no n at all
//     satisfies the congruence -- the prime divides no term;
//   * z != 1: z has order q and generates the q-th roots of unity; y is one
//     of them (y^q = wt^(p-1) = 1), y = z^j for one j < q, and n = j (mod q).
// For the powers of 2 the same holds with the 2^u-th roots (2^u | p - 1):
// z = 2^-((p-1)/2^u) has order 2^i, y must lie in the subgroup of order 2^i
// (y^(2^i) = 1), and n is fixed mod 2^i by a discrete logarithm in that
// cyclic 2-group (a scan of its at most 8 elements).  The conditions are
// necessary, never sufficient: the walk still tests every n of the class
// exactly, so the hits are exactly the walk's (no hit is lost: an n outside
// the class cannot satisfy z^n = y).  Over random primes the class keeps
// about E[2^-u] * (2/3) * (4/5) * (6/7) ~ 0.16 of the terms (u = the 2-adic
// valuation of p - 1, capped at 3: E[2^-u] = 0.34) for 2^3, 3, 5 and 7.
//
// The same idea is the "Legendre symbol" filter of classical sieving
// programs for k*2^n+-1 (a prime where -k is a quadratic non-residue and 2
// a residue divides no term); here it is carried to the 2-power, 3rd, 5th
// and 7th power residues.  __host__ __device__ so the host tests run the
// same code.
#pragma once

#include "ctd_arith.cuh"

namespace ctd {

// largest power of 2 taken from p - 1 (2^3 = 8 classes at most: the
// higher 2-power characters would shave about 3 % more terms for twice the
// set-up)
constexpr int POWRES_MAX_2EXP = 3;

// the class n = r (mod M) every zero of the doubling family must lie in
struct PowerClass {
    uint32_t M;  // 0: no n is a zero mod p
    uint32_t r;  // < M
};

// n = r (mod M) and n = j (mod q) for a prime q <= 127 not dividing M:
// n = r + M t with t = (j - r) M^-1 (mod q), the inverse by Fermat
// (M^(q-2)); 32-bit arithmetic
CTD_HD void crt_merge_small(PowerClass &c, uint32_t j, uint32_t q)
{
    const uint32_t d = c.M % q;
    uint32_t inv = 1, b = d;
    for (uint32_t e = q - 2; e; e >>= 1) {
        if (e & 1)
            inv = inv * b % q;
        b = b * b % q;
    }
    const uint32_t t = (j + q - c.r % q) % q * inv % q;
    c.r += c.M * t;
    c.M *= q;
}


// The classifier's fixed chains multiply through one out-of-line function
// on the device (the two powering loops keep theirs inline): with all ~140
// Montgomery products inlined the kernel was large enough that warps
// stalled on instruction fetch (ncu: "no instruction" the top stall).
#ifdef __CUDA_ARCH__
template <class MT>
__device__ __noinline__ uint64_t powres_mul(uint64_t a, uint64_t b, uint64_t p, uint64_t pinv)
{
    MT m;
    m.p = p;
    m.pinv = pinv;
    return m.mul(a, b);
}
#else
template <class MT>
inline uint64_t powres_mul(uint64_t a, uint64_t b, uint64_t p, uint64_t pinv)
{
    MT m;
    m.p = p;
    m.pinv = pinv;
    return m.mul(a, b);
}
#endif

// base^e (base in Montgomery form, e small)
template <class MT>
CTD_HD uint64_t small_pow(const MT &m, uint64_t base, uint32_t e)
{
    uint64_t r = m.one;
    while (e) {
        if (e & 1)
            r = m.mul(r, base);
        base = m.mul(base, base);
        e >>= 1;
    }
    return r;
}

// x^(2^s)
template <class MT>
CTD_HD uint64_t square_n(const MT &m, uint64_t x, int s)
{
    for (int i = 0; i < s; ++i)
        x = m.mul(x, x);
    return x;
}

// x * w for x in Montgomery form and a plain w < p (Shoup's quotient
// ws = floor(w 2^64 / p)): the Montgomery form of the product, p < 2^63
CTD_HD uint64_t shoup_mul(uint64_t x, uint64_t w, uint64_t ws, uint64_t p)
{
    const uint64_t q = mulhi64(x, ws);
    const uint64_t r = x * w - q * p;
    return r >= p ? r - p : r;
}

// x^105 = x^(3 5 7) and x^15, x^21, x^35 (the q-th power maps of q = 7, 5, 3
// applied to the 105-part): one addition chain
struct Pow105 {
    uint64_t p15, p21, p35, p105;
};
template <class MT>
CTD_HD Pow105 pow105(const MT &m, uint64_t x)
{
    auto mul = [&](uint64_t a, uint64_t b) { return powres_mul<MT>(a, b, m.p, m.pinv); };
    const uint64_t x2 = mul(x, x), x3 = mul(x2, x), x5 = mul(x3, x2), x7 = mul(x5, x2);
    const uint64_t x10 = mul(x5, x5), x15 = mul(x10, x5), x14 = mul(x7, x7), x21 = mul(x14, x7);
    const uint64_t x35 = mul(x21, x14), x70 = mul(x35, x35), x105 = mul(x70, x35);
    return Pow105{x15, x21, x35, x105};
}

// ---- the quadratic screen
// The classes' cheapest condition needs no power: when 2 is a quadratic
// residue mod p (p = +-1 mod 8) every 2^-n is one, so a target wt that is a
// non-residue is never reached -- p divides no term.  That is a quarter of
// the primes for a generic target, decided by Legendre symbols alone, so the
// kernels take those primes out before the two powers of doubling_class.

CTD_HD int ctz64(uint64_t x)
{
#ifdef __CUDA_ARCH__
    return __ffsll((long long)x) - 1;
#else
    return __builtin_ctzll(x);
#endif
}

// Jacobi symbol (a/n) for odd n: a reduced mod n once, then the binary
// algorithm (factors of 2 by (2/n) = -1 iff n = 3, 5 mod 8; quadratic
// reciprocity on each swap; subtraction)
CTD_HD int jacobi(uint64_t a, uint64_t n)
{
    a %= n;
    int t = 1;
    while (a) {
        const int z = ctz64(a);
        a >>= z;
        if ((z & 1) && ((n & 7) == 3 || (n & 7) == 5))
            t = -t;
        if (a < n) {
            if ((a & 3) == 3 && (n & 3) == 3)
                t = -t;
            const uint64_t x = a;
            a = n;
            n = x;
        }
        a -= n;
    }
    return n == 1 ? t : 0;
}

// The Legendre symbol (wt/p), wt = -k (negate) or k, for an odd prime p
// and k < 2^64: (2/p)^s (k'/p) (-1/p)^negate with k = 2^s k', and
// (k'/p) = (p/k') (-1)^((k'-1)/2 (p-1)/2) by reciprocity -- a reduction of p
// mod k' and a Jacobi symbol of k'-sized numbers.  0 when p | k.
CTD_HD int target_symbol(uint64_t p, uint64_t k, bool negate)
{
    const uint64_t kr = k < p ? k : k % p;
    if (!kr)
        return 0;
    const int s = ctz64(kr);
    const uint64_t k1 = kr >> s;
    const bool two_nr = (p & 7) == 3 || (p & 7) == 5;  // (2/p) = -1
    int t = (s & 1) && two_nr ? -1 : 1;
    if (k1 > 1) {
        t *= jacobi(p, k1);
        if ((k1 & 3) == 3 && (p & 3) == 3)
            t = -t;
    }
    if (negate && (p & 3) == 3)  // (-1/p) = -1
        t = -t;
    return t;
}

// true when the quadratic characters alone show that 2^-n = wt (mod p) has
// no solution (2 a residue, wt a non-residue), or p | k
CTD_HD bool quadratic_excluded(uint64_t p, uint64_t k, bool negate)
{
    const bool two_qr = (p & 7) == 1 || (p & 7) == 7;
    const int t = target_symbol(p, k, negate);
    return t == 0 || (two_qr && t < 0);
}

// A = 2^-e = (1/2)^e and B = wt^e = (-+1)^e k^e, both in Montgomery form,
// in one left-to-right loop over the bits of e: per bit a squaring of each,
// and for a set bit a halving of A's Montgomery representative ((x R)/2 =
// (x/2) R) and a Shoup multiplication of B by the plain k -- two
// independent chains per iteration.  0 < e < p - 1, p < 2^63 (m needs no r2).
template <class MT>
CTD_HD void power_pair(const MT &m, uint64_t k, bool negate, uint64_t e, uint64_t &A, uint64_t &B)
{
    const uint64_t p = m.p;
    const uint64_t kr = k < p ? k : k % p;
    const uint64_t ks = m.shoup_any(kr);
    A = m.one;
    B = m.one;
    // A and B stay below 2p (the narrow product's lazy form; a halving of
    // x < 2p is below 1.5p; Shoup's product of x < 2^64 is below p)
    for (int b = 63 - clz64(e); b >= 0; --b) {
        A = m.mul_lazy(A, A);  // inline: the hot loop stays small
        B = m.mul_lazy(B, B);
        if ((e >> b) & 1) {
            A = (A + ((A & 1) ? p : 0)) >> 1;
            B = shoup_mul(B, kr, ks, p);
        }
    }
    A = m.canon(A);
    B = m.canon(B);
    if (negate && (e & 1))
        B = B ? p - B : 0;
}

// The class of the zeros of 2^-n = wt (mod p), wt = -k (negate) or k, for
// an odd prime p < 2^63 and a plain k with k mod p != 0 (m needs no r2).
// The work is the same
// for every prime -- two full powers, fixed chains, loops of fixed length
// -- so the lanes of a warp stay together.
template <class MT>
CTD_HD PowerClass doubling_class(const MT &m, uint64_t k, bool negate)
{
    const uint64_t p = m.p;
    const uint64_t p1 = p - 1;
#ifdef __CUDA_ARCH__
    const int v = __ffsll((long long)p1) - 1;
#else
    const int v = __builtin_ctzll(p1);
#endif
    const int u = v < POWRES_MAX_2EXP ? v : POWRES_MAX_2EXP;
    const bool f3 = p1 % 3 == 0, f5 = p1 % 5 == 0, f7 = p1 % 7 == 0;
    // e0 = (p - 1) / D, D = 2^u 3^f3 5^f5 7^f7
    uint64_t e0 = p1 >> u;
    e0 = f3 ? e0 / 3 : e0;
    e0 = f5 ? e0 / 5 : e0;
    e0 = f7 ? e0 / 7 : e0;
    auto mul = [&](uint64_t a, uint64_t b) { return powres_mul<MT>(a, b, p, m.pinv); };
    uint64_t A, B;
    power_pair(m, k, negate, e0, A, B);
    // A and B lie in the D-th roots of unity.  For a q that does not divide
    // p - 1 the fixed exponents below map them to 1 (no condition); for one
    // that does, they differ from (p - 1)/q by a factor prime to q, which
    // changes neither the order of z nor the logarithm j of y = z^j.
    PowerClass c{1, 0};
    // ---- the 2-power part: z = A^105 of order 2^i (i <= u)
    const Pow105 pa = pow105(m, A), pb = pow105(m, B);
    {
        const uint64_t z = pa.p105, y = pb.p105;
        uint64_t zs = z, ys = y;
        int i = 0;
        bool y_ok = ys == m.one;
        bool found = zs == m.one;
#pragma unroll
        for (int t = 1; t <= POWRES_MAX_2EXP; ++t) {
            zs = mul(zs, zs);
            ys = mul(ys, ys);
            if (!found && t <= u) {
                i = t;
                y_ok = ys == m.one;
                found = zs == m.one;
            }
        }
        if (!y_ok)
            return PowerClass{0, 0};  // y outside <z>: no zero at all
        // the logarithm j < 2^i of y to the base z, by a scan of z^j
        uint32_t j = 0;
        uint64_t t = m.one;
#pragma unroll
        for (uint32_t jj = 0; jj < (1u << POWRES_MAX_2EXP); ++jj) {
            if (jj < (1u << i) && t == y)
                j = jj;
            if (jj + 1 < (1u << POWRES_MAX_2EXP))
                t = mul(t, z);
        }
        c.M = 1u << i;
        c.r = j;
    }
    // ---- q = 3, 5, 7: z = A^(2^u 105 / q) = (A^(105/q))^(2^u), squarings
    // of the chain's values (a loop of fixed length)
    uint64_t zq[3] = {pa.p35, pa.p21, pa.p15}, yq[3] = {pb.p35, pb.p21, pb.p15};
#pragma unroll
    for (int t = 0; t < POWRES_MAX_2EXP; ++t)
#pragma unroll
        for (int kq = 0; kq < 3; ++kq) {
            const uint64_t z2 = mul(zq[kq], zq[kq]), y2 = mul(yq[kq], yq[kq]);
            zq[kq] = t < u ? z2 : zq[kq];
            yq[kq] = t < u ? y2 : yq[kq];
        }
    const uint32_t qs[3] = {3, 5, 7};
#pragma unroll
    for (int kq = 0; kq < 3; ++kq) {
        const uint32_t q = qs[kq];
        const uint64_t z = zq[kq], y = yq[kq];
        if (z == m.one) {
            if (y != m.one)
                return PowerClass{0, 0};
            continue;
        }
        uint32_t j = q;
        uint64_t t = m.one;
#pragma unroll
        for (uint32_t jj = 0; jj < q; ++jj) {
            if (t == y)
                j = jj;
            if (jj + 1 < q)
                t = mul(t, z);
        }
        if (j >= q)  // cannot happen for prime p (y is a q-th root of unity)
            return PowerClass{1, 0};
        crt_merge_small(c, j, q);
    }
    return c;
}

// ---- the same class for a known divisibility pattern of p - 1
// PAT bit 0: 3 | p - 1, bit 1: 5 | p - 1, bit 2: 7 | p - 1.  A q that does
// not divide p - 1 gives no condition (x -> x^q permutes the group), so the
// kernels, which bucket the primes by pattern first, raise A and B only to
// the exponents the pattern needs: on average about 2.5 products for the
// odd part instead of the 11 of the full chain, one q's squarings and scan
// instead of three.  Every lane of a bucket runs the same code.
CTD_HD uint32_t powres_pattern(uint64_t p)
{
    return ((p - 1) % 3 == 0 ? 1u : 0u) | ((p - 1) % 5 == 0 ? 2u : 0u) | ((p - 1) % 7 == 0 ? 4u : 0u);
}

// x^D and x^(D/q) for the q of PAT, D the product of PAT's q: short chains
template <int PAT, class MT>
CTD_HD void odd_powers(const MT &m, uint64_t x, uint64_t &xd, uint64_t (&xq)[3])
{
    auto mul = [&](uint64_t a, uint64_t b) { return powres_mul<MT>(a, b, m.p, m.pinv); };
    xq[0] = xq[1] = xq[2] = x;
    if constexpr (PAT == 0) {
        xd = x;
    } else if constexpr (PAT == 1) {  // 3
        xd = mul(mul(x, x), x);
    } else if constexpr (PAT == 2) {  // 5
        const uint64_t x2 = mul(x, x), x4 = mul(x2, x2);
        xd = mul(x4, x);
    } else if constexpr (PAT == 4) {  // 7
        const uint64_t x3 = mul(mul(x, x), x), x6 = mul(x3, x3);
        xd = mul(x6, x);
    } else if constexpr (PAT == 3) {  // 15 = 3 5
        const uint64_t x2 = mul(x, x), x3 = mul(x2, x), x5 = mul(x3, x2), x10 = mul(x5, x5);
        xd = mul(x10, x5);
        xq[0] = x5;
        xq[1] = x3;
    } else if constexpr (PAT == 5) {  // 21 = 3 7
        const uint64_t x2 = mul(x, x), x3 = mul(x2, x), x4 = mul(x2, x2), x7 = mul(x4, x3), x14 = mul(x7, x7);
        xd = mul(x14, x7);
        xq[0] = x7;
        xq[2] = x3;
    } else if constexpr (PAT == 6) {  // 35 = 5 7
        const uint64_t x2 = mul(x, x), x3 = mul(x2, x), x5 = mul(x3, x2), x7 = mul(x5, x2);
        const uint64_t x14 = mul(x7, x7), x28 = mul(x14, x14);
        xd = mul(x28, x7);
        xq[1] = x7;
        xq[2] = x5;
    } else {  // 105
        const Pow105 c = pow105(m, x);
        xd = c.p105;
        xq[0] = c.p35;
        xq[1] = c.p21;
        xq[2] = c.p15;
    }
}

// doubling_class for a p whose pattern is PAT (powres_pattern(p) == PAT)
template <int PAT, class MT>
CTD_HD PowerClass doubling_class_pat(const MT &m, uint64_t k, bool negate)
{
    const uint64_t p = m.p;
    const uint64_t p1 = p - 1;
#ifdef __CUDA_ARCH__
    const int v = __ffsll((long long)p1) - 1;
#else
    const int v = __builtin_ctzll(p1);
#endif
    const int u = v < POWRES_MAX_2EXP ? v : POWRES_MAX_2EXP;
    // e0 = (p - 1) / D, D = 2^u 3^f3 5^f5 7^f7 (divisions by constants)
    uint64_t e0 = p1 >> u;
    if constexpr ((PAT & 1) != 0)
        e0 /= 3;
    if constexpr ((PAT & 2) != 0)
        e0 /= 5;
    if constexpr ((PAT & 4) != 0)
        e0 /= 7;
    auto mul = [&](uint64_t a, uint64_t b) { return powres_mul<MT>(a, b, p, m.pinv); };
    uint64_t A, B;
    power_pair(m, k, negate, e0, A, B);
    uint64_t ad, bd, aq[3], bq[3];
    odd_powers<PAT>(m, A, ad, aq);
    odd_powers<PAT>(m, B, bd, bq);
    PowerClass c{1, 0};
    // ---- the 2-power part: z = A^D_odd of order 2^i (i <= u)
    {
        const uint64_t z = ad, y = bd;
        uint64_t zs = z, ys = y;
        int i = 0;
        bool y_ok = ys == m.one;
        bool found = zs == m.one;
#pragma unroll
        for (int t = 1; t <= POWRES_MAX_2EXP; ++t) {
            zs = mul(zs, zs);
            ys = mul(ys, ys);
            if (!found && t <= u) {
                i = t;
                y_ok = ys == m.one;
                found = zs == m.one;
            }
        }
        if (!y_ok)
            return PowerClass{0, 0};
        uint32_t j = 0;
        uint64_t t = m.one;
#pragma unroll
        for (uint32_t jj = 0; jj < (1u << POWRES_MAX_2EXP); ++jj) {
            if (jj < (1u << i) && t == y)
                j = jj;
            if (jj + 1 < (1u << POWRES_MAX_2EXP))
                t = mul(t, z);
        }
        c.M = 1u << i;
        c.r = j;
    }
    // ---- the q of PAT: z = (A^(D_odd/q))^(2^u)
    const uint32_t qs[3] = {3, 5, 7};
#pragma unroll
    for (int kq = 0; kq < 3; ++kq) {
        if (!((PAT >> kq) & 1))
            continue;
        const uint32_t q = qs[kq];
        uint64_t z = aq[kq], y = bq[kq];
#pragma unroll
        for (int t = 0; t < POWRES_MAX_2EXP; ++t) {
            const uint64_t z2 = mul(z, z), y2 = mul(y, y);
            z = t < u ? z2 : z;
            y = t < u ? y2 : y;
        }
        if (z == m.one) {
            if (y != m.one)
                return PowerClass{0, 0};
            continue;
        }
        uint32_t j = q;
        uint64_t t = m.one;
#pragma unroll
        for (uint32_t jj = 0; jj < q; ++jj) {
            if (t == y)
                j = jj;
            if (jj + 1 < q)
                t = mul(t, z);
        }
        if (j >= q)  // cannot happen for prime p
            return PowerClass{1, 0};
        crt_merge_small(c, j, q);
    }
    return c;
}


// ---- refinement by the character of a rarer prime q = 11 .. 127
// A prime q divides p - 1 for one prime p in q - 1, and then its character
// keeps one term in q (or none), so over the classes above the walk shrinks
// by about prod (1 - 1/q): 0.58 for q = 11 .. 61, 0.50 up to 127 (measured
// over primes near 2^33: the walked fraction 0.063 -> 0.055 from 61 to 127).
// The refinement costs two more full powers, for the primes that have such
// a q only: the kernels run it as a separate pass over those primes (about
// 30 % of them), so no warp carries lanes that skip it.  It takes the
// smallest such q of each prime (the one that shrinks the walk most): one
// power pair and one discrete logarithm per prime, the same code for every
// lane whatever its q (taking every q of the primes that have two or more
// ran the pass twice as long for the extra 1/q of their walks).
constexpr int POWRES_RARE_COUNT = 27;
CTD_HD uint32_t powres_rare_q(int i)
{
    constexpr uint8_t Q[POWRES_RARE_COUNT] = {11, 13, 17, 19, 23, 29, 31, 37, 41, 43, 47, 53, 59, 61, 67, 71,
                                              73, 79, 83, 89, 97, 101, 103, 107, 109, 113, 127};
    return Q[i];
}
// the rare q grouped into products below 2^32 (p - 1 is reduced once per
// group in 64 bits, then by each q in 32 bits): the group of q_i
constexpr int POWRES_RARE_GROUPS = 6;
CTD_HD int powres_rare_group(int i) { return i < 6 ? 0 : i < 11 ? 1 : i < 16 ? 2 : i < 20 ? 3 : i < 24 ? 4 : 5; }
// classes stay below 2^16: the walks' item code packs M and r in 16 bits
// each (a merge past it is dropped; the class stays sound, only wider)
constexpr uint32_t POWRES_MAX_M = 65535;

// the smallest rare q <= qmax dividing p - 1; 0 when there is none
CTD_HD uint32_t rare_q_of(uint64_t p, uint32_t qmax)
{
    const uint64_t p1 = p - 1;
    const uint32_t r[POWRES_RARE_GROUPS] = {
        (uint32_t)(p1 % (11ull * 13 * 17 * 19 * 23 * 29)), (uint32_t)(p1 % (31ull * 37 * 41 * 43 * 47)),
        (uint32_t)(p1 % (53ull * 59 * 61 * 67 * 71)),      (uint32_t)(p1 % (73ull * 79 * 83 * 89)),
        (uint32_t)(p1 % (97ull * 101 * 103 * 107)),        (uint32_t)(p1 % (109ull * 113 * 127))};
    uint32_t found = 0;
#pragma unroll
    for (int i = POWRES_RARE_COUNT - 1; i >= 0; --i) {
        const uint32_t q = powres_rare_q(i);
        found = q <= qmax && r[powres_rare_group(i)] % q == 0 ? q : found;
    }
    return found;
}

// j < q with z^j = y, for z of prime order q, 11 <= q <= 127 (baby steps
// z^0 .. z^7, giant steps by z^-8 = z^(q - 8)); q when there is none
template <class MT>
CTD_HD uint32_t small_log(const MT &m, uint64_t z, uint64_t y, uint32_t q)
{
    auto mul = [&](uint64_t a, uint64_t b) { return powres_mul<MT>(a, b, m.p, m.pinv); };
    uint64_t baby[8];
    baby[0] = m.one;
#pragma unroll
    for (int j = 1; j < 8; ++j)
        baby[j] = mul(baby[j - 1], z);
    const uint64_t g = small_pow(m, z, q - 8);
    uint64_t t = y;
    uint32_t found = q;
    for (uint32_t i = 0; 8 * i < q && found == q; ++i) {
#pragma unroll
        for (int j = 0; j < 8; ++j)
            if (t == baby[j] && 8 * i + j < q && found == q)
                found = 8 * i + j;
        t = mul(t, g);
    }
    return found;
}

// c (a class of doubling_class, M != 0) narrowed by the q-th power
// character of q = rare_q_of(p, ...) (0: unchanged): with z = 2^-(p-1)/q
// and y = wt^((p-1)/q), either z = 1 (no condition, or no zero at all when
// y != 1) or n = log_z y (mod q).  M divides 420 here (where 8 | p - 1, 2
// is a quadratic residue, so the 2-part of M is at most 4), so M q <= 420 *
// 127 = 53340 stays within POWRES_MAX_M without a check.
template <class MT>
CTD_HD PowerClass refine_class(const MT &m, uint64_t k, bool negate, PowerClass c, uint32_t q)
{
    if (!c.M || !q)
        return c;
    uint64_t z, y;
    power_pair(m, k, negate, (m.p - 1) / q, z, y);
    if (z == m.one)
        return y == m.one ? c : PowerClass{0, 0};
    const uint32_t j = small_log(m, z, y, q);
    if (j < q)  // always, for prime p
        crt_merge_small(c, j, q);
    return c;
}

// ---- the 9th-power character (9 | p - 1, one prime in six)
// Where the cubic character fixed n mod 3, the 9th-power one fixes n mod 9
// (z = 2^-(p-1)/9 of order 9), a third of the walk of those primes; over all
// primes the walked fraction drops by another 11 %.  Its own pass over the
// primes with 9 | p - 1 (after the rare-prime refinement): in the same pass
// as the rare q the lanes split between the two characters, and that pass
// took 60 % longer than the walk it saved.

// n = log_z y (mod o) for z of order o | 9, merged with c (M has at most one
// factor 3): the solution mod lcm(M, o), or false when there is none (y
// outside <z>, or a residue mod 3 that contradicts c's) -- no zero at all.
// A merge that would take M past POWRES_MAX_M is dropped.
template <class MT>
CTD_HD bool merge_nine(const MT &m, PowerClass &c, uint64_t z, uint64_t y)
{
    auto mul = [&](uint64_t a, uint64_t b) { return powres_mul<MT>(a, b, m.p, m.pinv); };
    uint64_t pw[9];
    pw[0] = m.one;
#pragma unroll
    for (int i = 1; i < 9; ++i)
        pw[i] = mul(pw[i - 1], z);
    const uint32_t o = z == m.one ? 1u : pw[3] == m.one ? 3u : 9u;
    uint32_t j = 9;
#pragma unroll
    for (int i = 8; i >= 0; --i)
        j = (uint32_t)i < o && pw[i] == y ? (uint32_t)i : j;
    if (j == 9)
        return false;
    const uint32_t f = c.M % 3 == 0 && o > 1 ? o / 3 : o;  // lcm(M, o) = M f
    uint32_t t = f;
    for (uint32_t tt = 0; tt < f; ++tt)
        t = t == f && (c.r + c.M * tt) % o == j ? tt : t;
    if (t == f)
        return false;
    if (c.M * f <= POWRES_MAX_M) {
        c.r += c.M * t;
        c.M *= f;
    }
    return true;
}

// c (M != 0) narrowed by the 9th-power character, for p with 9 | p - 1
template <class MT>
CTD_HD PowerClass nine_class(const MT &m, uint64_t k, bool negate, PowerClass c)
{
    if (!c.M)
        return c;
    uint64_t z, y;
    power_pair(m, k, negate, (m.p - 1) / 9, z, y);
    return merge_nine(m, c, z, y) ? c : PowerClass{0, 0};
}

}  // namespace ctd
