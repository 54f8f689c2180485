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

// n = r (mod M) and n = j (mod q), gcd(M, q) = 1  ->  one class mod M q
CTD_HD void crt_merge(PowerClass &c, uint32_t j, uint32_t q)
{
    uint32_t t = 0;
    while ((c.r + (uint64_t)c.M * t) % q != j)
        ++t;
    c.r += c.M * t;
    c.M *= q;
}

// The classifier's fixed chains multiply through one out-of-line function
// on the device (the two powering loops keep theirs inline): with all ~140
// Montgomery products inlined the kernel was large enough that warps
// stalled on instruction fetch (ncu: "no instruction" the top stall).
#ifdef __CUDA_ARCH__
__device__ __noinline__ uint64_t powres_mul(uint64_t a, uint64_t b, uint64_t p, uint64_t pinv)
{
    Mont m;
    m.p = p;
    m.pinv = pinv;
    return m.mul(a, b);
}
#else
inline uint64_t powres_mul(uint64_t a, uint64_t b, uint64_t p, uint64_t pinv)
{
    Mont m;
    m.p = p;
    m.pinv = pinv;
    return m.mul(a, b);
}
#endif

// base^e (base in Montgomery form, e small)
CTD_HD uint64_t small_pow(const Mont &m, uint64_t base, uint32_t e)
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
CTD_HD uint64_t square_n(const Mont &m, uint64_t x, int s)
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
CTD_HD Pow105 pow105(const Mont &m, uint64_t x)
{
    auto mul = [&](uint64_t a, uint64_t b) { return powres_mul(a, b, m.p, m.pinv); };
    const uint64_t x2 = mul(x, x), x3 = mul(x2, x), x5 = mul(x3, x2), x7 = mul(x5, x2);
    const uint64_t x10 = mul(x5, x5), x15 = mul(x10, x5), x14 = mul(x7, x7), x21 = mul(x14, x7);
    const uint64_t x35 = mul(x21, x14), x70 = mul(x35, x35), x105 = mul(x70, x35);
    return Pow105{x15, x21, x35, x105};
}

// The class of the zeros of 2^-n = wt (mod p), wt = -k (negate) or k, for
// an odd prime p < 2^63 and a plain k with k mod p != 0; m fully
// initialised (r2 is needed for k's Shoup quotient).  The work is the same
// for every prime -- two full powers, fixed chains, loops of fixed length
// -- so the lanes of a warp stay together.
CTD_HD PowerClass doubling_class(const Mont &m, uint64_t k, bool negate)
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
    auto mul = [&](uint64_t a, uint64_t b) { return powres_mul(a, b, p, m.pinv); };
    // A = 2^-e0 = 2^(p - 1 - e0) (left-to-right, a set bit a doubling); B =
    // wt^e0 = (-+1)^e0 k^e0 by left-to-right powering with Shoup
    // multiplications by the plain k
    uint64_t A = m.one;
    {
        const uint64_t e = p1 - e0;
        for (int b = 63 - clz64(e); b >= 0; --b) {
            A = m.mul(A, A);  // inline: the hot loops stay small
            if ((e >> b) & 1)
                A = m.dbl(A);
        }
    }
    uint64_t B = m.one;
    {
        const uint64_t kr = k < p ? k : k % p;
        const uint64_t ks = m.shoup(kr);
        for (int b = 63 - clz64(e0); b >= 0; --b) {
            B = m.mul(B, B);
            if ((e0 >> b) & 1)
                B = shoup_mul(B, kr, ks, p);
        }
        if (negate && (e0 & 1))
            B = B ? p - B : 0;
    }
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
            t = mul(t, z);
        }
        c.M = 1u << i;
        c.r = j;
    }
    // ---- q = 3, 5, 7: z = A^(2^u 105 / q)
    uint64_t A2 = A, B2 = B;  // A^(2^u), B^(2^u): loops of fixed length
#pragma unroll
    for (int t = 0; t < POWRES_MAX_2EXP; ++t) {
        const uint64_t a2 = mul(A2, A2), b2 = mul(B2, B2);
        A2 = t < u ? a2 : A2;
        B2 = t < u ? b2 : B2;
    }
    const Pow105 qa = pow105(m, A2), qb = pow105(m, B2);
    const uint64_t zq[3] = {qa.p35, qa.p21, qa.p15}, yq[3] = {qb.p35, qb.p21, qb.p15};
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
        for (uint32_t jj = 0; jj < q; ++jj) {
            if (t == y)
                j = jj;
            t = mul(t, z);
        }
        if (j >= q)  // cannot happen for prime p (y is a q-th root of unity)
            return PowerClass{1, 0};
        crt_merge(c, j, q);
    }
    return c;
}

}  // namespace ctd
