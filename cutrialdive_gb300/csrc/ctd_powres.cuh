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
// cyclic 2-group (Pohlig-Hellman, one bit a step).  The conditions are
// necessary, never sufficient: the walk still tests every n of the class
// exactly, so the hits are exactly the walk's (no hit is lost: an n outside
// the class cannot satisfy z^n = y).  Over random primes the class keeps
// about E[2^-v] * (2/3) * (4/5) * (6/7) ~ 0.15 of the terms (v = 2-adic
// valuation of p - 1, E[2^-v] = 1/3) for the primes 2, 3, 5, 7 used here.
//
// The same idea is the "Legendre symbol" filter of classical sieving
// programs for k*2^n+-1 (a prime where -k is a quadratic non-residue and 2
// a residue divides no term); here it is carried to the 2-power, 3rd, 5th
// and 7th power residues.  __host__ __device__ so the host tests run the
// same code.
#pragma once

#include "ctd_arith.cuh"

namespace ctd {

// largest power of 2 taken from p - 1 (2^6 = 64 classes at most)
constexpr int POWRES_MAX_2EXP = 6;

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

// The class of the zeros of 2^-n = wt (mod p), for an odd prime p and
// wt != 0 (Montgomery form WT, m fully initialised).
CTD_HD PowerClass doubling_class(const Mont &m, uint64_t WT)
{
    const uint64_t p = m.p;
    const uint64_t p1 = p - 1;
    int v = 0;
    while (!((p1 >> v) & 1))
        ++v;
    const int u = v < POWRES_MAX_2EXP ? v : POWRES_MAX_2EXP;
    const bool f3 = p1 % 3 == 0, f5 = p1 % 5 == 0, f7 = p1 % 7 == 0;
    // e0 = (p - 1) / D, D = 2^u 3^f3 5^f5 7^f7
    uint64_t e0 = p1 >> u;
    if (f3)
        e0 /= 3;
    if (f5)
        e0 /= 5;
    if (f7)
        e0 /= 7;
    const uint32_t Dq = (f3 ? 3u : 1u) * (f5 ? 5u : 1u) * (f7 ? 7u : 1u);  // odd part of D
    // A = 2^-e0 = 2^(p - 1 - e0), B = wt^e0
    const uint64_t A = m.pow2(p1 - e0);
    const uint64_t B = m.pow(WT, e0);
    PowerClass c{1, 0};
    // ---- the 2-power part: z = A^Dq has order 2^i, i <= u
    {
        const uint64_t z = small_pow(m, A, Dq);
        const uint64_t y = small_pow(m, B, Dq);
        int i = 0;
        for (uint64_t t = z; t != m.one && i < u; ++i)
            t = m.mul(t, t);
        if (square_n(m, y, i) != m.one)
            return PowerClass{0, 0};  // y outside <z>: no zero at all
        if (i > 0) {
            // Pohlig-Hellman in the cyclic group <z> of order 2^i: bit k of
            // the logarithm j is set iff (y z^-j_k)^(2^(i-1-k)) = -1
            const uint64_t zinv = square_n(m, z, i) == m.one ? small_pow(m, z, (1u << i) - 1) : m.one;
            uint32_t j = 0;
            for (int k = 0; k < i; ++k) {
                const uint64_t t = m.mul(y, small_pow(m, zinv, j));
                if (square_n(m, t, i - 1 - k) != m.one)
                    j |= 1u << k;
            }
            c.M = 1u << i;
            c.r = j;
        }
    }
    // ---- q = 3, 5, 7 when q | p - 1: z = A^(2^u Dq / q)
    const uint64_t A2 = square_n(m, A, u), B2 = square_n(m, B, u);
    const uint32_t qs[3] = {3, 5, 7};
    const bool fs[3] = {f3, f5, f7};
    for (int k = 0; k < 3; ++k) {
        if (!fs[k])
            continue;
        const uint32_t q = qs[k];
        const uint64_t z = small_pow(m, A2, Dq / q);
        const uint64_t y = small_pow(m, B2, Dq / q);
        if (z == m.one) {
            if (y != m.one)
                return PowerClass{0, 0};
            continue;
        }
        uint32_t j = 0;
        uint64_t t = m.one;
        while (t != y && j < q) {
            t = m.mul(t, z);
            ++j;
        }
        if (j >= q)  // cannot happen for prime p (y is a q-th root of unity)
            return PowerClass{1, 0};
        crt_merge(c, j, q);
    }
    return c;
}

}  // namespace ctd
