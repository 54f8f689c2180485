// ctd_arith.cuh -- device modular arithmetic for the residue kernels.
//
// The reference reduces with Barrett multipliers mu64/mu128 recomputed per
// prime (src/modular_arithmetic_detail.hpp:249-355, a 128/64 division per
// prime).  Here the per-prime set-up (the jump to the first index of a tile)
// uses Montgomery multiplication with R = 2^64 (Montgomery 1985), whose only
// division-like step is a Newton iteration for p^-1 mod 2^64, and the
// per-step loops use forms that need no division at all (doubling, addition,
// and Shoup's precomputed-quotient multiplication for Smarandache).  Every
// function returns the exact residue, so results equal the reference's.
#pragma once

#include <cstdint>

#define CTD_HD __host__ __device__ __forceinline__

namespace ctd {

// ---------------------------------------------------------------- helpers
CTD_HD uint64_t mulhi64(uint64_t a, uint64_t b)
{
#ifdef __CUDA_ARCH__
    return __umul64hi(a, b);
#else
    return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

CTD_HD uint32_t mulhi32(uint32_t a, uint32_t b)
{
#ifdef __CUDA_ARCH__
    return __umulhi(a, b);
#else
    return (uint32_t)(((uint64_t)a * b) >> 32);
#endif
}

CTD_HD int clz64(uint64_t x)
{
#ifdef __CUDA_ARCH__
    return __clzll((long long)x);
#else
    return x ? __builtin_clzll(x) : 64;
#endif
}

// a + b mod p for a, b < p < 2^64 (no overflow assumptions)
CTD_HD uint64_t addmod(uint64_t a, uint64_t b, uint64_t p)
{
    return a < p - b ? a + b : a - (p - b);
}

// a - b mod p for a, b < p
CTD_HD uint64_t submod(uint64_t a, uint64_t b, uint64_t p)
{
    return a >= b ? a - b : p - (b - a);
}

// 2a mod p for a < p
CTD_HD uint64_t dblmod(uint64_t a, uint64_t p)
{
    return a < p - a ? a << 1 : a - (p - a);
}

// ------------------------------------------------------- Montgomery, R=2^64
// a b R^-1 mod p for a, b < p < 2^40, from 32-bit pieces: a = a1 2^32 + a0
// with a1 < 2^9, so the product T = a b < 2^82 takes three multiply-adds
// into three words, m = T pinv mod 2^64 two more, and the high half of m p
// (p1 < 2^8) three, with one carry test; (T + m p) / 2^64 < p + T / 2^64
// < 2p, also for a, b < 2p (the lazy form skips the final subtraction).  Measured on
// chains of squarings: 14 % more products per second than the general form
// (fewer instructions, more of them on the multiply-add pipe).
// (the same before the final subtraction: < 2p, also for a, b < 2p)
CTD_HD uint64_t mont_mul_narrow_lazy(uint64_t a, uint64_t b, uint64_t p, uint64_t pinv)
{
    const uint32_t a0 = (uint32_t)a, a1 = (uint32_t)(a >> 32), b0 = (uint32_t)b, b1 = (uint32_t)(b >> 32);
    const uint64_t x = (uint64_t)a0 * b0;
    uint64_t y = (uint64_t)a0 * b1 + (x >> 32);
    y += (uint64_t)a1 * b0;                                // < 2^42
    const uint32_t t0 = (uint32_t)x, t1 = (uint32_t)y;
    const uint32_t t2 = (uint32_t)(y >> 32) + a1 * b1;     // T = t2 t1 t0
    const uint32_t pi0 = (uint32_t)pinv, pi1 = (uint32_t)(pinv >> 32);
    const uint64_t w = (uint64_t)t0 * pi0;
    const uint32_t m0 = (uint32_t)w;
    const uint32_t m1 = (uint32_t)(w >> 32) + t0 * pi1 + t1 * pi0;  // m = T pinv mod 2^64
    const uint32_t p0 = (uint32_t)p, p1 = (uint32_t)(p >> 32);
    const uint64_t s = (uint64_t)m0 * p0;
    const uint64_t t = (uint64_t)m0 * p1 + (s >> 32);     // < 2^41
    const uint64_t u = (uint64_t)m1 * p0 + t;             // the 2^32 column, mod 2^64
    const uint64_t carry = u < t ? (1ull << 32) : 0ull;
    const uint64_t mph = (uint64_t)m1 * p1 + (u >> 32) + carry;  // high half of m p
    // T + m p = 0 mod 2^64, with a carry out of the low half iff T's is not 0
    return (uint64_t)t2 + mph + ((t0 | t1) != 0);
}
CTD_HD uint64_t mont_mul_narrow(uint64_t a, uint64_t b, uint64_t p, uint64_t pinv)
{
    const uint64_t r = mont_mul_narrow_lazy(a, b, p, pinv);
    return r >= p ? r - p : r;
}

// Values are kept in Montgomery form xR mod p, in [0, p).  Valid for every
// odd p < 2^64 (NARROW: p < 2^40, products by mont_mul_narrow): the REDC sum
// below keeps its carry.
template <bool NARROW>
struct MontT {
    uint64_t p;     // odd modulus
    uint64_t pinv;  // -p^-1 mod 2^64
    uint64_t one;   // R mod p
    uint64_t r2;    // R^2 mod p

    CTD_HD static uint64_t neg_inverse(uint64_t p)
    {
        // Newton-Hensel lifting: x <- x(2 - px) doubles the correct low bits;
        // x = p is correct to 3 bits for odd p (p*p = 1 mod 8).
        uint64_t x = p;
        #pragma unroll
        for (int i = 0; i < 5; ++i)
            x *= 2 - p * x;
        return (uint64_t)0 - x;
    }

    // Everything but r2: enough for pow2/pow/mul/from and for mul(X, y)
    // with X in Montgomery form and y plain, which returns a plain X*y/R.
    CTD_HD void init_lite(uint64_t modulus)
    {
        p = modulus;
        pinv = neg_inverse(p);
        one = ((uint64_t)0 - p) % p;  // 2^64 mod p
        r2 = 0;
    }

    // Full set-up, r2 included (needed by to()).  R^2 = 2^64 * R is the
    // Montgomery form of 2^64: six Montgomery squarings of the form of 2.
    CTD_HD void init(uint64_t modulus)
    {
        init_lite(modulus);
        uint64_t x = dblmod(one, p);
        #pragma unroll
        for (int i = 0; i < 6; ++i)
            x = mul(x, x);
        r2 = x;
    }

    // a * b * R^-1 mod p, in [0, 2p) for a, b < 2p (NARROW; exact otherwise)
    CTD_HD uint64_t mul_lazy(uint64_t a, uint64_t b) const
    {
        if constexpr (NARROW)
            return mont_mul_narrow_lazy(a, b, p, pinv);
        return mul(a, b);
    }
    // x mod p for x < 2p
    CTD_HD uint64_t canon(uint64_t x) const { return x >= p ? x - p : x; }

    // a * b * R^-1 mod p for a, b < p
    CTD_HD uint64_t mul(uint64_t a, uint64_t b) const
    {
        if constexpr (NARROW)
            return mont_mul_narrow(a, b, p, pinv);
        uint64_t lo = a * b;
        uint64_t hi = mulhi64(a, b);
        uint64_t m = lo * pinv;
        uint64_t mh = mulhi64(m, p);
        // (hi:lo + mh:ml) / 2^64, where lo + ml == 0 mod 2^64 with a carry iff lo != 0
        uint64_t u = hi + mh;
        bool ov = u < hi;
        uint64_t c = lo != 0;
        u += c;
        ov |= u < c;
        if (ov || u >= p)
            u -= p;
        return u;
    }

    CTD_HD uint64_t to(uint64_t x) const { return mul(x < p ? x : x % p, r2); }
    CTD_HD uint64_t from(uint64_t X) const { return mul(X, 1); }
    CTD_HD uint64_t add(uint64_t a, uint64_t b) const { return addmod(a, b, p); }
    CTD_HD uint64_t sub(uint64_t a, uint64_t b) const { return submod(a, b, p); }
    CTD_HD uint64_t dbl(uint64_t a) const { return dblmod(a, p); }

    // floor(2^64 / p): 2^64 = mu p + (R mod p), so mu p = -one mod 2^64 and
    // mu = -one * p^-1 = one * pinv mod 2^64 (an exact division).
    CTD_HD uint64_t mu() const { return one * pinv; }

    // Shoup's precomputed quotient floor(w 2^64 / p) for a plain w < p
    // (needs r2).  w 2^64 = w mu p + w one, so the quotient is
    // w mu + floor(w one / p), and floor(w one / p) = (w one - (w one mod p)) / p
    // is again an exact division, by p^-1 mod 2^64; w one mod p = to(w).
    // Every product wraps mod 2^64; the result is exact because it is < 2^64.
    CTD_HD uint64_t shoup(uint64_t w) const
    {
        const uint64_t r = to(w);
        return w * mu() + (w * one - r) * ((uint64_t)0 - pinv);
    }

    // the same quotient without r2: with W = w R mod p (the Montgomery form
    // of w), w 2^64 = q p + W, so q = -W p^-1 = W pinv mod 2^64 (exact: q <
    // 2^64).  W from doublings and additions of R mod p for w < 64, else
    // from R^2 made here (six squarings of 2R)
    CTD_HD uint64_t shoup_any(uint64_t w) const
    {
        uint64_t W = 0;
        if (w < 64) {
#pragma unroll
            for (int b = 5; b >= 0; --b) {
                W = dblmod(W, p);
                if ((w >> b) & 1)
                    W = addmod(W, one, p);
            }
        } else {
            uint64_t x = dblmod(one, p);
#pragma unroll
            for (int i = 0; i < 6; ++i)
                x = mul(x, x);
            W = mul(w, x);
        }
        return W * pinv;
    }

    // (2^e) in Montgomery form: left-to-right binary powering in which a set
    // bit costs a modular doubling instead of a multiplication.
    CTD_HD uint64_t pow2(uint64_t e) const
    {
        if (e == 0)
            return one;
        int b = 63 - clz64(e);
        uint64_t r = dbl(one);
        while (b-- > 0) {
            r = mul(r, r);
            if ((e >> b) & 1)
                r = dbl(r);
        }
        return r;
    }

    // base^e in Montgomery form (base in Montgomery form)
    CTD_HD uint64_t pow(uint64_t base, uint64_t e) const
    {
        uint64_t r = one;
        while (e) {
            if (e & 1)
                r = mul(r, base);
            base = mul(base, base);
            e >>= 1;
        }
        return r;
    }
};
using Mont = MontT<false>;
using MontN = MontT<true>;  // p < 2^40
constexpr uint64_t MONT_NARROW_LIMIT = 1ull << 40;

// ------------------------------------------------------- Montgomery, R=2^32
// The same interface for an odd p < 2^31 (values in uint64, below p): a
// product is one 32x32 multiply, m = T pinv mod 2^32 and one multiply-add,
// (T + m p) / 2^32 < 2p -- a few instructions where the R = 2^64 form takes
// about forty.  For the per-prime set-up of walks whose primes fit 31 bits.
struct Mont32 {
    uint64_t p;
    uint64_t pinv;  // -p^-1 mod 2^32
    uint64_t one;   // 2^32 mod p
    uint64_t r2;    // 2^64 mod p

    CTD_HD void init(uint64_t modulus)
    {
        p = modulus;
        const uint32_t p32 = (uint32_t)p;
        uint32_t x = p32;  // p^-1 mod 2^32 by Newton-Hensel lifting
#pragma unroll
        for (int i = 0; i < 4; ++i)
            x *= 2u - p32 * x;
        pinv = (uint32_t)(0u - x);
        one = (uint64_t)(0xffffffffu % p32 + 1u) % p32;
        r2 = one * one % p;
    }
    CTD_HD uint64_t mul(uint64_t a, uint64_t b) const
    {
        const uint64_t T = a * b;  // < 2^62
        const uint32_t m = (uint32_t)T * (uint32_t)pinv;
        const uint64_t r = (T + (uint64_t)m * p) >> 32;
        return r >= p ? r - p : r;
    }
    CTD_HD uint64_t to(uint64_t x) const { return mul(x < p ? x : x % p, r2); }
    CTD_HD uint64_t from(uint64_t X) const { return mul(X, 1); }
    CTD_HD uint64_t add(uint64_t a, uint64_t b) const { return addmod(a, b, p); }
    CTD_HD uint64_t sub(uint64_t a, uint64_t b) const { return submod(a, b, p); }
    CTD_HD uint64_t dbl(uint64_t a) const { return dblmod(a, p); }
    CTD_HD uint64_t pow(uint64_t base, uint64_t e) const
    {
        uint64_t r = one;
        while (e) {
            if (e & 1)
                r = mul(r, base);
            base = mul(base, base);
            e >>= 1;
        }
        return r;
    }
    // Shoup's quotient floor(w 2^32 / p) of the plain w whose Montgomery form
    // is W: w 2^32 = q p + W, so q = -W p^-1 = W pinv mod 2^32 (exact: q < 2^32)
    CTD_HD uint32_t shoup_of_form(uint64_t W) const { return (uint32_t)W * (uint32_t)pinv; }
};

// ------------------------------------------------------ Shoup, 32-bit words
// x * w mod p with the precomputed quotient ws = floor(w * 2^32 / p)
// (Shoup, "NTL: A library for doing number theory"; also Harvey 2014).
// For any x < 2^32 and w < p < 2^31 the result lies in [0, 2p).
CTD_HD uint32_t shoup_precompute32(uint32_t w, uint32_t p)
{
    return (uint32_t)(((uint64_t)w << 32) / p);
}

}  // namespace ctd
