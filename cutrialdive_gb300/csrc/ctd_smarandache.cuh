// ctd_smarandache.cuh -- the jump to Sm_b(s) mod p for the Smarandache
// residue kernel (host and device: the same code runs in the host tests).
//
// Sm_b(n) = Sm_b(n-1) * b^len(n) + n (smarandache.hpp:131-198).  Within a
// digit class (all m with the same number d of base-b digits) the step is the
// affine map x -> M x + m with M = b^d, so the t steps m = c0 .. c0+t-1 give
//   x_t = M^t x + c0 G(t) + H(t),  G(t) = sum_{j<t} M^j,  H(t) = sum_{i<t} i M^(t-1-i).
// For M != 1 mod p these are geometric sums: G = (M^t - 1) / (M - 1) and
// H = (G - t) / (M - 1).  smarandache_at composes the classes 1 .. s with one
// modular inversion for all of them (Montgomery's simultaneous inversion: the
// prefix products of the (M_d - 1), one Fermat inversion of the last, and two
// multiplications per class to peel the individual inverses back off).  A
// class with M = 1 mod p, or more classes than the local tables hold, falls
// back to affine_jump, the same composition by binary doubling
//   G(2t) = G(t)(1 + M^t), H(2t) = M^t H(t) + t G(t) + H(t),
//   G(t+1) = M G(t) + 1,   H(t+1) = M H(t) + t.
// Either replaces the reference's reduction of the multi-limb Sm_b(n0)
// (src/trial_factoring.cuh:197-202) and costs O(log n) per digit class.
#pragma once

#include "ctd_arith.cuh"

namespace ctd {

// smallest power of b above m (the end of m's digit class) into pw and as
// the return value; ~0 when that power does not fit in 64 bits (every
// m < 2^64 above the previous power then has the same digit count)
CTD_HD uint64_t class_end(uint64_t b, uint64_t m, uint64_t &pw)
{
    pw = b;
    while (pw <= m) {
        if (pw > ~0ull / b) {
            pw = ~0ull;
            return pw;
        }
        pw *= b;
    }
    return pw;
}

// number of base-b digits of m >= 1
CTD_HD uint32_t digit_count(uint64_t b, uint64_t m)
{
    uint32_t d = 1;
    while (m >= b) {
        m /= b;
        ++d;
    }
    return d;
}

// the multiplier b^len(m) mod p (plain) of the digit class holding m, given
// class_end's pw for m
template <class MT>
CTD_HD uint64_t class_multiplier(const MT &m, uint64_t b, uint64_t mcur, uint64_t pw)
{
    if (pw != ~0ull)
        return pw < m.p ? pw : pw % m.p;
    return m.from(m.pow(m.to(b), digit_count(b, mcur)));
}

// X (Montgomery form) -> after the steps m = c0 .. c0+t-1 with multiplier Mm
// (Montgomery form).  Left-to-right over the bits of t, keeping (M^k, G(k),
// H(k), k) for the prefix k read so far; k itself is kept in Montgomery form
// (K) and updated by doubling and adding one, so no conversion is needed.
template <class MT>
CTD_HD uint64_t affine_jump(const MT &m, uint64_t X, uint64_t Mm, uint64_t c0, uint64_t t)
{
    if (!t)
        return X;
    uint64_t Mt = m.one, G = 0, H = 0, K = 0;
    bool started = false;
    for (int bit = 63 - clz64(t); bit >= 0; --bit) {
        if (started) {  // k -> 2k
            const uint64_t H2 = m.add(m.add(m.mul(Mt, H), m.mul(K, G)), H);
            G = m.mul(G, m.add(m.one, Mt));
            Mt = m.mul(Mt, Mt);
            H = H2;
            K = m.dbl(K);
        }
        if ((t >> bit) & 1) {  // k -> k + 1
            H = m.add(m.mul(Mm, H), K);
            G = m.add(m.mul(Mm, G), m.one);
            Mt = m.mul(Mm, Mt);
            K = m.add(K, m.one);
            started = true;
        }
    }
    return m.add(m.add(m.mul(Mt, X), m.mul(m.to(c0), G)), H);
}

// Sm_b(s) mod p in Montgomery form by class-by-class doubling jumps (needs
// m.r2).
template <class MT>
CTD_HD uint64_t smarandache_at_doubling(const MT &m, uint64_t b, uint64_t s)
{
    uint64_t X = 0;
    uint64_t c = 1;  // next m to apply
    while (c <= s) {
        uint64_t pw;
        const uint64_t cend = class_end(b, c, pw);  // class of c: [c, cend)
        const uint64_t last = cend - 1 < s ? cend - 1 : s;
        X = affine_jump(m, X, m.to(class_multiplier(m, b, c, pw)), c, last - c + 1);
        c = last + 1;
        if (cend == ~0ull || c == 0)
            break;
    }
    return X;
}

constexpr int SM_MAX_CLASSES = 24;

// Sm_b(s) mod p in Montgomery form by the closed-form class jumps (needs
// m.r2; p prime, for the Fermat inversion).
template <class MT>
CTD_HD uint64_t smarandache_at_closed(const MT &m, uint64_t b, uint64_t s)
{
    // the digit classes of 1 .. s: [lo_d, hi_d], multiplier Md (Montgomery form)
    uint64_t Mt[SM_MAX_CLASSES];   // M_d
    uint64_t inv[SM_MAX_CLASSES];  // prefix products of (M_d - 1), then their inverses
    uint32_t K = 0;
    uint64_t prod = m.one;
    for (uint64_t c = 1; c <= s;) {
        if (K == SM_MAX_CLASSES)
            return smarandache_at_doubling(m, b, s);
        uint64_t pw;
        const uint64_t cend = class_end(b, c, pw);
        const uint64_t Md = m.to(class_multiplier(m, b, c, pw));
        const uint64_t D = m.sub(Md, m.one);
        if (D == 0)  // M = 1 mod p: no geometric closed form for this class
            return smarandache_at_doubling(m, b, s);
        Mt[K] = Md;
        prod = m.mul(prod, D);
        inv[K] = prod;
        ++K;
        if (cend == ~0ull || cend > s)
            break;
        c = cend;
    }
    if (!K)
        return 0;
    // simultaneous inversion: inv_all = 1 / prod(D_0 .. D_{K-1}) by Fermat
    uint64_t ia = m.pow(prod, m.p - 2);
    for (int d = (int)K - 1; d >= 0; --d) {
        const uint64_t D = m.sub(Mt[d], m.one);
        const uint64_t before = d ? inv[d - 1] : m.one;  // prefix product of the classes below d
        inv[d] = m.mul(ia, before);                       // 1 / D_d
        ia = m.mul(ia, D);
    }
    // compose the classes in order
    uint64_t X = 0;
    uint64_t c = 1;
    for (uint32_t d = 0; d < K; ++d) {
        uint64_t pw;
        const uint64_t cend = class_end(b, c, pw);
        const uint64_t last = cend - 1 < s ? cend - 1 : s;
        const uint64_t t = last - c + 1;
        const uint64_t P = m.pow(Mt[d], t);                          // M^t
        const uint64_t G = m.mul(m.sub(P, m.one), inv[d]);          // (M^t - 1) / (M - 1)
        const uint64_t H = m.mul(m.sub(G, m.to(t)), inv[d]);         // (G - t) / (M - 1)
        X = m.add(m.add(m.mul(P, X), m.mul(m.to(c), G)), H);
        c = last + 1;
    }
    return X;
}

// Sm_b(s) mod p in Montgomery form: the cheaper composition by a
// multiplication count.  The doubling jumps cost about 5.5 multiplications
// per bit of each class length; the closed form about 1.5 per bit (the powers
// M^t), 8 per class and 1.5 per bit of p (the one inversion), so short
// prefixes -- a few classes of a few terms -- go by doubling.
template <class MT>
CTD_HD uint64_t smarandache_at(const MT &m, uint64_t b, uint64_t s)
{
    uint32_t bits = 0, classes = 0;
    for (uint64_t c = 1; c <= s;) {
        uint64_t pw;
        const uint64_t cend = class_end(b, c, pw);
        const uint64_t last = cend - 1 < s ? cend - 1 : s;
        bits += 64 - clz64(last - c + 1);
        ++classes;
        if (cend == ~0ull || cend > s)
            break;
        c = cend;
    }
    const uint32_t pbits = 64 - clz64(m.p);
    // both sides doubled: 11 bits  vs  3 bits + 16 K + 3 log p
    if (11 * bits <= 3 * bits + 16 * classes + 3 * pbits)
        return smarandache_at_doubling(m, b, s);
    return smarandache_at_closed(m, b, s);
}

}  // namespace ctd
