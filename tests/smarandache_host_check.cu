// Host-side check of the Smarandache jump (ctd_smarandache.cuh is
// __host__ __device__).  Reads "p b s" lines on stdin and prints
// "closed doubling chosen small" per line: Sm_b(s) mod p from the closed-form
// class jumps with simultaneous inversion, from the binary-doubling jumps,
// from the kernel's choice between them, and that choice in 32-bit
// Montgomery arithmetic (p < 2^31; the first value otherwise), with the
// 32-bit Shoup quotient of b mod p from its Montgomery form checked against
// the division (a mismatch prints -1).
#include <cinttypes>
#include <cstdio>

#include "../cutrialdive_gb300/csrc/ctd_smarandache.cuh"

int main()
{
    unsigned long long p, b, s;
    while (std::scanf("%llu %llu %llu", &p, &b, &s) == 3) {
        ctd::Mont m;
        m.init(p);
        const uint64_t closed = m.from(ctd::smarandache_at_closed(m, b, s));
        long long small = (long long)closed;
        if (p < (1ull << 31)) {
            ctd::Mont32 m32;
            m32.init(p);
            small = (long long)m32.from(ctd::smarandache_at(m32, b, s));
            const uint32_t w = (uint32_t)(b % p);
            if (m32.shoup_of_form(m32.to(w)) != ctd::shoup_precompute32(w, (uint32_t)p))
                small = -1;
        }
        std::printf("%" PRIu64 " %" PRIu64 " %" PRIu64 " %lld\n", closed, m.from(ctd::smarandache_at_doubling(m, b, s)),
                    m.from(ctd::smarandache_at(m, b, s)), small);
    }
    return 0;
}
