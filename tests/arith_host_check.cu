// Host-side check of the device modular arithmetic (ctd_arith.cuh is
// __host__ __device__, so the same source runs on the CPU here).  Reads
// "p e k" lines on stdin, prints "one r2 pow2 kpow2 tok mu shoup" per line:
// R mod p, R^2 mod p, 2^e mod p, k*2^e mod p (Montgomery form times plain k),
// from(to(k)) for R = 2^64, floor(2^64 / p) and floor((k mod p) 2^64 / p);
// then, for p < 2^40 (0 0 otherwise), 2^e mod p and (k mod p)(k/2^7 mod p)
// R^-1 mod p through the narrow Montgomery product; then the Shoup quotient
// of k mod p without r2 (shoup_any), and of (k mod p) mod 64.
#include <cinttypes>
#include <cstdio>

#include "../cutrialdive_gb300/csrc/ctd_arith.cuh"

int main()
{
    unsigned long long p, e, k;
    while (std::scanf("%llu %llu %llu", &p, &e, &k) == 3) {
        ctd::Mont m;
        m.init(p);
        const uint64_t U = m.pow2(e);
        const uint64_t kk = k < p ? k : k % p;
        uint64_t npow = 0, nmul = 0;
        if (p < ctd::MONT_NARROW_LIMIT) {
            ctd::MontN n;
            n.init(p);
            npow = n.from(n.pow2(e));
            nmul = n.mul(kk, (k >> 7) % p);
        }
        ctd::Mont ml;
        ml.init_lite(p);  // no r2
        const uint64_t small = kk % 64 < p ? kk % 64 : 0;
        std::printf("%" PRIu64 " %" PRIu64 " %" PRIu64 " %" PRIu64 " %" PRIu64 " %" PRIu64 " %" PRIu64 " %" PRIu64
                    " %" PRIu64 " %" PRIu64 " %" PRIu64 " %" PRIu64 "\n",
                    m.one, m.r2, m.from(U), m.mul(U, kk), m.from(m.to(k)), m.mu(), m.shoup(kk), npow, nmul,
                    ml.shoup_any(kk), small, ml.shoup_any(small));
    }
    return 0;
}
