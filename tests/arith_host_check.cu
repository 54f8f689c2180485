// Host-side check of the device modular arithmetic (ctd_arith.cuh is
// __host__ __device__, so the same source runs on the CPU here).  Reads
// "p e k" lines on stdin, prints "one r2 pow2 kpow2 tok mu shoup" per line:
// R mod p, R^2 mod p, 2^e mod p, k*2^e mod p (Montgomery form times plain k),
// from(to(k)) for R = 2^64, floor(2^64 / p) and floor((k mod p) 2^64 / p).
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
        std::printf("%" PRIu64 " %" PRIu64 " %" PRIu64 " %" PRIu64 " %" PRIu64 " %" PRIu64 " %" PRIu64 "\n", m.one,
                    m.r2, m.from(U), m.mul(U, kk), m.from(m.to(k)), m.mu(), m.shoup(kk));
    }
    return 0;
}
