// Host-side check of the Smarandache jump (ctd_smarandache.cuh is
// __host__ __device__).  Reads "p b s" lines on stdin and prints
// "closed doubling chosen" per line: Sm_b(s) mod p from the closed-form class
// jumps with simultaneous inversion, from the binary-doubling jumps, and from
// the kernel's choice between them.
#include <cinttypes>
#include <cstdio>

#include "../cutrialdive_gb300/csrc/ctd_smarandache.cuh"

int main()
{
    unsigned long long p, b, s;
    while (std::scanf("%llu %llu %llu", &p, &b, &s) == 3) {
        ctd::Mont m;
        m.init(p);
        std::printf("%" PRIu64 " %" PRIu64 " %" PRIu64 "\n", m.from(ctd::smarandache_at_closed(m, b, s)),
                    m.from(ctd::smarandache_at_doubling(m, b, s)), m.from(ctd::smarandache_at(m, b, s)));
    }
    return 0;
}
