/*
 * primesieve compatibility header for compiling the reference CPU engine
 * here (primesieve is not installed).  generate_primes(start, stop, &v)
 * appends the primes in [start, stop] -- stop INCLUDED, as primesieve
 * documents -- computed by the oracle's own sieve.  Test infrastructure only.
 */
#ifndef CTD_REFSHIM_PRIMESIEVE_HPP
#define CTD_REFSHIM_PRIMESIEVE_HPP

#include <cstdint>
#include <vector>
#include "primesieve.h"

extern "C" uint64_t ctdo_sieve(uint64_t lo, uint64_t hi, uint64_t *out, uint64_t cap);

namespace primesieve {
template <typename T>
inline void generate_primes(uint64_t start, uint64_t stop, std::vector<T> *primes)
{
    if (stop < start)
        return;
    uint64_t hi = stop + 1; /* inclusive stop */
    if (hi == 0)
        hi = ~uint64_t{0};
    uint64_t n = ctdo_sieve(start, hi, nullptr, 0);
    std::vector<uint64_t> tmp(n);
    ctdo_sieve(start, hi, tmp.data(), n);
    primes->insert(primes->end(), tmp.begin(), tmp.end());
}
} // namespace primesieve

#endif
