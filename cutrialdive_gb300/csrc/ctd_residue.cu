// ctd_residue.cu -- residue-propagation kernels for every sequence family.
//
// One work item = (odd prime p, index tile [s, e)).  The item jumps to
// S(s) mod p with a per-family O(log s) method, then walks the recurrence
// e-s-1 steps, pushing p into the factors buffer of every index whose
// residue is zero.  This is the work of trial_div_by_odd_primes
// (src/trial_factoring.cuh:156-228) and of its CPU twin
// trial_factorer::process_chunk (src/trial_factoring_impl.hpp:193-248),
// re-planned for the GPU:
//   * each family walks an equivalent recurrence with the fewest integer
//     operations per step (doubling / addition / Shoup multiply) and a
//     32-bit candidate test, replaying the few candidate blocks exactly;
//   * the jump makes any index tile a unit of work, so short prime lists
//     still fill the GPU (the reference walks [n0, n1) per prime only).
// Hits are exact: a prime is pushed for index n iff p | S(n), exactly the
// set the reference's Barrett propagation yields.
#include "ctd_arith.cuh"
#include "ctd_powres.cuh"
#include "ctd_smarandache.cuh"
#include "ctd_internal.h"

#include <atomic>
#include <mutex>
#include <new>
#include <vector>

namespace ctd {

namespace {
std::atomic<uint64_t> g_launches{0};
}

void note_kernel_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void note_kernel_launches(uint64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
uint64_t kernel_launch_count() { return g_launches.load(std::memory_order_relaxed); }

// ----------------------------------------------------------------- push
// Keeps a term's max_factors smallest primes once more primes than slots
// divide it.  Called together by the lanes `peers` pushing to the same
// term; `pending` lanes still hold a prime without a slot.  Each round the
// leader finds the largest value in the slots (an empty slot, 0, counts as
// larger than any prime); every pending lane whose prime is not below it
// gives up (values only decrease, so it never will be), and the lowest
// remaining lane replaces that value with its prime by an exchange.  Each
// successful exchange replaces the current largest value by a smaller one,
// so after all pushes the slots hold the smallest primes pushed, whatever
// their order -- the set of the reference's CPU engine, which walks the
// primes in ascending order.  A failed exchange (another push changed the
// slots) leaves the lane pending; the rounds are bounded.
__device__ __forceinline__ void push_overflow(unsigned long long *slots, uint32_t k, unsigned long long p, bool pending,
                                           uint32_t peers, int leader)
{
    const int lane = (int)(threadIdx.x & 31u);
    for (int round = 0; round < (1 << 16); ++round) {
        if (!__any_sync(peers, pending))
            return;
        unsigned long long m = 0, raw = 0;
        uint32_t j = 0;
        if (lane == leader) {
            // volatile loads: another SM's exchanges must show (the
            // exchange below checks what they read); an empty slot ends it
            for (uint32_t i = 0; i < k; ++i) {
                const unsigned long long v = *(volatile unsigned long long *)&slots[i];
                const unsigned long long key = v ? v : ~0ull;
                if (key > m) {
                    m = key;
                    raw = v;
                    j = i;
                    if (!v)
                        break;
                }
            }
        }
        m = __shfl_sync(peers, m, leader);
        raw = __shfl_sync(peers, raw, leader);
        j = __shfl_sync(peers, j, leader);
        if (pending && p >= m)
            pending = false;
        const uint32_t want = __ballot_sync(peers, pending);
        if (want && lane == __ffs(want) - 1 && atomicCAS(&slots[j], raw, p) == raw)
            pending = false;
    }
}

// factors_buffer push (src/device_factors_buffer.hpp:119-129): atomic slot
// reservation; the count keeps growing past the per-term capacity so the
// excess is visible to the host.  Beyond the capacity the reference's device
// push drops whatever arrives late; here the term keeps its smallest primes
// (push_overflow), which is deterministic and equals the CPU engine's
// result.  Warp-aggregated: the lanes that push to the same term at the same
// time (every prime divides a zero term such as T(1)) are grouped with a
// match, their leader reserves all their slots with one atomic, and each
// lane takes the slot of its rank -- one atomic per (warp, term) instead of
// one per lane; past the capacity the group shares push_overflow's scans.
// Slots past a term's count must be zero on entry.
__device__ __forceinline__ void push(const FactorsView &fb, uint64_t idx, uint64_t p)
{
    const uint32_t active = __activemask();
    const uint32_t peers = __match_any_sync(active, (unsigned long long)idx);
    const uint32_t lane = threadIdx.x & 31u;
    const int leader = __ffs(peers) - 1;
    uint32_t base = 0;
    if ((int)lane == leader)
        base = atomicAdd(&fb.counts[idx], (uint32_t)__popc(peers));
    base = __shfl_sync(peers, base, leader);
    const uint32_t pos = base + (uint32_t)__popc(peers & ((1u << lane) - 1u));
    unsigned long long *const slots = (unsigned long long *)(fb.factors + idx * fb.max_factors);
    // the reserved slot, unless a push beyond the term's capacity took it
    // first; beyond capacity, the term keeps its smallest primes
    const bool pending = !(pos < fb.max_factors && atomicCAS(&slots[pos], 0ull, (unsigned long long)p) == 0ull);
    if (__builtin_expect(__any_sync(peers, pending), 0))
        push_overflow(slots, fb.max_factors, p, pending, peers, leader);
}

// push out of line, for the baby-step families (doubling, fixed-n): one call
// per site keeps their short walks compact (with the push inlined at every
// site, walks of a few blocks ran 24 % slower), while an out-of-line push in
// the Smarandache walk's loop cost it 2.5x, so the others keep push inlined
__device__ __noinline__ void push_call(const FactorsView &fb, uint64_t idx, uint64_t p) { push(fb, idx, p); }

// ------------------------------------------------------- step primitives
// For p < 2^63 the modular double / add is: v = a + b - p (one 3-input add
// pair), then v += p under the sign of v (a predicated add pair) -- five
// 32-bit integer instructions, no compare-and-select on the unreduced value.
__device__ __forceinline__ uint64_t add63(uint64_t a, uint64_t b, uint64_t p)
{
    uint64_t v;
    asm("{\n\t.reg .pred neg;\n\t"
        "add.u64 %0, %1, %2;\n\t"
        "sub.u64 %0, %0, %3;\n\t"
        "setp.lt.s64 neg, %0, 0;\n\t"
        "@neg add.u64 %0, %0, %3;\n\t"
        "}"
        : "=l"(v)
        : "l"(a), "l"(b), "l"(p));
    return v;
}

__device__ __forceinline__ uint64_t dbl63(uint64_t u, uint64_t p) { return add63(u, u, p); }

// One step of u <- u + c (c = u for doubling) with the candidate test folded
// into the predicate `hit`: hit |= (low word of u == T).  A block whose low
// words never matched needs no further test; false candidates come at about
// 2^-32 per step.  (A test accumulated as a product of low-word differences
// on the multiply pipe was measured 10x slower: products of 32-bit words hit
// zero often enough -- about 7e-4 per 8-step block -- that the replays kept
// warps diverged for the rest of their walks.)
#define CTD_ADD_STEP(U, C, P, T)                 \
    "add.u64 " U ", " U ", " C ";\n\t"           \
    "sub.u64 " U ", " U ", " P ";\n\t"           \
    "setp.lt.s64 neg, " U ", 0;\n\t"             \
    "@neg add.u64 " U ", " U ", " P ";\n\t"      \
    "mov.b64 {lo, hi}, " U ";\n\t"               \
    "setp.eq.or.u32 hit, lo, " T ", hit;\n\t"

// R: any 32-bit register operand (clears `hit` by comparing it with itself)
#define CTD_BLOCK_HEAD(R) "{\n\t.reg .pred neg, hit;\n\t.reg .b32 lo, hi;\n\tsetp.ne.u32 hit, " R ", " R ";\n\t"
#define CTD_BLOCK_TAIL(OUT) "selp.u32 " OUT ", 1, 0, hit;\n\t}"

// Eight steps of u <- u + c mod p (c == u: doubling) in one block of PTX;
// returns nonzero when a low word equalled tlo (the target's low word).
template <bool DOUBLE>
__device__ __forceinline__ uint32_t step8_add63(uint64_t &u, uint64_t c, uint64_t p, uint32_t tlo)
{
    uint32_t cand;
    // operands: %0 = u, %1 = candidate flag, %2 = p, %3 = tlo, %4 = c
#define CTD_S8(C)                                                                                   \
    CTD_ADD_STEP("%0", C, "%2", "%3") CTD_ADD_STEP("%0", C, "%2", "%3") CTD_ADD_STEP("%0", C, "%2", "%3") \
    CTD_ADD_STEP("%0", C, "%2", "%3") CTD_ADD_STEP("%0", C, "%2", "%3") CTD_ADD_STEP("%0", C, "%2", "%3") \
    CTD_ADD_STEP("%0", C, "%2", "%3") CTD_ADD_STEP("%0", C, "%2", "%3")
    if (DOUBLE) {
        asm(CTD_BLOCK_HEAD("%3") CTD_S8("%0") CTD_BLOCK_TAIL("%1")
            : "+l"(u), "=r"(cand)
            : "l"(p), "r"(tlo), "l"(c));
    } else {
        asm(CTD_BLOCK_HEAD("%3") CTD_S8("%4") CTD_BLOCK_TAIL("%1")
            : "+l"(u), "=r"(cand)
            : "l"(p), "r"(tlo), "l"(c));
    }
#undef CTD_S8
    return cand;
}

constexpr int UNROLL = 8;

// Walks u -> step(u) for `steps` steps from index `idx`, pushing p wherever
// u == target.  The unrolled body only tests the low 32 bits (one compare
// per step); a block whose low words matched is replayed with the full test.
template <class Step>
__device__ __forceinline__ void walk_target(uint64_t u, uint64_t target, uint64_t p, uint64_t idx, uint64_t steps,
                                            const FactorsView &fb, Step step)
{
    if (u == target)
        push_call(fb, idx, p);
    const uint32_t tlo = (uint32_t)target;
    uint64_t i = 0;
    for (; i + UNROLL <= steps; i += UNROLL) {
        const uint64_t u0 = u;
        bool cand = false;
#pragma unroll
        for (int j = 0; j < UNROLL; ++j) {
            u = step(u);
            cand |= ((uint32_t)u == tlo);
        }
        if (cand) {
            uint64_t v = u0;
#pragma unroll 1
            for (int j = 0; j < UNROLL; ++j) {
                v = step(v);
                if (v == target)
                    push_call(fb, idx + i + j + 1, p);
            }
        }
    }
    for (; i < steps; ++i) {
        u = step(u);
        if (u == target)
            push_call(fb, idx + i + 1, p);
    }
}

// walk_target for u <- u + c (DOUBLE: u <- 2u) with p < 2^63, blocks of
// eight steps in PTX with 32-bit block counters; a candidate block is
// replayed from its saved start with the full 64-bit test.
template <bool DOUBLE>
__device__ __forceinline__ void walk_add63(uint64_t u, uint64_t c, uint64_t target, uint64_t p, uint64_t idx,
                                           uint64_t steps, const FactorsView &fb)
{
    if (u == target)
        push_call(fb, idx, p);
    const uint32_t tlo = (uint32_t)target;
    uint64_t nb = steps / UNROLL;
    uint64_t base = idx;  // index of the state before the current block
    while (nb) {
        const uint32_t chunk = nb > 0x40000000ull ? 0x40000000u : (uint32_t)nb;
        for (uint32_t b = 0; b < chunk; ++b) {
            const uint64_t u0 = u;
            if (step8_add63<DOUBLE>(u, c, p, tlo)) {
                uint64_t v = u0;
                const uint64_t at = base + (uint64_t)b * UNROLL;
#pragma unroll 1
                for (int j = 0; j < UNROLL; ++j) {
                    v = DOUBLE ? add63(v, v, p) : add63(v, c, p);
                    if (v == target)
                        push_call(fb, at + j + 1, p);
                }
            }
        }
        base += (uint64_t)chunk * UNROLL;
        nb -= chunk;
    }
    for (uint64_t i = base - idx; i < steps; ++i) {
        u = DOUBLE ? add63(u, u, p) : add63(u, c, p);
        if (u == target)
            push_call(fb, idx + i + 1, p);
    }
}

// p^-1 mod 2^32 for odd p (Newton-Hensel lifting from 3 correct bits)
__device__ __forceinline__ uint32_t inverse_mod_2_32(uint32_t p)
{
    uint32_t x = p;
#pragma unroll
    for (int i = 0; i < 4; ++i)
        x *= 2u - p * x;
    return x;
}

// ---------------------------------------------- lazily reduced blocks
// For p < 2^40 the linear recurrences run a block of steps on unreduced
// 64-bit values: from states below 3p, each step at most adds the previous
// two (three) values, so after step j of a block every value is below
// K[j] p, K growing like the recurrence itself (7752 p after 16 Fibonacci
// steps, 6627 p after 12 tribonacci steps: below 2^53).  A value x = k p,
// k < K[j], satisfies x_lo p^-1 = k mod 2^32, so "x_lo p^-1 mod 2^32 < K[j]"
// (one multiply, one compare) flags every zero; false candidates come at
// K[j] 2^-32 and are settled by an exact replay.  At the block's end each
// state is brought back below 3p by a Barrett step from one 32-bit high
// multiply (q = mulhi(x >> sh, mu) undershoots floor(x / p) by at most 2).
struct Lazy {
    uint64_t p;
    uint32_t pinv32;  // p^-1 mod 2^32
    uint32_t sh;      // floor(log2 p)
    uint32_t mu;      // floor(2^(sh+32) / p)
    uint32_t nplo, nphi;  // 2^64 - p

    __device__ __forceinline__ void init(const Mont &m)
    {
        p = m.p;
        pinv32 = inverse_mod_2_32((uint32_t)p);
        sh = 63 - clz64(p);
        const uint64_t mu64 = m.mu();
        mu = sh <= 32 ? (uint32_t)(mu64 >> (32 - sh)) : (uint32_t)((mu64 << (sh - 32)) + ((m.one << (sh - 32)) / p));
        const uint64_t np = (uint64_t)0 - p;
        nplo = (uint32_t)np;
        nphi = (uint32_t)(np >> 32);
    }
    // x < 2^(sh+32) -> a value = x mod p in [0, 3p)
    __device__ __forceinline__ uint64_t reduce(uint64_t x) const
    {
        const uint32_t top = (uint32_t)(x >> sh);
        const uint32_t q = __umulhi(top, mu);
        uint64_t r = (uint64_t)q * nplo + x;
        r += (uint64_t)(q * nphi) << 32;
        return r;
    }
    // x < 3p -> x mod p
    __device__ __forceinline__ uint64_t full(uint64_t x) const
    {
        x = x >= p ? x - p : x;
        return x >= p ? x - p : x;
    }
};

// ------------------------------------------- baby-step / giant-step walks
// For the recurrences whose step is an affine map of a single residue --
// u -> 2u (Proth, Riesel, Mersenne) and v -> v + c (the fixed-n pair) -- the
// test of BS consecutive terms needs no stepping: term idx + j is a zero of
// S iff the state at idx equals a per-prime "baby-step target" T_j (the
// target pulled back j steps: target * 2^-j, or target - j c).  A block of
// BS terms is then BS compares of the state's low word against the targets'
// low words, held in registers, and one giant step to the state BS terms on
// (a Montgomery multiplication by 2^BS, or one modular add of BS c).  The
// integer ALU, which bounds the per-step walk, does one compare per term
// instead of a modular add and a compare; the giant step's multiplication
// runs on the multiply pipe.  A block whose low words matched is replayed
// term by term with the full test, so results are those of the walk.
constexpr int BS = 32;

// Target filter of the baby-step blocks: per thread, 32 slots of two 32-bit
// words in shared memory.  A target's low word t is hashed once, h = t *
// FILTER_A; slot h >> 27 gets bit t mod 32 set in its first word and bit
// (h >> 22) mod 32 in its second.  A state whose low word equals a target
// always passes (both bits set); any other passes with probability about
// E[X^2]/32^2 = 2/1024 for the X ~ Poisson(1) targets in its slot, so the
// exact compares run for about 5 % of the warps' blocks.  A test is one
// 64-bit load and two funnel-shift bit tests (the funnel shift takes its
// amount mod 32, so no masking).  Layout: slot k of thread t at [k *
// blockDim.x + t] (conflict-free: the lanes of a warp read consecutive
// slots).
constexpr int FILTER_WORDS = 64;  // 32-bit words per thread
constexpr int FILTER_SLOTS = FILTER_WORDS / 2;
constexpr uint32_t FILTER_A = 0x9E3779B1u;  // odd multiplier of the hash
// blocks a prime needs before building its filter pays off
constexpr uint64_t FILTER_MIN_BLOCKS = 16;
extern __shared__ __align__(16) uint32_t ctd_filter_smem[];

template <uint32_t FAM>
constexpr bool uses_filter()
{
    return FAM == PROTH || FAM == RIESEL || FAM == MERSENNE;
}

struct TargetFilter {
    uint2 *col;       // this thread's slot 0
    uint32_t stride;  // slots between a thread's consecutive slots

    __device__ __forceinline__ TargetFilter()
        : col(reinterpret_cast<uint2 *>(ctd_filter_smem) + threadIdx.x), stride(blockDim.x)
    {
    }

    __device__ __forceinline__ uint2 &slot(uint32_t h) const { return col[(h >> 27) * stride]; }

    // marks the 32 targets' low words
    __device__ __forceinline__ void build(const uint32_t (&tlo)[BS]) const
    {
#pragma unroll 8
        for (int k = 0; k < FILTER_SLOTS; ++k)
            col[k * stride] = uint2{0, 0};
#pragma unroll 4
        for (int j = 0; j < BS; ++j) {
            const uint32_t t = tlo[j], h = t * FILTER_A;
            uint2 &sl = slot(h);
            sl.x |= 1u << (t & 31);
            sl.y |= 1u << ((h >> 22) & 31);
        }
    }

    // bit 0 set if lo may equal one of the targets (always when it does);
    // the other bits are arbitrary
    __device__ __forceinline__ uint32_t test(uint32_t lo) const
    {
        const uint32_t h = lo * FILTER_A;
        const uint2 sl = slot(h);
        return __funnelshift_r(sl.x, sl.x, lo) & __funnelshift_r(sl.y, sl.y, h >> 22);
    }
};

// halving mod odd p < 2^63: x/2 or (x + p)/2
__device__ __forceinline__ uint64_t half63(uint64_t x, uint64_t p) { return (x + ((x & 1) ? p : 0)) >> 1; }

// Nonzero iff lo equals one of the 32 targets t[K .. K+31]: 32 predicate-
// accumulating compares (one ALU instruction each) in four independent
// chains, merged into one flag.
#define CTD_M4(A, B, C, D)                                                                        \
    "setp.eq.or.u32 c0, %1, %" #A ", c0;\n\tsetp.eq.or.u32 c1, %1, %" #B ", c1;\n\t"           \
    "setp.eq.or.u32 c2, %1, %" #C ", c2;\n\tsetp.eq.or.u32 c3, %1, %" #D ", c3;\n\t"
template <int K = 0, int N = BS>
__device__ __forceinline__ uint32_t match32(uint32_t lo, const uint32_t (&t)[N])
{
    uint32_t f;
    asm("{\n\t.reg .pred c<4>;\n\t"
        "setp.eq.u32 c0, %1, %2;\n\tsetp.eq.u32 c1, %1, %3;\n\t"
        "setp.eq.u32 c2, %1, %4;\n\tsetp.eq.u32 c3, %1, %5;\n\t"
        CTD_M4(6, 7, 8, 9) CTD_M4(10, 11, 12, 13) CTD_M4(14, 15, 16, 17) CTD_M4(18, 19, 20, 21)
        CTD_M4(22, 23, 24, 25) CTD_M4(26, 27, 28, 29) CTD_M4(30, 31, 32, 33)
        "or.pred c0, c0, c1;\n\tor.pred c2, c2, c3;\n\tor.pred c0, c0, c2;\n\t"
        "selp.u32 %0, 1, 0, c0;\n\t}"
        : "=r"(f)
        : "r"(lo), "r"(t[K + 0]), "r"(t[K + 1]), "r"(t[K + 2]), "r"(t[K + 3]), "r"(t[K + 4]), "r"(t[K + 5]), "r"(t[K + 6]), "r"(t[K + 7]),
          "r"(t[K + 8]), "r"(t[K + 9]), "r"(t[K + 10]), "r"(t[K + 11]), "r"(t[K + 12]), "r"(t[K + 13]), "r"(t[K + 14]), "r"(t[K + 15]),
          "r"(t[K + 16]), "r"(t[K + 17]), "r"(t[K + 18]), "r"(t[K + 19]), "r"(t[K + 20]), "r"(t[K + 21]), "r"(t[K + 22]), "r"(t[K + 23]),
          "r"(t[K + 24]), "r"(t[K + 25]), "r"(t[K + 26]), "r"(t[K + 27]), "r"(t[K + 28]), "r"(t[K + 29]), "r"(t[K + 30]), "r"(t[K + 31]));
    return f;
}
#undef CTD_M4

// nb blocks of BS terms from state x, block numbers b0, b0 + 1, ..., with
// the 32 compares of every block and lane-wise replays of the rare matches;
// returns the state after them.  step(x) is the giant step to the next
// block's state; replay(x, b) re-walks block b term by term with the full
// test.
template <typename Step, typename Replay>
__device__ __forceinline__ uint64_t plain_blocks(const uint32_t (&tlo)[BS], uint64_t x, uint64_t b0, uint64_t nb,
                                                 Step step, Replay replay)
{
    for (uint64_t done = 0; done < nb;) {
        const uint32_t chunk = nb - done > 0x40000000ull ? 0x40000000u : (uint32_t)(nb - done);
        for (uint32_t bk = 0; bk < chunk; ++bk) {
            if (match32((uint32_t)x, tlo))
                replay(x, b0 + done + bk);
            x = step(x);
        }
        done += chunk;
    }
    return x;
}

// ng groups of FILTER_GROUP blocks from state x through the target filter,
// one warp vote a group; returns the state after them.  In a group with a
// passing lane, the blocks some lane passed get the exact compares (lanes
// that passed) and, on a match, the replay (all lanes together, so the warp
// never splits).  That path keeps only the group's first state and steps
// from it, so little stays live across the loop (the targets fill 32
// registers) and its code exists once.  Four blocks a group: over the
// power-residue classes, where most giant steps are 64-bit Shoup products,
// re-stepping into a group costs more than the extra votes (class walk on a
// 2^27 Proth segment: 2.25 ms with groups of 8, 2.17 with 4, 2.24 with 2).
constexpr int FILTER_GROUP = 4;
template <typename Step, typename Replay>
__device__ __forceinline__ uint64_t filtered_groups(const uint32_t (&tlo)[BS], uint64_t x, uint64_t ng, Step step,
                                                    Replay replay)
{
    const TargetFilter flt;
    flt.build(tlo);
    for (uint64_t done = 0; done < ng;) {
        const uint32_t chunk = ng - done > 0x10000000ull ? 0x10000000u : (uint32_t)(ng - done);
        for (uint32_t g = 0; g < chunk; ++g) {
            const uint64_t x0 = x;
            uint32_t fs[FILTER_GROUP], any = 0;
#pragma unroll
            for (int i = 0; i < FILTER_GROUP; ++i) {
                fs[i] = flt.test((uint32_t)x) & 1;
                any |= fs[i];
                x = step(x);
            }
            if (__any_sync(__activemask(), any)) {
                const uint32_t act = __activemask();
                uint32_t pass = 0;
#pragma unroll
                for (int i = 0; i < FILTER_GROUP; ++i)
                    pass |= fs[i] << i;
                // the blocks some lane passed, lowest first (warp-uniform)
                uint64_t z = x0;
                int at = 0;
                for (uint32_t todo = __reduce_or_sync(act, pass); todo; todo &= todo - 1) {
                    const int i = __ffs(todo) - 1;
                    for (; at < i; ++at)
                        z = step(z);
                    const uint32_t cand = (pass >> i) & 1 ? match32((uint32_t)z, tlo) : 0u;
                    if (__any_sync(act, cand))
                        replay(z, (done + g) * FILTER_GROUP + i);
                }
            }
        }
        done += chunk;
    }
    return x;
}

// the blocks of a range: filtered when it is long enough to pay for the
// filter (the last nb mod FILTER_GROUP blocks unfiltered)
template <typename Step, typename Replay>
__device__ __forceinline__ uint64_t run_blocks(const uint32_t (&tlo)[BS], uint64_t x, uint64_t nb, Step step,
                                               Replay replay)
{
    uint64_t b0 = 0;
    if (nb >= FILTER_MIN_BLOCKS) {
        x = filtered_groups(tlo, x, nb / FILTER_GROUP, step, replay);
        b0 = nb - nb % FILTER_GROUP;
    }
    return plain_blocks(tlo, x, b0, nb - b0, step, replay);
}

// u * 2^-32 mod p for u < p, odd p < 2^63: one 32-bit Montgomery reduction,
// m = u_lo (-p^-1) mod 2^32, r = (u + m p) / 2^32.  u + m p = 0 mod 2^32 and
// r < (p + 2^32 p) / 2^32, so r < p with no final subtraction; every step is
// a 32x32(+64) multiply-add on the multiply pipe (`one` is 1, passed at run
// time so the last add stays a multiply-add).
__device__ __forceinline__ uint64_t redc32(uint64_t u, uint32_t plo, uint32_t phi, uint32_t pinv32, uint32_t one)
{
    const uint32_t ulo = (uint32_t)u, uhi = (uint32_t)(u >> 32);
    const uint32_t m = ulo * pinv32;
    const uint64_t t1 = (uint64_t)m * plo + ulo;  // low word 0; high word carries
    const uint64_t h = (uint64_t)(uint32_t)(t1 >> 32) * one + uhi;
    return (uint64_t)m * phi + h;
}

// ------------------------------------------------------------- families

// Proth k*2^n+1, Riesel k*2^n-1, Mersenne 2^n-1 (riesel_proth.hpp:90-115,
// mersenne.hpp:256-303).  With u(n) = k*2^n mod p the recurrence
// S(n+1) = 2S(n) -+ 1 becomes pure doubling, and S(n) = 0 mod p becomes
// u == p-1 (Proth) or u == 1 (Riesel, Mersenne).
template <uint32_t FAM>
__device__ __forceinline__ void run_doubling(const JobView &job, uint64_t p, uint64_t s, uint64_t e)
{
    Mont m;
    m.init_lite(p);
    const uint64_t target = (FAM == PROTH) ? p - 1 : 1;
    const uint64_t steps = e - s - 1;
    // u(s) = k 2^s mod p, for the per-step walks
    auto start = [&]() {
        const uint64_t U = m.pow2(s);  // 2^s in Montgomery form
        if (FAM == MERSENNE)
            return m.from(U);
        // Montgomery form times a plain k leaves the plain k*2^s mod p
        const uint64_t k = job.param < p ? job.param : job.param % p;
        return m.mul(U, k);
    };
    if (p < (1ull << 63) && (e - s) / BS >= 2 && job.variant != CTD_VARIANT_WALK) {
        // Walk w(n) = 2^-n instead: k 2^n = -1 (Proth) / 1 (Riesel, Mersenne
        // with k = 1) mod p iff w(n) = -k / k, a fixed target, and the giant
        // step w -> w 2^-32 is one reduction on the multiply pipe (redc32).
        // Term n + j of a block starting at n is a zero iff w(n) = target 2^j.
        const uint64_t k = FAM == MERSENNE ? 1 : (job.param < p ? job.param : job.param % p);
        const uint64_t wt = (FAM == PROTH) ? (k ? p - k : 0) : k;  // target of w
        const uint64_t sr = s < p - 1 ? s : s % (p - 1);
        uint64_t w = m.from(m.pow2(p - 1 - sr));  // 2^-s mod p (Fermat)
        const uint64_t nb = (e - s) / BS;
        uint32_t tlo[BS];
        uint64_t t = wt;
#pragma unroll
        for (int j = 0; j < BS; ++j) {
            tlo[j] = (uint32_t)t;
            t = add63(t, t, p);
        }
        const uint32_t plo = (uint32_t)p, phi = (uint32_t)(p >> 32), pinv32 = (uint32_t)m.pinv;
        const uint32_t one = (uint32_t)(p & 1);
        const uint64_t at0 = s - job.n0;  // index of the first term
        auto giant = [&](uint64_t x) { return redc32(x, plo, phi, pinv32, one); };
        auto replay = [&](uint64_t v, uint64_t b) {
#pragma unroll 1
            for (int j = 0; j < BS; ++j) {
                if (v == wt)
                    push_call(job.fb, at0 + b * BS + j, p);
                v = half63(v, p);
            }
        };
        w = run_blocks(tlo, w, nb, giant, replay);
        for (uint64_t n = s + nb * BS; n < e; ++n) {  // the short tail, term by term
            if (w == wt)
                push_call(job.fb, n - job.n0, p);
            w = half63(w, p);
        }
    } else if (p < (1ull << 63))
        walk_add63<true>(start(), 0, target, p, s - job.n0, steps, job.fb);
    else
        walk_target(start(), target, p, s - job.n0, steps, job.fb, [p](uint64_t x) { return dblmod(x, p); });
}

// ------------------------------------- doubling over power-residue classes
// For long index ranges the doubling families first classify each prime
// (ctd_powres.cuh): every zero n of k*2^n-+1 (2^n-1) mod p satisfies
// n = r (mod M) for a class M | 2^3 * 3 * 5 * 7 read off the 2-power, 3rd,
// 5th and 7th power residues of 2 and of the target, and about 40 % of the
// primes (Proth k = 3) divide no term at all.  The walk then visits only
// n = r, r + M, r + 2M, ... with the same baby-step/giant-step blocks over
// w(n) = 2^-n: block b's 32 terms are zeros iff its state equals one of the
// targets wt * 2^(M j), the giant step multiplies by 2^-32M.  Every term of
// the class is still tested exactly, so the hits are those of the full walk.

// x * w mod p for x < 2^64, w < p < 2^63, with Shoup's quotient
// ws = floor(w 2^64 / p): x w - mulhi(x, ws) p lies in [0, 2p).
struct MulConst {
    uint64_t w, ws;
    __device__ __forceinline__ uint64_t mul(uint64_t x, uint64_t p) const
    {
        const uint64_t q = mulhi64(x, ws);
        const uint64_t r = x * w - q * p;
        return r >= p ? r - p : r;
    }
};

// the target of w(n) = 2^-n: -k (Proth), k (Riesel), 1 (Mersenne); 0 when p | k
template <uint32_t FAM>
__device__ __forceinline__ uint64_t doubling_target(const JobView &job, uint64_t p)
{
    const uint64_t k = FAM == MERSENNE ? 1 : (job.param < p ? job.param : job.param % p);
    return FAM == PROTH ? (k ? p - k : 0) : k;
}

// The doubling families for p >= 2^63 (beyond the classes' Shoup products):
// the term-by-term walk of u = k 2^n with carry-safe doubling, out of line so
// the class walks that call it for such primes keep their registers.
__device__ __noinline__ void run_doubling_wide(const JobView &job, uint64_t p, uint64_t s, uint64_t e)
{
    Mont m;
    m.init_lite(p);
    const uint64_t U = m.pow2(s);  // 2^s in Montgomery form
    uint64_t u;
    if (job.family == MERSENNE) {
        u = m.from(U);
    } else {
        const uint64_t k = job.param < p ? job.param : job.param % p;
        u = m.mul(U, k);  // Montgomery form times a plain k: the plain k 2^s mod p
    }
    const uint64_t target = job.family == PROTH ? p - 1 : 1;
    walk_target(u, target, p, s - job.n0, e - s - 1, job.fb, [p](uint64_t x) { return dblmod(x, p); });
}

// the target of w for the job's doubling family, chosen at run time
__device__ __forceinline__ uint64_t doubling_target_of(const JobView &job, uint64_t p)
{
    return job.family == PROTH    ? doubling_target<PROTH>(job, p)
           : job.family == RIESEL ? doubling_target<RIESEL>(job, p)
                                  : doubling_target<MERSENNE>(job, p);
}

// The doubling walk over n = r (mod M) in [s, e), p < 2^63.  One body for
// the three families (they differ only in the target), so the kernels that
// walk classes of several families hold one copy of it.
// 2^-x in Montgomery form: left-to-right powering of 2^-1, each set bit a
// halving of the Montgomery representative ((x R) / 2 = (x / 2) R) -- as many
// squarings as x has bits
__device__ __forceinline__ uint64_t pow_half(const Mont &m, uint64_t x)
{
    uint64_t h = m.one;
    for (int b = 63 - clz64(x | 1); b >= 0; --b) {
        h = m.mul(h, h);
        if ((x >> b) & 1)
            h = half63(h, m.p);
    }
    return h;
}

// x mod M, x / M for a class modulus M < 2^16 (32-bit division when x fits)
__device__ __forceinline__ uint32_t mod_small(uint64_t x, uint32_t M)
{
    return x >> 32 ? (uint32_t)(x % M) : (uint32_t)x % M;
}
__device__ __forceinline__ uint64_t div_small(uint64_t x, uint32_t M)
{
    return x >> 32 ? x / M : (uint32_t)x / M;
}

__device__ void run_doubling_class(const JobView &job, uint64_t p, uint32_t M, uint32_t r, uint64_t s, uint64_t e)
{
    const uint32_t sr = mod_small(s, M);
    const uint64_t off = r >= sr ? r - sr : M - sr + r;
    if (off >= e - s)
        return;
    const uint64_t nf = s + off;                   // first term of the class
    const uint64_t cnt = div_small(e - 1 - nf, M) + 1;  // terms nf, nf + M, ... below e
    // Shoup quotients straight from Montgomery forms: for W = w R mod p,
    // floor(w 2^64 / p) = (w 2^64 - W) / p = W (-p^-1) mod 2^64 = W pinv
    // (exact: the quotient is below 2^64), so no R^2 is needed
    Mont m;
    m.init_lite(p);
    const uint64_t wt = doubling_target_of(job, p);
    const uint64_t nr = nf < p - 1 ? nf : nf % (p - 1);
    uint64_t w = m.from(pow_half(m, nr));  // 2^-nf
    const uint64_t HM = pow_half(m, M);    // 2^-M in Montgomery form
    const MulConst step{m.from(HM), HM * m.pinv};  // w -> w 2^-M: the next term of the class
    const uint64_t at0 = nf - job.n0;
    uint64_t i = 0;
    if (cnt >= 2 * BS) {
        // targets wt 2^(M j), j < 32: term j of a block is a zero iff the
        // block's state equals target j
        const uint64_t C = m.pow2(M);
        const MulConst up{m.from(C), C * m.pinv};
        uint32_t tlo[BS];
        uint64_t t = wt;
#pragma unroll
        for (int j = 0; j < BS; ++j) {
            tlo[j] = (uint32_t)t;
            t = up.mul(t, p);
        }
        auto replay = [&](uint64_t v, uint64_t b) {
#pragma unroll 1
            for (int j = 0; j < BS; ++j) {
                if (v == wt)
                    push_call(job.fb, at0 + (b * BS + j) * M, p);
                v = step.mul(v, p);
            }
        };
        const uint64_t nb = cnt / BS;
        if (M <= 2) {
            // giant step w 2^-32M: one or two 32-bit Montgomery reductions
            // (a loop of M reductions for M up to 4, measured, ran the walk
            // 34 % slower than the 64-bit Shoup product for M = 3, 4)
            const uint32_t plo = (uint32_t)p, phi = (uint32_t)(p >> 32), pinv32 = (uint32_t)m.pinv;
            const uint32_t one = (uint32_t)(p & 1);
            if (M == 1)
                w = run_blocks(tlo, w, nb, [&](uint64_t x) { return redc32(x, plo, phi, pinv32, one); }, replay);
            else
                w = run_blocks(tlo, w, nb,
                               [&](uint64_t x) { return redc32(redc32(x, plo, phi, pinv32, one), plo, phi, pinv32, one); },
                               replay);
        } else {
            const uint64_t G = square_n(m, HM, 5);  // 2^-32M in Montgomery form
            const MulConst giant{m.from(G), G * m.pinv};
            w = run_blocks(tlo, w, nb, [&](uint64_t x) { return giant.mul(x, p); }, replay);
        }
        i = nb * BS;
    }
    for (; i < cnt; ++i) {  // the tail, term by term
        if (w == wt)
            push_call(job.fb, at0 + i * M, p);
        w = step.mul(w, p);
    }
}

// warp-aggregated atomicAdd of 1 per lane on counter[key] (lanes with the
// same key share one atomic); returns this lane's old value
__device__ __forceinline__ uint32_t aggregated_increment(uint32_t *counter, uint32_t key)
{
    const uint32_t act = __activemask();
    const uint32_t peers = __match_any_sync(act, key);
    const int leader = __ffs(peers) - 1;
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t base = 0;
    if ((int)lane == leader)
        base = atomicAdd(&counter[key], (uint32_t)__popc(peers));
    base = __shfl_sync(peers, base, leader);
    return base + (uint32_t)__popc(peers & ((1u << lane) - 1u));
}

// k*2^n +- 1 with fixed n over the index k (riesel_proth_fixed_n.hpp:88-151).
// The reference walks v(k) = k*2^n mod p term by term (S(k) = 0 iff v ==
// p-1 for Proth, v == 1 for Riesel).  The congruence is linear in k: p
// divides S(k) iff k = -+2^-n (mod p), so the zeros in [s, e) are k0, k0 + p,
// k0 + 2p, ... from the first k0 >= s of that class -- one power of 2 per
// prime and no walk; the pushed (k, p) pairs are exactly the walk's.
// CTD_VARIANT_WALK keeps the term-by-term walk (a second algorithm for the
// cross-checks).
template <uint32_t FAM>
__device__ __forceinline__ void run_fixed_n(const JobView &job, uint64_t p, uint64_t s, uint64_t e)
{
    Mont m;
    m.init_lite(p);
    if (job.variant == CTD_VARIANT_WALK) {
        const uint64_t C = m.pow2(job.param);  // 2^n in Montgomery form
        const uint64_t c = m.from(C);
        const uint64_t v = m.mul(C, s < p ? s : s % p);  // plain s*2^n mod p
        const uint64_t target = (FAM == PROTH_FIXED_N) ? p - 1 : 1;
        if (p < (1ull << 63))
            walk_add63<false>(v, c, target, p, s - job.n0, e - s - 1, job.fb);
        else
            walk_target(v, target, p, s - job.n0, e - s - 1, job.fb, [p, c](uint64_t x) { return addmod(x, c, p); });
        return;
    }
    // u = 2^-n = 2^(p-1-(n mod (p-1))) (Fermat; p odd, so 2 is invertible)
    const uint64_t nr = job.param < p - 1 ? job.param : job.param % (p - 1);
    const uint64_t u = m.from(m.pow2(p - 1 - nr));
    const uint64_t k0 = FAM == PROTH_FIXED_N ? p - u : u;  // u in [1, p-1]
    const uint64_t sr = s < p ? s : s % p;
    const uint64_t off = k0 >= sr ? k0 - sr : p - sr + k0;  // first k >= s with k = k0 (mod p)
    if (off >= e - s)
        return;
    for (uint64_t k = s + off;; k += p) {
        push(job.fb, k - job.n0, p);
        if (e - k <= p)
            break;
    }
}

// (F(k), F(k+1)) mod p in Montgomery form by the doubling identities
// F(2j) = F(j)(2F(j+1) - F(j)), F(2j+1) = F(j)^2 + F(j+1)^2.
__device__ __forceinline__ void fib_pair(const Mont &m, uint64_t k, uint64_t &fk, uint64_t &fk1)
{
    uint64_t a = 0, b = m.one;
    for (int bit = 63 - (k ? __clzll(k) : 63); k && bit >= 0; --bit) {
        uint64_t c = m.mul(a, m.sub(m.dbl(b), a));
        uint64_t d = m.add(m.mul(a, a), m.mul(b, b));
        if ((k >> bit) & 1) {
            a = d;
            b = m.add(c, d);
        } else {
            a = c;
            b = d;
        }
    }
    fk = a;
    fk1 = b;
}

// Odd primes below 2^20 for the trial division of the rank-of-apparition
// path, one 16-byte entry each: {q^-1 mod 2^64 (low, high word), high word
// of floor((2^64 - 1) / q), q}.  x = R q^-1 mod 2^64 equals R / q when q | R,
// which holds iff x q < 2^64; a high word of x above the bound's rules that
// out with one compare.  Filled once per device by prepare_residue_tables.
constexpr uint32_t TRIAL_LIMIT = 1u << 20;
constexpr uint32_t TRIAL_PRIMES = 82024;  // odd primes below 2^20
__device__ uint4 g_trial_div[TRIAL_PRIMES];

// number of table primes <= b (b < TRIAL_LIMIT)
__device__ __forceinline__ uint32_t trial_count(uint64_t b)
{
    uint32_t lo = 0, hi = TRIAL_PRIMES;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (g_trial_div[mid].w <= b)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

// Fibonacci / Lucas by the rank of apparition.  For a prime p other than 2
// and 5, p | F(n) iff a(p) | n, where a(p), the rank of apparition, divides
// D = p - (5/p) (Legendre symbol: +1 for p = +-1 mod 5, -1 for p = +-2);
// p | L(n) iff a(p) is even and n is an odd multiple of a(p)/2 (L(n) =
// F(2n)/F(n) and gcd(F(n), L(n)) | 2).  Hits in [s, e) need a(p) <= 2(e - 1),
// so every odd prime factor of a(p) is at most e - 1 (for Lucas it divides
// a(p)/2 <= e - 1): a(p) then divides S, the part of D built from 2 and the
// primes up to e - 1, found by trial division.  F(S) = 0 mod p tells whether
// it does; if so, a(p) is S reduced prime by prime while F stays zero.  The
// pushed (n, p) pairs are exactly those of the walk.  Needs s >= 1, odd
// p != 5 below 2^63 and e - 1 < TRIAL_LIMIT.
template <uint32_t FAM>
__device__ void run_fibonacci_rank(const JobView &job, uint64_t p, uint64_t s, uint64_t e)
{
    const uint64_t r5 = p % 5;
    const uint64_t D = (r5 == 1 || r5 == 4) ? p - 1 : p + 1;
    const uint64_t bmax = e - 1;  // largest prime factor that can matter
    const int v2 = __ffsll((long long)D) - 1;
    uint64_t R = D >> v2;  // part of D not yet factored
    uint64_t S = 1ull << v2;
    uint32_t fq[16], fv[16];
    int nf = 0;
    const uint32_t nq = trial_count(bmax);
    const uint4 *__restrict__ tab = g_trial_div;
    uint32_t i = 0;
    // 64 primes at a time; between rounds, stop once q^2 > R (R is then 1
    // or a prime)
    while (i < nq) {
        const uint32_t stop = nq - i > 64 ? i + 64 : nq;
#pragma unroll 8
        for (; i < stop; ++i) {
            const uint4 t = tab[i];
            const uint64_t inv = (uint64_t)t.y << 32 | t.x;
            uint64_t x = R * inv;
            if ((uint32_t)(x >> 32) <= t.z && __umul64hi(x, t.w) == 0) {
                uint32_t v = 0;
                do {  // x = R / q
                    R = x;
                    S *= t.w;
                    ++v;
                    x = R * inv;
                } while (__umul64hi(x, t.w) == 0);
                if (nf < 16) {
                    fq[nf] = t.w;
                    fv[nf] = v;
                }
                ++nf;
            }
        }
        if (i < nq) {
            const uint64_t q = tab[i].w;
            if (q * q > R)
                break;
        }
    }
    if (R > 1 && R <= bmax) {
        // stopped early with a prime cofactor no larger than bmax (after a
        // full pass R keeps only prime factors above bmax)
        if (nf < 16) {
            fq[nf] = (uint32_t)R;
            fv[nf] = 1;
        }
        ++nf;
        S *= R;
        R = 1;
    }
    Mont m;
    m.init(p);
    uint64_t f0, f1;
    fib_pair(m, S, f0, f1);
    if (f0 != 0)
        return;  // a(p) does not divide S: no hits below e
    // a(p): S with each prime taken out while F stays zero, the largest
    // primes first (D < 2^63 has at most 15 odd prime factors, so fq holds
    // them all).  Once a prime is done, its power in a(p) is final; when the
    // product of the final parts exceeds what the hits allow, stop.
    const uint64_t amax = FAM == FIBONACCI ? bmax : 2 * bmax;
    uint64_t a = S, fixed = 1;
    for (int k = (nf < 16 ? nf : 16) - 1; k >= -1; --k) {
        const uint64_t q = k >= 0 ? fq[k] : 2;
        const uint32_t v = k >= 0 ? fv[k] : (uint32_t)v2;
        uint32_t t = 0;
        for (; t < v; ++t) {
            fib_pair(m, a / q, f0, f1);
            if (f0 != 0)
                break;
            a /= q;
        }
        for (uint32_t r = t; r < v && fixed <= amax; ++r)
            fixed *= q;
        if (fixed > amax)
            return;
    }
    uint64_t first, step = a;
    if (FAM == FIBONACCI) {
        first = (s + a - 1) / a * a;
    } else {
        if (a & 1)
            return;
        const uint64_t h = a >> 1;  // n = h mod a
        const uint64_t r = s % a;
        first = s + (h >= r ? h - r : a - r + h);
    }
    for (uint64_t n = first; n < e; n += step)
        push(job.fb, n - job.n0, p);
}

// Fibonacci / Lucas: state (S(n-1), S(n)), one addmod per step
// (fibonacci.hpp:245-285, lucas.hpp:394-418).  The reference's
// make_state(0) leaves S(-1) = 0 and S(0) = 0, so a job starting at n0 = 0
// propagates zeros: every prime is recorded for every term.  That behaviour
// is kept (it is what the reference outputs).
template <uint32_t FAM>
__device__ __forceinline__ void run_fibonacci(const JobView &job, uint64_t p, uint64_t s, uint64_t e)
{
    // measured on a GB300, a table prime of the rank-of-apparition path costs
    // about 3.9 terms of the walk: taken when e - s > 3.9 pi(e), with pi(e) ~
    // e / ln e and ln e ~ 0.69 floor(log2 e), i.e. (e - s) floor(log2 e) >
    // 6 e (+4096 for its fixed cost)
    if (job.n0 != 0 && s != 0 && (p & 1) && p != 5 && p < (1ull << 62) && e <= TRIAL_LIMIT &&
        (e - s) * (uint64_t)(63 - __clzll(e)) > 6 * e + 4096 && job.variant != CTD_VARIANT_WALK) {
        run_fibonacci_rank<FAM>(job, p, s, e);
        return;
    }
    uint64_t a = 0, b = 0;  // (S(s-1), S(s))
    if (job.n0 != 0 && s != 0) {
        Mont m;
        m.init(p);
        uint64_t F0, F1;  // F(s-1), F(s)
        fib_pair(m, s - 1, F0, F1);
        if (FAM == LUCAS) {
            // L(s-1) = 2F(s) - F(s-1), L(s) = F(s) + 2F(s-1)
            uint64_t L0 = m.sub(m.dbl(F1), F0);
            uint64_t L1 = m.add(F1, m.dbl(F0));
            F0 = L0;
            F1 = L1;
        }
        a = m.from(F0);
        b = m.from(F1);
    }
    uint64_t idx = s - job.n0;
    const uint64_t steps = e - s - 1;
    if (b == 0)
        push(job.fb, idx, p);
    uint64_t i = 0;
    if (p < (1ull << 40)) {
        Mont mt;
        mt.init_lite(p);
        Lazy lz;
        lz.init(mt);
        constexpr int FB = 16;  // steps per block
        // bounds K[j] (in the PTX below): values after step j of a block are
        // below K[j] p = 6, 9, 15, 24, ... 7752 p (from states below 3p)
        uint64_t nb = steps / FB;
        while (nb) {
          const uint32_t chunk = nb > 0x40000000ull ? 0x40000000u : (uint32_t)nb;
          for (uint32_t bk = 0; bk < chunk; ++bk) {
            uint32_t cand;
            // a <- a + b, b <- b + a alternately ((a, b) is (S(n-1), S(n))
            // again after every second step); after each add the low word
            // times p^-1 is compared with the step's bound K[j].
            // operands: %0 = a, %1 = b, %2 = candidate flag, %3 = p^-1 mod 2^32
#define CTD_LZ_STEP(X, Y, KJ)                                                                  \
    "add.u64 " X ", " X ", " Y ";\n\tmov.b64 {lo, hi}, " X ";\n\tmul.lo.u32 t, lo, %3;\n\t"   \
    "setp.lt.or.u32 c, t, " #KJ ", c;\n\t"
            asm("{\n\t.reg .pred c;\n\t.reg .b32 lo, hi, t;\n\tsetp.ne.u32 c, %3, %3;\n\t"
                CTD_LZ_STEP("%0", "%1", 6) CTD_LZ_STEP("%1", "%0", 9) CTD_LZ_STEP("%0", "%1", 15)
                CTD_LZ_STEP("%1", "%0", 24) CTD_LZ_STEP("%0", "%1", 39) CTD_LZ_STEP("%1", "%0", 63)
                CTD_LZ_STEP("%0", "%1", 102) CTD_LZ_STEP("%1", "%0", 165) CTD_LZ_STEP("%0", "%1", 267)
                CTD_LZ_STEP("%1", "%0", 432) CTD_LZ_STEP("%0", "%1", 699) CTD_LZ_STEP("%1", "%0", 1131)
                CTD_LZ_STEP("%0", "%1", 1830) CTD_LZ_STEP("%1", "%0", 2961) CTD_LZ_STEP("%0", "%1", 4791)
                CTD_LZ_STEP("%1", "%0", 7752)
                "selp.u32 %2, 1, 0, c;\n\t}"
                : "+l"(a), "+l"(b), "=r"(cand)
                : "r"(lz.pinv32));
#undef CTD_LZ_STEP
            // the converged lanes replay together when any of them has a
            // candidate: a replay taken by some lanes only would leave the
            // warp diverged for the rest of the walk
            if (__any_sync(__activemask(), cand)) {
                // the block's values are exact integers: undo its FB adds to
                // recover the start, reduce it, and replay with the full test
                uint64_t x = a, y = b;
#pragma unroll 1
                for (int j = 0; j < FB; ++j) {
                    const uint64_t w = y - x;
                    y = x;
                    x = w;
                }
                x = lz.full(x);
                y = lz.full(y);
                const uint64_t at = idx + i + (uint64_t)bk * FB;
#pragma unroll 1
                for (int j = 0; j < FB; ++j) {
                    uint64_t c = add63(x, y, p);
                    x = y;
                    y = c;
                    if (c == 0)
                        push(job.fb, at + j + 1, p);
                }
            }
            a = lz.reduce(a);
            b = lz.reduce(b);
          }
          i += (uint64_t)chunk * FB;
          nb -= chunk;
        }
        a = lz.full(a);
        b = lz.full(b);
    } else if (p < (1ull << 63)) {
        const uint32_t zero = 0;
        constexpr int FB = 16;  // steps per block
        // blocks of FB steps counted in 32-bit chunks; the state at a block's
        // start is not saved: a block with a candidate steps back FB times
        // ((S(k-1), S(k)) -> (S(k) - S(k-1), S(k-1))) and replays
        uint64_t nb = steps / FB;
        while (nb) {
          const uint32_t chunk = nb > 0x40000000ull ? 0x40000000u : (uint32_t)nb;
          for (uint32_t bk = 0; bk < chunk; ++bk) {
            uint32_t cand;
            // a <- a + b, b <- b + a alternately: (a, b) is (S(n-1), S(n))
            // again after every second step, with no register moves
            // operands: %0 = a, %1 = b, %2 = candidate flag, %3 = p, %4 = 0
            asm(CTD_BLOCK_HEAD("%4")
                CTD_ADD_STEP("%0", "%1", "%3", "%4") CTD_ADD_STEP("%1", "%0", "%3", "%4")
                CTD_ADD_STEP("%0", "%1", "%3", "%4") CTD_ADD_STEP("%1", "%0", "%3", "%4")
                CTD_ADD_STEP("%0", "%1", "%3", "%4") CTD_ADD_STEP("%1", "%0", "%3", "%4")
                CTD_ADD_STEP("%0", "%1", "%3", "%4") CTD_ADD_STEP("%1", "%0", "%3", "%4")
                CTD_ADD_STEP("%0", "%1", "%3", "%4") CTD_ADD_STEP("%1", "%0", "%3", "%4")
                CTD_ADD_STEP("%0", "%1", "%3", "%4") CTD_ADD_STEP("%1", "%0", "%3", "%4")
                CTD_ADD_STEP("%0", "%1", "%3", "%4") CTD_ADD_STEP("%1", "%0", "%3", "%4")
                CTD_ADD_STEP("%0", "%1", "%3", "%4") CTD_ADD_STEP("%1", "%0", "%3", "%4")
                CTD_BLOCK_TAIL("%2")
                : "+l"(a), "+l"(b), "=r"(cand)
                : "l"(p), "r"(zero));
            if (cand) {
                uint64_t x = a, y = b;
#pragma unroll 1
                for (int j = 0; j < FB; ++j) {
                    const uint64_t w = submod(y, x, p);
                    y = x;
                    x = w;
                }
                const uint64_t at = idx + i + (uint64_t)bk * FB;
#pragma unroll 1
                for (int j = 0; j < FB; ++j) {
                    uint64_t c = add63(x, y, p);
                    x = y;
                    y = c;
                    if (c == 0)
                        push(job.fb, at + j + 1, p);
                }
            }
          }
          i += (uint64_t)chunk * FB;
          nb -= chunk;
        }
    }
    for (; i < steps; ++i) {
        uint64_t c = addmod(a, b, p);
        a = b;
        b = c;
        if (c == 0)
            push(job.fb, idx + i + 1, p);
    }
}

// (T(n), T(n+1), T(n+2)) mod p in Montgomery form by the doubling identities
// T(2j)   = 2T(j+2)T(j) + T(j+1)^2 - 2T(j+1)T(j) - T(j)^2
// T(2j+1) = T(j)^2 + 2T(j+2)T(j+1) - T(j+1)^2
// T(2j+2) = 2T(j+1)T(j) + T(j+2)^2 + T(j+1)^2
// (the formula section of OEIS A000073, as tribonacci.hpp:499-551 uses).
__device__ __forceinline__ void trib_triple(const Mont &m, uint64_t n, uint64_t &t0, uint64_t &t1, uint64_t &t2)
{
    uint64_t x = 0, y = 0, z = m.one;
    for (int bit = 63 - (n ? __clzll(n) : 63); n && bit >= 0; --bit) {
        uint64_t xx = m.mul(x, x), yy = m.mul(y, y);
        uint64_t xy2 = m.mul(m.dbl(y), x);
        uint64_t nx = m.sub(m.sub(m.add(m.mul(m.dbl(z), x), yy), xy2), xx);
        uint64_t ny = m.sub(m.add(xx, m.mul(m.dbl(z), y)), yy);
        uint64_t nz = m.add(m.add(xy2, m.mul(z, z)), yy);
        x = nx;
        y = ny;
        z = nz;
        if ((n >> bit) & 1) {
            uint64_t w = m.add(m.add(x, y), z);
            x = y;
            y = z;
            z = w;
        }
    }
    t0 = x;
    t1 = y;
    t2 = z;
}

// x <- x + y + z mod p for x, y, z < p < 2^62: the sum minus 2p, then p
// added back up to twice under the sign; the candidate test on the result.
// operands of the tribonacci block: %0..%2 = x, y, z, %3 = candidate flag,
// %4 = p, %5 = 2p, %6 = 0
#define CTD_TRIB_STEP(X, Y, Z)                   \
    "add.u64 " X ", " X ", " Y ";\n\t"           \
    "add.u64 " X ", " X ", " Z ";\n\t"           \
    "sub.u64 " X ", " X ", %5;\n\t"              \
    "setp.lt.s64 neg, " X ", 0;\n\t"             \
    "@neg add.u64 " X ", " X ", %4;\n\t"         \
    "setp.lt.s64 neg, " X ", 0;\n\t"             \
    "@neg add.u64 " X ", " X ", %4;\n\t"         \
    "mov.b64 {lo, hi}, " X ";\n\t"               \
    "setp.eq.or.u32 hit, lo, %6, hit;\n\t"

__device__ __forceinline__ uint64_t trib_add(uint64_t x, uint64_t y, uint64_t z, uint64_t p)
{
    return addmod(addmod(x, y, p), z, p);
}

// Tribonacci: state (T(n), T(n+1), T(n+2)), two addmods per step
// (tribonacci.hpp:566-590).  Each step computes T(n+3), which is the residue
// of index n+3: the first three indices are tested from the jump, then every
// new value at its own index, so the state rotates in place (x, y, z take
// turns holding the newest value) and the steps need no register moves.
__device__ __forceinline__ void run_tribonacci(const JobView &job, uint64_t p, uint64_t s, uint64_t e)
{
    Mont m;
    m.init(p);
    uint64_t X, Y, Z;
    trib_triple(m, s, X, Y, Z);
    uint64_t x = m.from(X), y = m.from(Y), z = m.from(Z);
    const uint64_t idx = s - job.n0;
    const uint64_t len = e - s;
    const uint64_t first[3] = {x, y, z};
    for (uint64_t j = 0; j < 3 && j < len; ++j)
        if (first[j] == 0)
            push(job.fb, idx + j, p);
    if (len <= 3)
        return;
    const uint64_t steps = len - 3;  // values T(s+3) .. T(e-1)
    uint64_t i = 0;                   // value T(s+3+i) goes to index idx+3+i
    if (p < (1ull << 40)) {
        Lazy lz;
        lz.init(m);
        constexpr int TB = 18;  // steps per block (a multiple of 3: the roles rotate back)
        // bounds K[j] (in the PTX below): values after step j of a block are
        // below K[j] p = 9, 15, 27, 51, ... 256575 p (from states below 3p;
        // K[j] = K[j-1] + K[j-2] + K[j-3]), so below 2^58 for p < 2^40 and
        // within Lazy::reduce's range (K < 2^31); a non-multiple passes the
        // test of step j with probability K[j] / 2^32, so a lane-block sees a
        // false candidate about once in 7600
        uint64_t nb = steps / TB;
        while (nb) {
          const uint32_t chunk = nb > 0x40000000ull ? 0x40000000u : (uint32_t)nb;
          for (uint32_t bk = 0; bk < chunk; ++bk) {
            uint32_t cand;
            // T(k+3) replaces T(k): the roles rotate every step
            // operands: %0..%2 = x, y, z, %3 = candidate flag, %4 = p^-1 mod 2^32
#define CTD_LZ3_STEP(X, Y, Z, KJ)                                                                         \
    "add.u64 " X ", " X ", " Y ";\n\tadd.u64 " X ", " X ", " Z ";\n\tmov.b64 {lo, hi}, " X ";\n\t"     \
    "mul.lo.u32 t, lo, %4;\n\tsetp.lt.or.u32 c, t, " #KJ ", c;\n\t"
            asm("{\n\t.reg .pred c;\n\t.reg .b32 lo, hi, t;\n\tsetp.ne.u32 c, %4, %4;\n\t"
                CTD_LZ3_STEP("%0", "%1", "%2", 9) CTD_LZ3_STEP("%1", "%2", "%0", 15)
                CTD_LZ3_STEP("%2", "%0", "%1", 27) CTD_LZ3_STEP("%0", "%1", "%2", 51)
                CTD_LZ3_STEP("%1", "%2", "%0", 93) CTD_LZ3_STEP("%2", "%0", "%1", 171)
                CTD_LZ3_STEP("%0", "%1", "%2", 315) CTD_LZ3_STEP("%1", "%2", "%0", 579)
                CTD_LZ3_STEP("%2", "%0", "%1", 1065) CTD_LZ3_STEP("%0", "%1", "%2", 1959)
                CTD_LZ3_STEP("%1", "%2", "%0", 3603) CTD_LZ3_STEP("%2", "%0", "%1", 6627)
                CTD_LZ3_STEP("%0", "%1", "%2", 12189) CTD_LZ3_STEP("%1", "%2", "%0", 22419)
                CTD_LZ3_STEP("%2", "%0", "%1", 41235) CTD_LZ3_STEP("%0", "%1", "%2", 75843)
                CTD_LZ3_STEP("%1", "%2", "%0", 139497) CTD_LZ3_STEP("%2", "%0", "%1", 256575)
                "selp.u32 %3, 1, 0, c;\n\t}"
                : "+l"(x), "+l"(y), "+l"(z), "=r"(cand)
                : "r"(lz.pinv32));
#undef CTD_LZ3_STEP
            if (__any_sync(__activemask(), cand)) {  // lanes replay together (see the Fibonacci block)
                // exact integers within the block: undo its TB adds
                uint64_t a = x, b = y, c = z;
#pragma unroll 1
                for (int j = 0; j < TB; ++j) {
                    const uint64_t w = c - b - a;
                    c = b;
                    b = a;
                    a = w;
                }
                a = lz.full(a);
                b = lz.full(b);
                c = lz.full(c);
                const uint64_t at = idx + 3 + i + (uint64_t)bk * TB;
#pragma unroll 1
                for (int j = 0; j < TB; ++j) {
                    uint64_t w = trib_add(a, b, c, p);
                    a = b;
                    b = c;
                    c = w;
                    if (w == 0)
                        push(job.fb, at + j, p);
                }
            }
            x = lz.reduce(x);
            y = lz.reduce(y);
            z = lz.reduce(z);
          }
          i += (uint64_t)chunk * TB;
          nb -= chunk;
        }
        x = lz.full(x);
        y = lz.full(y);
        z = lz.full(z);
    } else if (p < (1ull << 62)) {
        constexpr int TB = 12;  // steps per block
        const uint32_t zero = 0;
        const uint64_t p2 = 2 * p;
        // blocks of TB steps counted in 32-bit chunks; a block with a
        // candidate steps back TB times ((T(k), T(k+1), T(k+2)) ->
        // (T(k+2) - T(k+1) - T(k), T(k), T(k+1))) and replays
        uint64_t nb = steps / TB;
        while (nb) {
          const uint32_t chunk = nb > 0x40000000ull ? 0x40000000u : (uint32_t)nb;
          for (uint32_t bk = 0; bk < chunk; ++bk) {
            uint32_t cand;
            asm(CTD_BLOCK_HEAD("%6")
                CTD_TRIB_STEP("%0", "%1", "%2") CTD_TRIB_STEP("%1", "%2", "%0")
                CTD_TRIB_STEP("%2", "%0", "%1") CTD_TRIB_STEP("%0", "%1", "%2")
                CTD_TRIB_STEP("%1", "%2", "%0") CTD_TRIB_STEP("%2", "%0", "%1")
                CTD_TRIB_STEP("%0", "%1", "%2") CTD_TRIB_STEP("%1", "%2", "%0")
                CTD_TRIB_STEP("%2", "%0", "%1") CTD_TRIB_STEP("%0", "%1", "%2")
                CTD_TRIB_STEP("%1", "%2", "%0") CTD_TRIB_STEP("%2", "%0", "%1")
                CTD_BLOCK_TAIL("%3")
                : "+l"(x), "+l"(y), "+l"(z), "=r"(cand)
                : "l"(p), "l"(p2), "r"(zero));
            if (cand) {
                uint64_t a = x, b = y, c = z;
#pragma unroll 1
                for (int j = 0; j < TB; ++j) {
                    const uint64_t w = submod(submod(c, b, p), a, p);
                    c = b;
                    b = a;
                    a = w;
                }
                const uint64_t at = idx + 3 + i + (uint64_t)bk * TB;
#pragma unroll 1
                for (int j = 0; j < TB; ++j) {
                    uint64_t w = trib_add(a, b, c, p);
                    a = b;
                    b = c;
                    c = w;
                    if (w == 0)
                        push(job.fb, at + j, p);
                }
            }
          }
          i += (uint64_t)chunk * TB;
          nb -= chunk;
        }
    }
    for (; i < steps; ++i) {
        uint64_t w = trib_add(x, y, z, p);
        x = y;
        y = z;
        z = w;
        if (w == 0)
            push(job.fb, idx + 3 + i, p);
    }
}

// ----------------------------------------------------------- Smarandache
// The jump to Sm_b(s) mod p (class_end, affine_jump, smarandache_at) lives in
// ctd_smarandache.cuh; the walks below step within one digit class.

// Steps m = mm .. mend-1 of x <- x M + m (x in [1, 3p), M < p, Ms its Shoup
// quotient); SMALL: M < 2^32.  Returns the final x.
template <bool SMALL>
__device__ __forceinline__ uint64_t smarandache_walk64(const JobView &job, uint64_t p, uint64_t x, uint64_t M,
                                                       uint64_t Ms, uint64_t mm, uint64_t mend)
{
    const uint32_t plo = (uint32_t)p, p2lo = (uint32_t)(2 * p);
    auto step = [&](uint64_t v, uint64_t mv) {
        const uint64_t q = mulhi64(v, Ms);
        const uint64_t vm = SMALL ? v * (uint64_t)(uint32_t)M : v * M;
        return vm + mv - q * p;
    };
    while (mm + UNROLL <= mend) {
        const uint64_t x0 = x;
        bool cand = false;
#pragma unroll
        for (int j = 0; j < UNROLL; ++j) {
            x = step(x, mm + j);
            cand |= ((uint32_t)x == plo) | ((uint32_t)x == p2lo);
        }
        if (cand) {
            uint64_t y = x0;
#pragma unroll 1
            for (int j = 0; j < UNROLL; ++j) {
                y = step(y, mm + j);
                if (y == p || y == 2 * p)
                    push(job.fb, (mm + j) - job.n0, p);
            }
        }
        mm += UNROLL;
    }
    for (; mm < mend; ++mm) {
        x = step(x, mm);
        if (x == p || x == 2 * p)
            push(job.fb, mm - job.n0, p);
    }
    return x;
}

// Steps m = mm .. mend-1 of x <- x M + m with a Barrett quotient from one
// 32x32 high multiply: for 2^sh <= p < 2^(sh+1), mu = floor(2^(sh+32) / p)
// (< 2^32), T = x M + m < 2^(sh+32), q = mulhi(T >> sh, mu) is within 2 of
// floor(T / p) from below, so x' = T - q p stays in [0, 3p) and
// x = 0 mod p <=> x in {0, p, 2p}.  T and T - q p are multiply-adds
// (T - q p = T + q (2^64 - p) mod 2^64).  Needs 3p M + e < 2^64 and
// 3M + 1 <= 2^31 (checked by the caller).  WIDE: sh >= 32.
template <bool WIDE>
__device__ __forceinline__ uint64_t smarandache_walk_b32(const JobView &job, uint64_t p, uint64_t x, uint32_t M,
                                                         uint32_t sh, uint32_t mu, uint64_t mm, uint64_t mend)
{
    const uint64_t np = (uint64_t)0 - p;
    const uint32_t nplo = (uint32_t)np, nphi = (uint32_t)(np >> 32);
    // low words of p and 2p (the multiply pipe bounds this walk, so the zero
    // test stays three compares on the ALU rather than one multiply)
    const uint32_t plo = (uint32_t)p, p2lo = (uint32_t)(2 * p);
    auto step = [&](uint64_t v, uint64_t mv) {
        uint64_t T = (uint64_t)(uint32_t)v * M + mv;
        T += (uint64_t)((uint32_t)(v >> 32) * M) << 32;
        const uint32_t top = WIDE ? ((uint32_t)(T >> 32) >> (sh - 32)) : __funnelshift_r((uint32_t)T, (uint32_t)(T >> 32), sh);
        const uint32_t q = __umulhi(top, mu);
        uint64_t r = (uint64_t)q * nplo + T;
        r += (uint64_t)(q * nphi) << 32;
        return r;
    };
    while (mm + UNROLL <= mend) {
        const uint64_t x0 = x;
        bool cand = false;
#pragma unroll
        for (int j = 0; j < UNROLL; ++j) {
            x = step(x, mm + j);
            const uint32_t lo = (uint32_t)x;
            cand |= (lo == 0u) | (lo == plo) | (lo == p2lo);
        }
        if (cand) {
            uint64_t y = x0;
#pragma unroll 1
            for (int j = 0; j < UNROLL; ++j) {
                y = step(y, mm + j);
                if (y == 0 || y == p || y == 2 * p)
                    push(job.fb, (mm + j) - job.n0, p);
            }
        }
        mm += UNROLL;
    }
    for (; mm < mend; ++mm) {
        x = step(x, mm);
        if (x == 0 || x == p || x == 2 * p)
            push(job.fb, mm - job.n0, p);
    }
    return x;
}

__device__ __forceinline__ void run_smarandache(const JobView &job, uint64_t p, uint64_t s, uint64_t e)
{
    const uint64_t b = job.param;
    uint64_t mcur = s + 1;  // m = n + 1 of the next step
    if (p < (1u << 30) && p >= e && e <= 0xffffffffull && job.variant != CTD_VARIANT_MONTGOMERY) {
        // 32-bit Shoup path: x kept in [0, 3p) (Shoup output < 2p, plus m < p),
        // so x = 0 mod p <=> x == p or x == 2p (x >= 1 after a step).  The
        // set-up (the jump to Sm_b(s), the class multipliers and their Shoup
        // quotients) in 32-bit Montgomery arithmetic: with the 64-bit form it
        // was about 40 % of the instructions of base 10 over n = 10..1000
        // (991 steps a prime) with every prime below 2^28
        Mont32 m;
        m.init(p);
        const uint64_t X = smarandache_at(m, b, s);
        if (X == 0)
            push(job.fb, s - job.n0, p);
        const uint32_t p32 = (uint32_t)p, p2 = 2 * p32;
        uint32_t x = (uint32_t)m.from(X);
        while (mcur < e) {
            uint64_t pw;
            uint64_t cend = class_end(b, mcur, pw);
            const uint32_t M = (uint32_t)class_multiplier(m, b, mcur, pw);
            const uint32_t Ms = m.shoup_of_form(m.to(M));
            uint32_t mm = (uint32_t)mcur;
            const uint32_t mend = (uint32_t)(cend < e ? cend : e);
            while (mm + UNROLL <= mend) {
                const uint32_t x0 = x;
                bool cand = false;
#pragma unroll
                for (int j = 0; j < UNROLL; ++j) {
                    uint32_t q = mulhi32(x, Ms);
                    x = x * M + (mm + j) - q * p32;
                    cand |= (x == p32) | (x == p2);
                }
                if (cand) {
                    uint32_t y = x0;
#pragma unroll 1
                    for (int j = 0; j < UNROLL; ++j) {
                        uint32_t q = mulhi32(y, Ms);
                        y = y * M + (mm + j) - q * p32;
                        if (y == p32 || y == p2)
                            push(job.fb, (mm + j) - job.n0, p);
                    }
                }
                mm += UNROLL;
            }
            for (; mm < mend; ++mm) {
                uint32_t q = mulhi32(x, Ms);
                x = x * M + mm - q * p32;
                if (x == p32 || x == p2)
                    push(job.fb, mm - job.n0, p);
            }
            mcur = mend;
        }
        return;
    }
    Mont m;
    m.init(p);
    uint64_t X = smarandache_at(m, b, s);
    if (X == 0)
        push(job.fb, s - job.n0, p);
    if (p < (1ull << 62) && e <= p && job.variant != CTD_VARIANT_MONTGOMERY) {
        // 64-bit Shoup path (every m < p): x kept in [1, 3p) as r + m with
        // r = x M - q p in [0, 2p), q = mulhi(x, floor(M 2^64 / p)); so
        // x = 0 mod p <=> x == p or x == 2p.  The unrolled body tests the low
        // words only; a block with a candidate is replayed with the full test.
        uint64_t x = m.from(X);
        // Barrett-32 constants (p < 2^48): sh = floor(log2 p), mu = floor(2^(sh+32) / p)
        const uint32_t sh = 63 - clz64(p);
        uint32_t mu = 0;
        if (p < (1ull << 48) && job.variant == CTD_VARIANT_AUTO) {
            const uint64_t mu64 = m.mu();
            mu = sh <= 32 ? (uint32_t)(mu64 >> (32 - sh))
                          : (uint32_t)((mu64 << (sh - 32)) + ((m.one << (sh - 32)) / p));
        }
        while (mcur < e) {
            uint64_t pw;
            const uint64_t cend = class_end(b, mcur, pw);
            const uint64_t mend = cend < e ? cend : e;
            const uint64_t M = class_multiplier(m, b, mcur, pw);
            // Barrett-32 when 3pM + e < 2^64 and 3M + 1 <= 2^31 (x < 3p on entry either way)
            const bool b32 = mu && M < (1ull << 29) && M * 3 + 1 <= (1ull << 31) && p <= (~0ull - e) / (3 * M + 1);
            if (b32 && sh >= 32)
                x = smarandache_walk_b32<true>(job, p, x, (uint32_t)M, sh, mu, mcur, mend);
            else if (b32)
                x = smarandache_walk_b32<false>(job, p, x, (uint32_t)M, sh, mu, mcur, mend);
            else if (M >> 32)
                x = smarandache_walk64<false>(job, p, x, M, m.shoup(M), mcur, mend);
            else
                x = smarandache_walk64<true>(job, p, x, M, m.shoup(M), mcur, mend);
            mcur = mend;
        }
        return;
    }
    // general path: Montgomery form, X' = X * (M R) + m R
    const uint64_t Rm = m.one;
    uint64_t C = m.to(mcur);
    while (mcur < e) {
        uint64_t pw;
        uint64_t cend = class_end(b, mcur, pw);
        const uint64_t Mm = m.to(class_multiplier(m, b, mcur, pw));
        const uint64_t mend = cend < e ? cend : e;
        for (; mcur < mend; ++mcur) {
            X = m.add(m.mul(X, Mm), C);
            C = m.add(C, Rm);
            if (X == 0)
                push(job.fb, mcur - job.n0, p);
        }
    }
}

// Peano S(n) = n, the reference's engine test sequence (tests/peano.hpp).
__device__ __forceinline__ void run_peano(const JobView &job, uint64_t p, uint64_t s, uint64_t e)
{
    uint64_t r = s % p;
    for (uint64_t n = s;; ++n) {
        if (r == 0)
            push(job.fb, n - job.n0, p);
        if (n + 1 >= e)
            break;
        r = (r + 1 == p) ? 0 : r + 1;
    }
}

// Resident CTAs of 256 threads the register budget is sized for: the
// baby-step families keep 32 targets in registers, the linear recurrences
// and Smarandache carry block-start copies and reduction constants, the
// fixed-n solve and Peano hold a few values.
constexpr int min_ctas_per_sm(uint32_t fam)
{
    return fam == PEANO ? 6 : (fam == PROTH || fam == RIESEL || fam == MERSENNE) ? 3 : 4;
}

template <uint32_t FAM>
__device__ __forceinline__ void run_item(const JobView &job, uint64_t p, uint64_t s, uint64_t e)
{
    if (FAM == PROTH || FAM == RIESEL || FAM == MERSENNE)
        run_doubling<FAM>(job, p, s, e);
    else if (FAM == PROTH_FIXED_N || FAM == RIESEL_FIXED_N)
        run_fixed_n<FAM>(job, p, s, e);
    else if (FAM == FIBONACCI || FAM == LUCAS)
        run_fibonacci<FAM>(job, p, s, e);
    else if (FAM == TRIBONACCI)
        run_tribonacci(job, p, s, e);
    else if (FAM == SMARANDACHE)
        run_smarandache(job, p, s, e);
    else
        run_peano(job, p, s, e);
}

// one (prime, tile) item: item k is tile k mod tiles of prime k / tiles
template <uint32_t FAM>
__device__ __forceinline__ void residue_item(const JobView &job, const uint64_t *__restrict__ primes, uint64_t k)
{
    if (job.tiles == 1) {
        run_item<FAM>(job, primes[k], job.n0, job.n1);
        return;
    }
    const uint64_t i = k / job.tiles;
    const uint64_t t = k - i * job.tiles;
    const uint64_t s = job.n0 + t * job.tile_len;
    const uint64_t e = s + job.tile_len < job.n1 ? s + job.tile_len : job.n1;
    if (s < e)
        run_item<FAM>(job, primes[i], s, e);
}

// Persistent grid.  With a work counter (zero at launch) each warp takes
// the next 32 items until none are left, so an SM that runs slower than the
// others -- or holds the costliest primes -- simply takes fewer items and
// every SM finishes within one item of the others; without one, threads
// stride over the items.
template <uint32_t FAM>
__global__ void __launch_bounds__(256, min_ctas_per_sm(FAM))
residue_kernel(JobView job, const uint64_t *__restrict__ primes, uint64_t nprimes, unsigned long long *next)
{
    const uint64_t items = nprimes * job.tiles;
    if (!next) {
        const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
        for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < items; k += stride)
            residue_item<FAM>(job, primes, k);
        return;
    }
    const uint32_t lane = threadIdx.x & 31u;
    for (;;) {
        unsigned long long base = 0;
        if (lane == 0)
            base = atomicAdd(next, 32ull);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= items)
            break;
        if (base + lane < items)
            residue_item<FAM>(job, primes, base + lane);
    }
}

// ------------------------------------------ classified doubling launches
// classify -> regroup -> walk, all on the stream, no host wait:
//   classify_kernel: each prime's class code and a count per class;
//   regroup_kernel:  the primes (with their codes) written class by class,
//                    smallest M (the longest walks) first;
//   class_walk_kernel: a persistent grid whose warps take 32 consecutive
//                    (prime, tile) items from a counter, so a warp's lanes
//                    walk classes of the same M -- equal lengths, no lane
//                    waiting on a longer one.
// Buckets rank the classes by M: M <= 840 by the number of divisors of 840
// below it (a divisor's own rank; a class with a rare prime, M = 11, 22, 13,
// ..., shares the bucket of the next divisor), M above 840 by half octaves.
__device__ __forceinline__ uint32_t class_bucket(uint32_t M)
{
    if (M > 840) {
        const uint32_t b = 31 - __clz(M);  // 9 .. 15
        const uint32_t h = (uint64_t)M * M >= (2ull << (2 * b)) ? 1u : 0u;
        const uint32_t f = 2 * b + h;  // 19 .. 31
        return 32 + (f - 19 < CLASS_BUCKETS - 33 ? f - 19 : CLASS_BUCKETS - 33);
    }
    uint32_t rank = 0;
#pragma unroll
    for (int i = 0; i <= POWRES_MAX_2EXP; ++i)
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const uint32_t d = (1u << i) * ((q & 1) ? 3u : 1u) * ((q & 2) ? 5u : 1u) * ((q & 4) ? 7u : 1u);
            rank += d < M;
        }
    return rank;
}

// the largest rare prime of a job's refinement
__device__ __forceinline__ uint32_t refine_qmax(const JobView &job) { return job.refine_q ? job.refine_q : 127u; }

// whether a classified prime goes to the rare-prime refinement
__device__ __forceinline__ bool wants_refine(const JobView &job, uint64_t p, uint32_t code)
{
    return code && p < (1ull << 63) && rare_q_of(p, refine_qmax(job)) != 0;
}

// whether a classified prime goes to the 9th-power character's pass
__device__ __forceinline__ bool wants_nine(const JobView &job, uint64_t p, uint32_t code)
{
    return code && p < (1ull << 63) && refine_qmax(job) >= 11 && (p - 1) % 9 == 0;
}

// the code of a classified prime narrowed by the 9th-power character
template <uint32_t FAM, class MT>
__device__ __forceinline__ uint32_t nine_code(const JobView &job, uint64_t p, uint32_t code)
{
    const uint64_t k = FAM == MERSENNE ? 1 : (job.param < p ? job.param : job.param % p);
    MT m;
    m.init_lite(p);  // the power pairs need no R^2
    const PowerClass c = nine_class(m, k, FAM == PROTH, PowerClass{code >> 16, code & 0xffffu});
    return c.M ? (c.M << 16) | c.r : 0u;
}

// the refined code of a classified prime (0: it divides no term)
template <uint32_t FAM, class MT>
__device__ __forceinline__ uint32_t refined_code(const JobView &job, uint64_t p, uint32_t code, uint32_t q)
{
    const uint64_t k = FAM == MERSENNE ? 1 : (job.param < p ? job.param : job.param % p);
    MT m;
    m.init_lite(p);  // the power pairs need no R^2
    const PowerClass c = refine_class(m, k, FAM == PROTH, PowerClass{code >> 16, code & 0xffffu}, q);
    return c.M ? (c.M << 16) | c.r : 0u;
}

// The quadratic screen (Proth, Riesel): the primes whose target is a
// quadratic non-residue while 2 is a residue (a quarter of them) divide no
// term and get code 0 here; the others are listed for classify_kernel, so
// its warps spend the two powers on primes that need them.  Every family:
// cc->wide is set when a prime is 2^40 or above (the class kernels then take
// the general Montgomery product instead of the narrow one).
// Tiles of 256 x SCREEN_PER_THREAD primes per CTA: the listed primes are
// counted per pattern in shared memory and each tile takes its places in
// the eight lists with one global atomic per pattern (a global atomic per
// pattern and warp doubled the kernel's time).
constexpr int SCREEN_PER_THREAD = 8;
template <uint32_t FAM>
__global__ void __launch_bounds__(256) screen_kernel(JobView job, const uint64_t *__restrict__ primes,
                                                     uint64_t nprimes, uint32_t *__restrict__ codes,
                                                     ClassCounters *__restrict__ cc, uint32_t *__restrict__ listed,
                                                     uint64_t cap)
{
    __shared__ uint32_t hist[8], tile_base[8];
    const uint32_t tid = threadIdx.x;
    const uint64_t tile = (uint64_t)blockDim.x * SCREEN_PER_THREAD;
    bool wide = false;
    for (uint64_t t0 = (uint64_t)blockIdx.x * tile; t0 < nprimes; t0 += (uint64_t)gridDim.x * tile) {
        if (tid < 8)
            hist[tid] = 0;
        __syncthreads();
        uint32_t pat[SCREEN_PER_THREAD], off[SCREEN_PER_THREAD];
#pragma unroll
        for (int j = 0; j < SCREEN_PER_THREAD; ++j) {
            const uint64_t i = t0 + (uint64_t)j * blockDim.x + tid;
            pat[j] = 8;  // nothing to list
            if (i < nprimes) {
                const uint64_t p = primes[i];
                wide |= p >= MONT_NARROW_LIMIT;
                if (FAM != MERSENNE && quadratic_excluded(p, job.param, FAM == PROTH))
                    codes[i] = 0;
                else
                    pat[j] = powres_pattern(p);
            }
            if (pat[j] < 8)
                off[j] = aggregated_increment(hist, pat[j]);
        }
        __syncthreads();
        if (tid < 8)
            tile_base[tid] = hist[tid] ? atomicAdd(&cc->nlisted[tid], hist[tid]) : 0u;
        __syncthreads();
#pragma unroll
        for (int j = 0; j < SCREEN_PER_THREAD; ++j)
            if (pat[j] < 8)
                listed[pat[j] * cap + tile_base[pat[j]] + off[j]] = (uint32_t)(t0 + (uint64_t)j * blockDim.x + tid);
        __syncthreads();
    }
    if (wide)
        cc->wide = 1;
}

// the class code of a prime whose divisibility pattern is PAT
template <uint32_t FAM, int PAT, class MT>
__device__ __forceinline__ uint32_t class_code_pat(const JobView &job, uint64_t p)
{
    if (p >= (1ull << 63))
        return 1u << 16;
    const uint64_t k = FAM == MERSENNE ? 1 : (job.param < p ? job.param : job.param % p);
    if (!k)
        return 0;
    MT m;
    m.init_lite(p);  // the power pairs need no R^2
    const PowerClass c = doubling_class_pat<PAT>(m, k, FAM == PROTH);
    return c.M ? (c.M << 16) | c.r : 0u;
}

template <uint32_t FAM, int PAT, class MT>
__device__ __forceinline__ void classify_range(const JobView &job, const uint64_t *__restrict__ primes, uint64_t n,
                                               uint32_t *__restrict__ codes, ClassCounters *__restrict__ cc,
                                               uint32_t *__restrict__ refine, uint8_t *__restrict__ refine_q,
                                               uint32_t *__restrict__ nine, const uint32_t *__restrict__ listed)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += stride) {
        const uint64_t i = listed[t];
        const uint64_t p = primes[i];
        const uint32_t code = class_code_pat<FAM, PAT, MT>(job, p);
        codes[i] = code;
        const uint32_t q = code && p < (1ull << 63) ? rare_q_of(p, refine_qmax(job)) : 0u;
        if (q) {
            const uint32_t at = aggregated_increment(&cc->nrefine, 0);
            refine[at] = (uint32_t)i;
            refine_q[at] = (uint8_t)q;
        }
        else if (wants_nine(job, p, code))
            nine[aggregated_increment(&cc->nnine, 0)] = (uint32_t)i;
        else if (code)
            aggregated_increment(cc->count, class_bucket(code >> 16));
    }
}

// the classes of the primes the screen listed under divisibility pattern
// PAT, by the narrow Montgomery product unless the screen saw a prime of
// 2^40 or more (one launch per pattern: every lane of a launch runs the
// same chains)
template <uint32_t FAM, int PAT>
__global__ void __launch_bounds__(256, 4) classify_kernel(JobView job, const uint64_t *__restrict__ primes,
                                                       uint32_t *__restrict__ codes, ClassCounters *__restrict__ cc,
                                                       uint32_t *__restrict__ refine, uint8_t *__restrict__ refine_q,
                                                       uint32_t *__restrict__ nine, const uint32_t *__restrict__ listed,
                                                       uint64_t cap)
{
    const uint64_t n = cc->nlisted[PAT];
    if (cc->wide)
        classify_range<FAM, PAT, Mont>(job, primes, n, codes, cc, refine, refine_q, nine, listed + PAT * cap);
    else
        classify_range<FAM, PAT, MontN>(job, primes, n, codes, cc, refine, refine_q, nine, listed + PAT * cap);
}

// Tiles of 256 x REFINE_PER_THREAD listed primes per CTA, sorted by their q
// in shared memory before the powers: the logarithm's giant steps, z^(q-8)
// and the inverse mod q run as long as the warp's largest q, so warps of
// like q keep their lanes busy (in list order 22 of 32 lanes were active).
constexpr int REFINE_PER_THREAD = 2;
template <uint32_t FAM, class MT>
__device__ __forceinline__ void refine_range(const JobView &job, const uint64_t *__restrict__ primes,
                                             uint32_t *__restrict__ codes, ClassCounters *__restrict__ cc,
                                             const uint32_t *__restrict__ refine, const uint8_t *__restrict__ refine_q,
                                             uint32_t *__restrict__ nine, uint32_t n)
{
    constexpr uint32_t TILE = 256 * REFINE_PER_THREAD;
    __shared__ uint32_t start[128];  // per q: the tile's count, then its first place
    __shared__ uint32_t sorted_i[TILE];
    __shared__ uint8_t sorted_q[TILE];
    const uint32_t tid = threadIdx.x;
    for (uint64_t t0 = (uint64_t)blockIdx.x * TILE; t0 < n; t0 += (uint64_t)gridDim.x * TILE) {
        if (tid < 128)
            start[tid] = 0;
        __syncthreads();
        uint32_t idx[REFINE_PER_THREAD], q[REFINE_PER_THREAD], off[REFINE_PER_THREAD];
        bool valid[REFINE_PER_THREAD];
#pragma unroll
        for (int j = 0; j < REFINE_PER_THREAD; ++j) {
            const uint64_t t = t0 + (uint64_t)j * 256 + tid;
            valid[j] = t < n;
            if (valid[j]) {
                idx[j] = refine[t];
                q[j] = refine_q[t] & 127u;
                off[j] = aggregated_increment(start, q[j]);
            }
        }
        __syncthreads();
        if (tid < 32) {  // exclusive scan of the 128 counts, four a lane
            const uint32_t c0 = start[4 * tid], c1 = start[4 * tid + 1], c2 = start[4 * tid + 2],
                           c3 = start[4 * tid + 3];
            const uint32_t sum = c0 + c1 + c2 + c3;
            uint32_t incl = sum;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t v = __shfl_up_sync(0xffffffffu, incl, d);
                if ((int)tid >= d)
                    incl += v;
            }
            const uint32_t base = incl - sum;
            start[4 * tid] = base;
            start[4 * tid + 1] = base + c0;
            start[4 * tid + 2] = base + c0 + c1;
            start[4 * tid + 3] = base + c0 + c1 + c2;
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < REFINE_PER_THREAD; ++j)
            if (valid[j]) {
                const uint32_t at = start[q[j]] + off[j];
                sorted_i[at] = idx[j];
                sorted_q[at] = (uint8_t)q[j];
            }
        __syncthreads();
        const uint32_t count = n - t0 < TILE ? (uint32_t)(n - t0) : TILE;
#pragma unroll
        for (int j = 0; j < REFINE_PER_THREAD; ++j) {
            const uint32_t at = (uint32_t)j * 256 + tid;
            if (at < count) {
                const uint32_t i = sorted_i[at];
                const uint64_t p = primes[i];
                const uint32_t code = refined_code<FAM, MT>(job, p, codes[i], sorted_q[at]);
                codes[i] = code;
                if (wants_nine(job, p, code))
                    nine[aggregated_increment(&cc->nnine, 0)] = i;
                else if (code)
                    aggregated_increment(cc->count, class_bucket(code >> 16));
            }
        }
        __syncthreads();  // the next tile reuses the shared arrays
    }
}

// The rare-prime refinement over the primes classify listed (compacted, so
// every lane of a warp does the same two powers)
template <uint32_t FAM>
__global__ void __launch_bounds__(256) refine_kernel(JobView job, const uint64_t *__restrict__ primes,
                                                     uint32_t *__restrict__ codes, ClassCounters *__restrict__ cc,
                                                     const uint32_t *__restrict__ refine,
                                                     const uint8_t *__restrict__ refine_q, uint32_t *__restrict__ nine)
{
    if (cc->wide)
        refine_range<FAM, Mont>(job, primes, codes, cc, refine, refine_q, nine, cc->nrefine);
    else
        refine_range<FAM, MontN>(job, primes, codes, cc, refine, refine_q, nine, cc->nrefine);
}

template <uint32_t FAM, class MT>
__device__ __forceinline__ void nine_range(const JobView &job, const uint64_t *__restrict__ primes,
                                           uint32_t *__restrict__ codes, ClassCounters *__restrict__ cc,
                                           const uint32_t *__restrict__ nine, uint32_t n)
{
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += stride) {
        const uint32_t i = nine[t];
        const uint32_t code = nine_code<FAM, MT>(job, primes[i], codes[i]);
        codes[i] = code;
        if (code)
            aggregated_increment(cc->count, class_bucket(code >> 16));
    }
}

// The 9th-power character over the primes with 9 | p - 1 that classify or
// the refinement listed (after the refinement, whose codes it narrows)
template <uint32_t FAM>
__global__ void __launch_bounds__(256) nine_kernel(JobView job, const uint64_t *__restrict__ primes,
                                                   uint32_t *__restrict__ codes, ClassCounters *__restrict__ cc,
                                                   const uint32_t *__restrict__ nine)
{
    if (cc->wide)
        nine_range<FAM, Mont>(job, primes, codes, cc, nine, cc->nnine);
    else
        nine_range<FAM, MontN>(job, primes, codes, cc, nine, cc->nnine);
}

// Each CTA regroups tiles of 256 x REGROUP_PER_THREAD primes: a histogram of
// the tile's classes in shared memory, one global atomic per class and tile
// to reserve the tile's places in the class, then the scatter.  (One global
// atomic per class and warp, as first written, left the kernel waiting on
// atomics: long-scoreboard stalls of ~140 cycles per instruction.)  Eight
// primes a thread (16 took 103 registers and ran 0.14 ms on a 2^27 Proth
// segment against 0.09 ms).
constexpr int REGROUP_PER_THREAD = 8;
__global__ void __launch_bounds__(256) regroup_kernel(const uint64_t *__restrict__ primes, uint64_t nprimes,
                                                      const uint32_t *__restrict__ codes, ClassCounters *__restrict__ cc,
                                                      ClassItem *__restrict__ items)
{
    __shared__ uint32_t base[CLASS_BUCKETS];       // first place of each class
    __shared__ uint32_t hist[CLASS_BUCKETS];       // the tile's primes per class
    __shared__ uint32_t tile_base[CLASS_BUCKETS];  // the tile's first place per class
    const uint32_t tid = threadIdx.x;
    if (tid < CLASS_BUCKETS) {
        // a fixed trip count: the 48 loads go out together
        uint32_t run = 0;
#pragma unroll
        for (uint32_t b = 0; b < CLASS_BUCKETS; ++b)
            run += b < tid ? cc->count[b] : 0u;
        base[tid] = run;
    }
    const uint64_t tile = (uint64_t)blockDim.x * REGROUP_PER_THREAD;
    for (uint64_t t0 = (uint64_t)blockIdx.x * tile; t0 < nprimes; t0 += (uint64_t)gridDim.x * tile) {
        if (tid < CLASS_BUCKETS)
            hist[tid] = 0;
        __syncthreads();
        uint32_t code[REGROUP_PER_THREAD], off[REGROUP_PER_THREAD];
#pragma unroll
        for (int j = 0; j < REGROUP_PER_THREAD; ++j) {
            const uint64_t i = t0 + (uint64_t)j * blockDim.x + tid;
            code[j] = i < nprimes ? codes[i] : 0u;
            if (code[j])
                off[j] = aggregated_increment(hist, class_bucket(code[j] >> 16));
        }
        __syncthreads();
        if (tid < CLASS_BUCKETS)
            tile_base[tid] = hist[tid] ? base[tid] + atomicAdd(&cc->fill[tid], hist[tid]) : 0u;
        __syncthreads();
#pragma unroll
        for (int j = 0; j < REGROUP_PER_THREAD; ++j) {
            const uint64_t i = t0 + (uint64_t)j * blockDim.x + tid;
            if (code[j])
                items[tile_base[class_bucket(code[j] >> 16)] + off[j]] = ClassItem{primes[i], code[j], 0};
        }
        __syncthreads();
    }
}

template <uint32_t FAM>
__global__ void __launch_bounds__(256, min_ctas_per_sm(FAM))
class_walk_kernel(JobView job, const ClassItem *__restrict__ items, ClassCounters *__restrict__ cc)
{
    __shared__ unsigned long long total_s;
    if (threadIdx.x == 0) {
        unsigned long long t = 0;
#pragma unroll
        for (uint32_t b = 0; b < CLASS_BUCKETS; ++b)
            t += cc->count[b];
        total_s = t * job.tiles;
    }
    __syncthreads();
    const unsigned long long total = total_s;
    const uint32_t lane = threadIdx.x & 31u;
    for (;;) {
        unsigned long long base = 0;
        if (lane == 0)
            base = atomicAdd(&cc->next, 32ull);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= total)
            break;
        const uint64_t k = base + lane;
        if (k < total) {
            const uint64_t i = job.tiles == 1 ? k : k / job.tiles;
            const uint64_t t = k - i * job.tiles;
            const uint64_t s = job.n0 + t * job.tile_len;
            const uint64_t e = s + job.tile_len < job.n1 ? s + job.tile_len : job.n1;
            const ClassItem it = items[i];
            if (s < e) {
                if (it.p >= (1ull << 63))
                    run_doubling_wide(job, it.p, s, e);
                else
                    run_doubling_class(job, it.p, it.code >> 16, it.code & 0xffffu, s, e);
            }
        }
    }
}

// dynamic shared memory of a family's kernels at `block` threads
template <uint32_t FAM>
constexpr size_t smem_bytes(int block)
{
    return uses_filter<FAM>() ? (size_t)FILTER_WORDS * sizeof(uint32_t) * (size_t)block : 0;
}

// lets a kernel take more than the default 48 KiB of dynamic shared memory
template <class K>
static cudaError_t allow_smem(K kernel, size_t bytes)
{
    if (bytes <= 48 * 1024)
        return cudaSuccess;
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

// ------------------------------------------------------ batched launches
// Many jobs over one segment's prime list, any mix of families, in one
// persistent walk launch.  Per segment (all on the stream, nothing waits on
// the host, so a whole schedule is captured in one CUDA graph):
//   batch_bounds_kernel   each active job's sub-range of the sorted primes,
//                         and for the classified (doubling) jobs their
//                         offsets in the class buffers;
//   batch_screen_kernel, batch_classify_kernel, batch_refine_kernel
//                         power-residue class of every (classified job,
//                         prime) pair, as in the plain launch (screen,
//                         classes, rare-prime refinement), counted per job
//                         and class;
//   batch_plan_kernel     per job: class bases, its (prime, tile) units and
//                         the exclusive prefix of warp items over the jobs;
//   batch_regroup_kernel  the classified pairs written class by class;
//   batch_walk_kernel     a persistent grid taking one warp item (32 units
//                         of one job: same family, same class) at a time
//                         from a counter -- every family in one kernel.
// Work items are (job, 32 primes, index tile): long index ranges are cut
// into tiles that start with the families' O(log n) jumps, so a long job is
// spread over many warps instead of serialising on its primes.

__device__ __forceinline__ uint64_t lower_bound_u64(const uint64_t *a, uint64_t n, uint64_t x)
{
    uint64_t lo = 0, hi = n;
    while (lo < hi) {
        uint64_t mid = (lo + hi) >> 1;
        if (a[mid] < x)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

// the last active job i with key(i) <= x (keys nondecreasing, key(0) <= x)
template <class Key>
__device__ __forceinline__ uint32_t last_le(uint32_t n, uint64_t x, Key key)
{
    uint32_t lo = 0, hi = n;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (key(mid) <= x)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

__global__ void __launch_bounds__(1024) batch_bounds_kernel(BatchJob *__restrict__ jobs,
                                                            const uint32_t *__restrict__ active, uint32_t nactive,
                                                            const uint64_t *__restrict__ primes,
                                                            const uint64_t *__restrict__ d_count, uint64_t lo,
                                                            uint64_t hi, BatchSpan *__restrict__ spans,
                                                            BatchControl *__restrict__ ctl)
{
    const uint64_t n = *d_count;
    for (uint32_t i = threadIdx.x; i < nactive; i += blockDim.x) {
        BatchJob &j = jobs[active[i]];
        // the job's primes of this segment: [max(f0, lo), min(f1, hi))
        const uint64_t a = j.f0 > lo ? j.f0 : lo;
        const uint64_t b = j.f1 < hi ? j.f1 : hi;
        uint64_t pb = 0, pe = 0;
        if (a < b) {
            pb = lower_bound_u64(primes, n, a);
            pe = lower_bound_u64(primes, n, b);
            j.cursor = b;  // progress: the end of the segment the walk completes
        }
        spans[i].pbeg = pb;
        spans[i].pend = pe;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint64_t run = 0;
        for (uint32_t i = 0; i < nactive; ++i) {
            spans[i].coff = run;
            if (jobs[active[i]].classified)
                run += spans[i].pend - spans[i].pbeg;
        }
        spans[nactive].coff = run;
        ctl->nclass = run;
        ctl->nlisted = 0;
        ctl->nrefine = 0;
    }
}

// the classified job holding class pair t
__device__ __forceinline__ uint32_t class_job(const BatchSpan *spans, uint32_t nactive, uint64_t t)
{
    return last_le(nactive, t, [&](uint32_t i) { return spans[i].coff; });
}

// warp-aggregated atomicAdd of 1 per active lane on a 64-bit counter;
// returns this lane's old value
__device__ __forceinline__ unsigned long long aggregated_append(unsigned long long *counter)
{
    const uint32_t act = __activemask();
    const int leader = __ffs(act) - 1;
    const uint32_t lane = threadIdx.x & 31u;
    unsigned long long base = 0;
    if ((int)lane == leader)
        base = atomicAdd(counter, (unsigned long long)__popc(act));
    base = __shfl_sync(act, base, leader);
    return base + (unsigned long long)__popc(act & ((1u << lane) - 1u));
}

// the class code of a prime for a job of any doubling family (the family
// read at run time: one copy of the classification per product)
template <class MT>
__device__ __forceinline__ uint32_t class_code_rt(const JobView &v, uint64_t p)
{
    if (p >= (1ull << 63))
        return 1u << 16;
    const uint64_t k = v.family == MERSENNE ? 1 : (v.param < p ? v.param : v.param % p);
    if (!k)
        return 0;
    MT m;
    m.init_lite(p);  // the power pairs need no R^2
    const PowerClass c = doubling_class(m, k, v.family == PROTH);
    return c.M ? (c.M << 16) | c.r : 0u;
}
template <class MT>
__device__ __forceinline__ uint32_t refined_code_rt(const JobView &v, uint64_t p, uint32_t code)
{
    const uint64_t k = v.family == MERSENNE ? 1 : (v.param < p ? v.param : v.param % p);
    MT m;
    m.init_lite(p);  // the power pairs need no R^2
    const PowerClass c = refine_class(m, k, v.family == PROTH, PowerClass{code >> 16, code & 0xffffu},
                                      rare_q_of(p, refine_qmax(v)));
    return c.M ? (c.M << 16) | c.r : 0u;
}

// The batched forms of screen_kernel, classify_kernel and refine_kernel
// over the segment's (classified job, prime) pairs t: the screen lists the
// pairs it does not exclude, classification lists the pairs with a rare q,
// the refinement narrows them; the pairs with a class are counted per job
// and class.  Lists of pair numbers in the items buffer (free until the
// regroup).  Primes below 2^40 multiply with the narrow product.
__global__ void __launch_bounds__(256) batch_screen_kernel(const BatchJob *__restrict__ jobs,
                                                           const uint32_t *__restrict__ active, uint32_t nactive,
                                                           const uint64_t *__restrict__ primes,
                                                           const BatchSpan *__restrict__ spans,
                                                           BatchControl *__restrict__ ctl,
                                                           uint32_t *__restrict__ codes, uint64_t *__restrict__ listed)
{
    const uint64_t total = ctl->nclass;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += stride) {
        const uint32_t i = class_job(spans, nactive, t);
        const JobView &v = jobs[active[i]].view;
        const uint64_t p = primes[spans[i].pbeg + (t - spans[i].coff)];
        if (v.family != MERSENNE && quadratic_excluded(p, v.param, v.family == PROTH))
            codes[t] = 0;
        else
            listed[aggregated_append(&ctl->nlisted)] = t;
    }
}

__global__ void __launch_bounds__(256, 4) batch_classify_kernel(const BatchJob *__restrict__ jobs,
                                                                const uint32_t *__restrict__ active, uint32_t nactive,
                                                                const uint64_t *__restrict__ primes,
                                                                const BatchSpan *__restrict__ spans,
                                                                BatchControl *__restrict__ ctl,
                                                                uint32_t *__restrict__ codes,
                                                                uint32_t *__restrict__ bucket_count,
                                                                const uint64_t *__restrict__ listed,
                                                                uint64_t *__restrict__ refine)
{
    const uint64_t total = ctl->nlisted;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t x = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; x < total; x += stride) {
        const uint64_t t = listed[x];
        const uint32_t i = class_job(spans, nactive, t);
        const JobView &v = jobs[active[i]].view;
        const uint64_t p = primes[spans[i].pbeg + (t - spans[i].coff)];
        const uint32_t code = p < MONT_NARROW_LIMIT ? class_code_rt<MontN>(v, p) : class_code_rt<Mont>(v, p);
        codes[t] = code;
        if (wants_refine(v, p, code))
            refine[aggregated_append(&ctl->nrefine)] = t;
        else if (code)
            aggregated_increment(bucket_count, i * CLASS_BUCKETS + class_bucket(code >> 16));
    }
}

__global__ void __launch_bounds__(256) batch_refine_kernel(const BatchJob *__restrict__ jobs,
                                                           const uint32_t *__restrict__ active, uint32_t nactive,
                                                           const uint64_t *__restrict__ primes,
                                                           const BatchSpan *__restrict__ spans,
                                                           const BatchControl *__restrict__ ctl,
                                                           uint32_t *__restrict__ codes,
                                                           uint32_t *__restrict__ bucket_count,
                                                           const uint64_t *__restrict__ refine)
{
    const uint64_t total = ctl->nrefine;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t x = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; x < total; x += stride) {
        const uint64_t t = refine[x];
        const uint32_t i = class_job(spans, nactive, t);
        const JobView &v = jobs[active[i]].view;
        const uint64_t p = primes[spans[i].pbeg + (t - spans[i].coff)];
        const uint32_t code = p < MONT_NARROW_LIMIT ? refined_code_rt<MontN>(v, p, codes[t])
                                                    : refined_code_rt<Mont>(v, p, codes[t]);
        codes[t] = code;
        if (code)
            aggregated_increment(bucket_count, i * CLASS_BUCKETS + class_bucket(code >> 16));
    }
}

// Per job: class bases (classified jobs), its (prime, tile) units and the
// exclusive prefix of warp items, restarted at each walk group's first job
// (the active list is group-major: g.n[0] jobs of group 0, then group 1 ...).
struct GroupCounts {
    uint32_t n[BATCH_GROUPS];
};
__global__ void __launch_bounds__(1024) batch_plan_kernel(const BatchJob *__restrict__ jobs,
                                                          const uint32_t *__restrict__ active, uint32_t nactive,
                                                          BatchSpan *__restrict__ spans, BatchControl *__restrict__ ctl,
                                                          const uint32_t *__restrict__ bucket_count,
                                                          uint32_t *__restrict__ bucket_base, GroupCounts gc)
{
    for (uint32_t i = threadIdx.x; i < nactive; i += blockDim.x) {
        const BatchJob &j = jobs[active[i]];
        uint64_t primes_i = spans[i].pend - spans[i].pbeg;
        if (j.classified) {
            uint64_t run = 0;
            for (uint32_t b = 0; b < CLASS_BUCKETS; ++b) {
                bucket_base[i * CLASS_BUCKETS + b] = (uint32_t)run;
                run += bucket_count[i * CLASS_BUCKETS + b];
            }
            primes_i = run;  // pairs with a class (the others divide no term)
        }
        spans[i].units = primes_i * j.view.tiles;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t start[BATCH_GROUPS + 1];
        start[0] = 0;
        for (int g = 0; g < BATCH_GROUPS; ++g)
            start[g + 1] = start[g] + gc.n[g];
        for (int g = 0; g < BATCH_GROUPS; ++g) {
            uint64_t run = 0;
            for (uint32_t i = start[g]; i < start[g + 1]; ++i) {
                spans[i].warp_prefix = run;
                run += (spans[i].units + 31) / 32;
            }
            ctl->total_warps[g] = run;
            ctl->next[g] = 0;
        }
    }
}

// Tiles of 256 x REGROUP_PER_THREAD pairs: a tile inside one job (the
// usual case: a job's pairs are consecutive) takes a shared-memory
// histogram and one global atomic per class, as regroup_kernel does; a tile
// across jobs takes one global atomic per (job, class) and warp.
__global__ void __launch_bounds__(256) batch_regroup_kernel(const uint32_t *__restrict__ active, uint32_t nactive,
                                                            const uint64_t *__restrict__ primes,
                                                            const BatchSpan *__restrict__ spans,
                                                            const BatchControl *__restrict__ ctl,
                                                            const uint32_t *__restrict__ codes,
                                                            const uint32_t *__restrict__ bucket_base,
                                                            uint32_t *__restrict__ bucket_fill,
                                                            ClassItem *__restrict__ items)
{
    __shared__ uint32_t hist[CLASS_BUCKETS];
    __shared__ uint32_t tile_base[CLASS_BUCKETS];
    const uint32_t tid = threadIdx.x;
    const uint64_t total = ctl->nclass;
    const uint64_t tile = (uint64_t)blockDim.x * REGROUP_PER_THREAD;
    for (uint64_t t0 = (uint64_t)blockIdx.x * tile; t0 < total; t0 += (uint64_t)gridDim.x * tile) {
        const uint64_t t1 = t0 + tile < total ? t0 + tile : total;
        const uint32_t i0 = class_job(spans, nactive, t0);
        if (class_job(spans, nactive, t1 - 1) != i0) {
            for (uint64_t t = t0 + tid; t < t1; t += blockDim.x) {
                const uint32_t code = codes[t];
                if (!code)
                    continue;
                const uint32_t i = class_job(spans, nactive, t);
                const uint32_t key = i * CLASS_BUCKETS + class_bucket(code >> 16);
                const uint64_t pos = spans[i].coff + bucket_base[key] + aggregated_increment(bucket_fill, key);
                items[pos] = ClassItem{primes[spans[i].pbeg + (t - spans[i].coff)], code, 0};
            }
            continue;  // uniform over the CTA: no barrier skipped unevenly
        }
        if (tid < CLASS_BUCKETS)
            hist[tid] = 0;
        __syncthreads();
        uint32_t code[REGROUP_PER_THREAD], off[REGROUP_PER_THREAD];
#pragma unroll
        for (int j = 0; j < REGROUP_PER_THREAD; ++j) {
            const uint64_t t = t0 + (uint64_t)j * blockDim.x + tid;
            code[j] = t < t1 ? codes[t] : 0u;
            if (code[j])
                off[j] = aggregated_increment(hist, class_bucket(code[j] >> 16));
        }
        __syncthreads();
        if (tid < CLASS_BUCKETS)
            tile_base[tid] = hist[tid] ? bucket_base[i0 * CLASS_BUCKETS + tid] +
                                             atomicAdd(&bucket_fill[i0 * CLASS_BUCKETS + tid], hist[tid])
                                       : 0u;
        __syncthreads();
        const BatchSpan sp = spans[i0];
#pragma unroll
        for (int j = 0; j < REGROUP_PER_THREAD; ++j) {
            const uint64_t t = t0 + (uint64_t)j * blockDim.x + tid;
            if (code[j])
                items[sp.coff + tile_base[class_bucket(code[j] >> 16)] + off[j]] =
                    ClassItem{primes[sp.pbeg + (t - sp.coff)], code[j], 0};
        }
        __syncthreads();
    }
}

// one (prime, tile) unit of a job of walk group G
template <int G>
__device__ __forceinline__ void batch_unit(const BatchJob &j, uint64_t p, uint32_t code, uint64_t s, uint64_t e)
{
    const JobView &v = j.view;
    if (G == BATCH_CLASSES) {
        if (p < (1ull << 63))
            run_doubling_class(v, p, code >> 16, code & 0xffffu, s, e);
        else
            run_doubling_wide(v, p, s, e);
    } else if (G == BATCH_DOUBLING) {
        switch (v.family) {
        case PROTH: run_item<PROTH>(v, p, s, e); return;
        case RIESEL: run_item<RIESEL>(v, p, s, e); return;
        default: run_item<MERSENNE>(v, p, s, e); return;
        }
    } else if (G == BATCH_MULTIPLY) {
        run_item<SMARANDACHE>(v, p, s, e);
    } else {
        switch (v.family) {
        case FIBONACCI: run_item<FIBONACCI>(v, p, s, e); break;
        case LUCAS: run_item<LUCAS>(v, p, s, e); break;
        case PROTH_FIXED_N: run_item<PROTH_FIXED_N>(v, p, s, e); break;
        case RIESEL_FIXED_N: run_item<RIESEL_FIXED_N>(v, p, s, e); break;
        case TRIBONACCI: run_item<TRIBONACCI>(v, p, s, e); break;
        default: run_item<PEANO>(v, p, s, e); break;
        }
    }
}

// resident CTAs of a group's walk: the doubling walks keep the target
// filter's 64 KiB per CTA and 80 registers a thread; the others fit four
constexpr bool batch_filter(int g) { return g == BATCH_CLASSES || g == BATCH_DOUBLING; }
constexpr int batch_ctas_per_sm(int g) { return batch_filter(g) ? 3 : 4; }

// The walk of one group: a persistent grid taking one warp item (32 units
// of one job: same family, same class) at a time from the group's counter.
template <int G>
__global__ void __launch_bounds__(256, batch_ctas_per_sm(G))
batch_walk_kernel(const BatchJob *__restrict__ jobs, const uint32_t *__restrict__ active, uint32_t nactive,
                  const uint64_t *__restrict__ primes, const BatchSpan *__restrict__ spans,
                  BatchControl *__restrict__ ctl, const ClassItem *__restrict__ items)
{
    const uint64_t total = ctl->total_warps[G];
    const uint32_t lane = threadIdx.x & 31u;
    for (;;) {
        unsigned long long w = 0;
        if (lane == 0)
            w = atomicAdd(&ctl->next[G], 1ull);
        w = __shfl_sync(0xffffffffu, w, 0);
        if (w >= total)
            break;
        const uint32_t i = last_le(nactive, w, [&](uint32_t k) { return spans[k].warp_prefix; });
        const uint64_t u = (w - spans[i].warp_prefix) * 32 + lane;
        if (u < spans[i].units) {
            const BatchJob &j = jobs[active[i]];
            const uint32_t tiles = j.view.tiles;
            const uint64_t idx = tiles == 1 ? u : u / tiles;
            const uint64_t t = u - idx * tiles;
            const uint64_t s = j.view.n0 + t * j.view.tile_len;
            const uint64_t e = s + j.view.tile_len < j.view.n1 ? s + j.view.tile_len : j.view.n1;
            uint64_t p;
            uint32_t code = 0;
            if (G == BATCH_CLASSES) {
                const ClassItem it = items[spans[i].coff + idx];
                p = it.p;
                code = it.code;
            } else {
                p = primes[spans[i].pbeg + idx];
            }
            if (s < e)
                batch_unit<G>(j, p, code, s, e);
        }
    }
}

template <int G>
static cudaError_t launch_walk(const BatchJob *jobs, const uint32_t *active, uint32_t n, const uint64_t *primes,
                               const BatchSpan *spans, BatchControl *ctl, const ClassItem *items, int sm_count,
                               cudaStream_t st)
{
    const size_t sm = batch_filter(G) ? (size_t)FILTER_WORDS * sizeof(uint32_t) * 256 : 0;
    cudaError_t rc = allow_smem(batch_walk_kernel<G>, sm);
    int occ = 0;
    if (rc == cudaSuccess)
        rc = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, batch_walk_kernel<G>, 256, sm);
    if (rc == cudaSuccess) {
        batch_walk_kernel<G><<<sm_count * (occ > 0 ? occ : 1), 256, sm, st>>>(jobs, active, n, primes, spans, ctl,
                                                                              items);
        rc = cudaGetLastError();
        note_kernel_launch();
    }
    return rc;
}

int launch_batch(BatchJob *d_jobs, const uint32_t *d_active, const uint32_t gcount[BATCH_GROUPS], bool any_classified,
                 const uint64_t *d_primes, const uint64_t *d_count, uint64_t lo, uint64_t hi,
                 const BatchScratch &bs, int sm_count, cudaStream_t st, std::string &err)
{
    GroupCounts gc;
    uint32_t nactive = 0, first[BATCH_GROUPS];
    for (int g = 0; g < BATCH_GROUPS; ++g) {
        gc.n[g] = gcount[g];
        first[g] = nactive;
        nactive += gcount[g];
    }
    if (!nactive)
        return CTD_OK;
    cudaError_t rc = cudaSuccess;
    const int cgrid = sm_count * 8;
    if (any_classified)
        rc = cudaMemsetAsync(bs.bucket_count, 0, 2ull * nactive * CLASS_BUCKETS * sizeof(uint32_t), st);
    if (rc == cudaSuccess) {
        batch_bounds_kernel<<<1, 1024, 0, st>>>(d_jobs, d_active, nactive, d_primes, d_count, lo, hi, bs.spans,
                                                bs.ctl);
        rc = cudaGetLastError();
        note_kernel_launch();
    }
    if (rc == cudaSuccess && any_classified) {
        // the pair lists in the items buffer: [0, class_cap) and [class_cap, 2 class_cap) words
        uint64_t *listed = reinterpret_cast<uint64_t *>(bs.items);
        uint64_t *refine = listed + bs.class_cap;
        batch_screen_kernel<<<cgrid, 256, 0, st>>>(d_jobs, d_active, nactive, d_primes, bs.spans, bs.ctl, bs.codes,
                                                   listed);
        rc = cudaGetLastError();
        note_kernel_launch();
        if (rc == cudaSuccess) {
            batch_classify_kernel<<<cgrid, 256, 0, st>>>(d_jobs, d_active, nactive, d_primes, bs.spans, bs.ctl,
                                                         bs.codes, bs.bucket_count, listed, refine);
            rc = cudaGetLastError();
            note_kernel_launch();
        }
        if (rc == cudaSuccess) {
            batch_refine_kernel<<<cgrid, 256, 0, st>>>(d_jobs, d_active, nactive, d_primes, bs.spans, bs.ctl,
                                                       bs.codes, bs.bucket_count, refine);
            rc = cudaGetLastError();
            note_kernel_launch();
        }
    }
    if (rc == cudaSuccess) {
        batch_plan_kernel<<<1, 1024, 0, st>>>(d_jobs, d_active, nactive, bs.spans, bs.ctl, bs.bucket_count,
                                              bs.bucket_base, gc);
        rc = cudaGetLastError();
        note_kernel_launch();
    }
    if (rc == cudaSuccess && any_classified) {
        // bucket_fill follows bucket_count (cleared together above)
        batch_regroup_kernel<<<cgrid, 256, 0, st>>>(d_active, nactive, d_primes, bs.spans, bs.ctl, bs.codes,
                                                    bs.bucket_base, bs.bucket_count + nactive * CLASS_BUCKETS,
                                                    bs.items);
        rc = cudaGetLastError();
        note_kernel_launch();
    }
    // the walks, one launch per group present (heaviest work per term first)
#define CTD_WALK(G)                                                                                              \
    if (rc == cudaSuccess && gcount[G])                                                                          \
        rc = launch_walk<G>(d_jobs, d_active + first[G], gcount[G], d_primes, bs.spans + first[G], bs.ctl, bs.items, \
                            sm_count, st);
    CTD_WALK(BATCH_MULTIPLY)
    CTD_WALK(BATCH_OTHER)
    CTD_WALK(BATCH_CLASSES)
    CTD_WALK(BATCH_DOUBLING)
#undef CTD_WALK
    if (rc != cudaSuccess) {
        err = std::string("batched residue launch: ") + cudaGetErrorString(rc);
        return CTD_ERR_CUDA;
    }
    return CTD_OK;
}

// --------------------------------------------------------- the prime 2
// value_mod_2 / next_value_mod_2 of each family (number_sequence_helpers.hpp:14-37
// and the per-family closed forms cited in the oracle).
__device__ __forceinline__ uint64_t value_mod_2(uint32_t fam, uint64_t param, uint64_t n)
{
    switch (fam) {
    case MERSENNE: return n > 0;
    case PROTH:
    case RIESEL: return n > 0 ? 1 : ((param & 1) ^ 1);
    case SMARANDACHE: return (param & 1) ? (uint64_t)((n & 3) && ((n & 3) != 3)) : (n & 1);
    case FIBONACCI:
    case LUCAS: return n % 3 == 0 ? 0 : 1;
    case PROTH_FIXED_N:
    case RIESEL_FIXED_N: return 1;
    case TRIBONACCI: return (n & 3) >> 1;
    default: return n & 1;
    }
}

__device__ __forceinline__ uint64_t next_value_mod_2(uint32_t fam, uint64_t param, uint64_t r, uint64_t n)
{
    switch (fam) {
    case SMARANDACHE: return (param & 1) ? (r ^ (n & 1) ^ 1) : ((n & 1) ^ 1);
    case FIBONACCI:
    case LUCAS: return (n + 1) % 3 == 0 ? 0 : 1;
    case TRIBONACCI: return ((n + 1) & 3) >> 1;
    case CTD_PEANO: return r ^ 1;
    default: return 1;
    }
}

__global__ void mod2_kernel(JobView job)
{
    uint64_t r = value_mod_2(job.family, job.param, job.n0);
    if (!r)
        push(job.fb, 0, 2);
    for (uint64_t n = job.n0; n + 1 < job.n1; ++n) {
        r = next_value_mod_2(job.family, job.param, r, n);
        if (!r)
            push(job.fb, n + 1 - job.n0, 2);
    }
}

// ----------------------------------------------------- per-device tables
int prepare_residue_tables(int device, std::string &err)
{
    static std::mutex mu;
    static std::vector<int> done;
    static std::vector<uint4> div;
    std::lock_guard<std::mutex> lock(mu);
    for (int d : done)
        if (d == device)
            return CTD_OK;
    if (div.empty()) {
        std::vector<uint8_t> composite(TRIAL_LIMIT, 0);
        for (uint32_t q = 3; q < TRIAL_LIMIT; q += 2) {
            if (composite[q])
                continue;
            for (uint64_t k = (uint64_t)q * q; k < TRIAL_LIMIT; k += 2ull * q)
                composite[k] = 1;
            uint64_t inv = q;  // q^-1 mod 2^64 by Newton steps (3, 6, ..., 96 bits)
            for (int it = 0; it < 5; ++it)
                inv *= 2 - (uint64_t)q * inv;
            const uint64_t lim = ~0ull / q;
            div.push_back(uint4{(uint32_t)inv, (uint32_t)(inv >> 32), (uint32_t)(lim >> 32), q});
        }
        if (div.size() != TRIAL_PRIMES) {
            err = "trial-division table: unexpected prime count";
            div.clear();
            return CTD_ERR_CUDA;
        }
    }
    cudaError_t rc = cudaMemcpyToSymbol(g_trial_div, div.data(), div.size() * sizeof(uint4));
    if (rc != cudaSuccess) {
        err = std::string("trial-division table upload: ") + cudaGetErrorString(rc);
        return CTD_ERR_CUDA;
    }
    done.push_back(device);
    return CTD_OK;
}

// ----------------------------------------------------------- launchers
template <uint32_t FAM>
static cudaError_t launch_fam(const JobView &v, const uint64_t *d_primes, uint64_t n, int grid, int block,
                              cudaStream_t st, unsigned long long *next)
{
    const size_t sm = smem_bytes<FAM>(block);
    cudaError_t e = allow_smem(residue_kernel<FAM>, sm);
    if (e == cudaSuccess && next)
        e = cudaMemsetAsync(next, 0, sizeof(*next), st);
    if (e != cudaSuccess)
        return e;
    residue_kernel<FAM><<<grid, block, sm, st>>>(v, d_primes, n, next);
    return cudaGetLastError();
}

ResidueScratch *residue_scratch_create(int device, int sm_count)
{
    auto *rs = new (std::nothrow) ResidueScratch();
    if (rs) {
        rs->device = device;
        rs->sm_count = sm_count > 0 ? sm_count : 1;
    }
    return rs;
}

void residue_scratch_destroy(ResidueScratch *rs)
{
    if (!rs)
        return;
    cudaFree(rs->codes);
    cudaFree(rs->items);
    cudaFree(rs->refine);
    cudaFree(rs->refine_q);
    cudaFree(rs->listed);
    cudaFree(rs->nine);
    cudaFree(rs->counters);
    delete rs;
}

static int ensure_class_scratch(ResidueScratch *rs, uint64_t nprimes, std::string &err)
{
    if (!rs->counters) {
        cudaError_t e = cudaMalloc(&rs->counters, sizeof(ClassCounters));
        if (e != cudaSuccess) {
            err = std::string("class counters: ") + cudaGetErrorString(e);
            return e == cudaErrorMemoryAllocation ? CTD_ERR_OUT_OF_MEMORY : CTD_ERR_CUDA;
        }
    }
    if (nprimes <= rs->cap)
        return CTD_OK;
    cudaFree(rs->codes);
    cudaFree(rs->items);
    cudaFree(rs->refine);
    cudaFree(rs->refine_q);
    cudaFree(rs->listed);
    cudaFree(rs->nine);
    rs->codes = nullptr;
    rs->items = nullptr;
    rs->refine = nullptr;
    rs->refine_q = nullptr;
    rs->listed = nullptr;
    rs->nine = nullptr;
    rs->cap = 0;
    cudaError_t e = cudaMalloc(&rs->codes, nprimes * sizeof(uint32_t));
    if (e == cudaSuccess)
        e = cudaMalloc(&rs->items, nprimes * sizeof(ClassItem));
    if (e == cudaSuccess)
        e = cudaMalloc(&rs->refine, nprimes * sizeof(uint32_t));
    if (e == cudaSuccess)
        e = cudaMalloc(&rs->refine_q, nprimes);
    if (e == cudaSuccess)
        e = cudaMalloc(&rs->listed, 8 * nprimes * sizeof(uint32_t));
    if (e == cudaSuccess)
        e = cudaMalloc(&rs->nine, nprimes * sizeof(uint32_t));
    if (e != cudaSuccess) {
        err = std::string("class scratch: ") + cudaGetErrorString(e);
        // give back what was allocated, so that the caller's other path has
        // the room, and clear the (non-sticky) allocation error
        cudaFree(rs->codes);
        cudaFree(rs->items);
        cudaFree(rs->refine);
        cudaFree(rs->refine_q);
        cudaFree(rs->listed);
        cudaFree(rs->nine);
        rs->codes = nullptr;
        rs->items = nullptr;
        rs->refine = nullptr;
        rs->refine_q = nullptr;
        rs->listed = nullptr;
        rs->nine = nullptr;
        if (e == cudaErrorMemoryAllocation) {
            (void)cudaGetLastError();
            return CTD_ERR_OUT_OF_MEMORY;
        }
        return CTD_ERR_CUDA;
    }
    rs->cap = nprimes;
    return CTD_OK;
}

template <uint32_t FAM>
static int class_walk_occupancy(int block)
{
    int n = 0;
    const size_t sm = smem_bytes<FAM>(block);
    if (allow_smem(class_walk_kernel<FAM>, sm) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, class_walk_kernel<FAM>, block, sm) != cudaSuccess)
        return 0;
    return n;
}

template <uint32_t FAM>
static int launch_classified(const JobView &v, const uint64_t *d_primes, uint64_t n, cudaStream_t st,
                             ResidueScratch *rs, std::string &err)
{
    int rc = ensure_class_scratch(rs, n, err);
    if (rc)
        return rc;
    cudaError_t e = cudaMemsetAsync(rs->counters, 0, sizeof(ClassCounters), st);
    const uint64_t want = (n + 255) / 256;
    const int cgrid = (int)(want < (uint64_t)rs->sm_count * 8 ? want : (uint64_t)rs->sm_count * 8);
    // the quadratic screen (Mersenne's target 1 is always a residue) and the
    // primes' buckets by divisibility pattern, then one classification
    // launch per pattern
    if (e == cudaSuccess) {
        screen_kernel<FAM><<<cgrid, 256, 0, st>>>(v, d_primes, n, rs->codes, rs->counters, rs->listed, rs->cap);
        e = cudaGetLastError();
        if (e == cudaSuccess)
            note_kernel_launch();
    }
#define CTD_CLASSIFY(PAT)                                                                                         \
    if (e == cudaSuccess) {                                                                                       \
        classify_kernel<FAM, PAT><<<cgrid, 256, 0, st>>>(v, d_primes, rs->codes, rs->counters, rs->refine,       \
                                                         rs->refine_q, rs->nine, rs->listed, rs->cap);            \
        e = cudaGetLastError();                                                                                   \
        if (e == cudaSuccess && PAT < 7)                                                                          \
            note_kernel_launch();                                                                                 \
    }
    CTD_CLASSIFY(0) CTD_CLASSIFY(1) CTD_CLASSIFY(2) CTD_CLASSIFY(3)
    CTD_CLASSIFY(4) CTD_CLASSIFY(5) CTD_CLASSIFY(6) CTD_CLASSIFY(7)
#undef CTD_CLASSIFY
    if (e == cudaSuccess) {
        note_kernel_launch();
        // the listed primes are about a quarter of n: a grid for that many
        // (refine_kernel's tiles are 256 x REFINE_PER_THREAD of them)
        const uint64_t rwant = (n / 4 + 256 * REFINE_PER_THREAD - 1) / (256 * REFINE_PER_THREAD);
        const int rgrid = (int)(rwant < (uint64_t)rs->sm_count * 8 ? (rwant ? rwant : 1) : (uint64_t)rs->sm_count * 8);
        refine_kernel<FAM><<<rgrid, 256, 0, st>>>(v, d_primes, rs->codes, rs->counters, rs->refine, rs->refine_q,
                                                  rs->nine);
        e = cudaGetLastError();
        if (e == cudaSuccess) {
            note_kernel_launch();
            nine_kernel<FAM><<<rgrid, 256, 0, st>>>(v, d_primes, rs->codes, rs->counters, rs->nine);
            e = cudaGetLastError();
        }
    }
    if (e == cudaSuccess) {
        note_kernel_launch();
        regroup_kernel<<<cgrid, 256, 0, st>>>(d_primes, n, rs->codes, rs->counters, rs->items);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        note_kernel_launch();
        const size_t sm = smem_bytes<FAM>(256);
        e = allow_smem(class_walk_kernel<FAM>, sm);
        const int occ = class_walk_occupancy<FAM>(256);
        if (e == cudaSuccess) {
            class_walk_kernel<FAM><<<rs->sm_count * (occ > 0 ? occ : 1), 256, sm, st>>>(v, rs->items, rs->counters);
            e = cudaGetLastError();
        }
    }
    if (e != cudaSuccess) {
        err = std::string("classified doubling launch: ") + cudaGetErrorString(e);
        return CTD_ERR_CUDA;
    }
    note_kernel_launch();
    return CTD_OK;
}

int launch_residues(const JobView &view, const uint64_t *d_primes, uint64_t nprimes, int grid, int block,
                    cudaStream_t stream, std::string &err, ResidueScratch *scratch)
{
    if (!nprimes || view.n1 <= view.n0)
        return CTD_OK;
    const bool doubling = view.family == PROTH || view.family == RIESEL || view.family == MERSENNE;
    const uint32_t cmin = view.classify_min ? view.classify_min : DEFAULT_CLASSIFY_MIN;
    // (the class passes index the primes with 32 bits)
    if (scratch && doubling && view.variant == CTD_VARIANT_AUTO && view.n1 - view.n0 >= cmin &&
        nprimes <= 0xffffffffull) {
        // the class buffers (about 61 bytes a prime); without the device
        // memory for them the walk over every term below gives the same
        // factors
        std::string serr;
        const int src = ensure_class_scratch(scratch, nprimes, serr);
        if (src == CTD_OK) {
            switch (view.family) {
            case PROTH: return launch_classified<PROTH>(view, d_primes, nprimes, stream, scratch, err);
            case RIESEL: return launch_classified<RIESEL>(view, d_primes, nprimes, stream, scratch, err);
            default: return launch_classified<MERSENNE>(view, d_primes, nprimes, stream, scratch, err);
            }
        }
        if (src != CTD_ERR_OUT_OF_MEMORY) {
            err = serr;
            return src;
        }
    }
    // the work counter of the persistent grid (the context's scratch)
    unsigned long long *next = nullptr;
    if (scratch) {
        int rc0 = ensure_class_scratch(scratch, 0, err);
        if (rc0)
            return rc0;
        next = &scratch->counters->next;
    }
    cudaError_t rc;
    switch (view.family) {
    case MERSENNE: rc = launch_fam<MERSENNE>(view, d_primes, nprimes, grid, block, stream, next); break;
    case PROTH: rc = launch_fam<PROTH>(view, d_primes, nprimes, grid, block, stream, next); break;
    case RIESEL: rc = launch_fam<RIESEL>(view, d_primes, nprimes, grid, block, stream, next); break;
    case SMARANDACHE: rc = launch_fam<SMARANDACHE>(view, d_primes, nprimes, grid, block, stream, next); break;
    case FIBONACCI: rc = launch_fam<FIBONACCI>(view, d_primes, nprimes, grid, block, stream, next); break;
    case LUCAS: rc = launch_fam<LUCAS>(view, d_primes, nprimes, grid, block, stream, next); break;
    case PROTH_FIXED_N: rc = launch_fam<PROTH_FIXED_N>(view, d_primes, nprimes, grid, block, stream, next); break;
    case RIESEL_FIXED_N: rc = launch_fam<RIESEL_FIXED_N>(view, d_primes, nprimes, grid, block, stream, next); break;
    case TRIBONACCI: rc = launch_fam<TRIBONACCI>(view, d_primes, nprimes, grid, block, stream, next); break;
    case PEANO: rc = launch_fam<PEANO>(view, d_primes, nprimes, grid, block, stream, next); break;
    default: err = "unknown sequence family"; return CTD_ERR_INVALID_ARGUMENT;
    }
    if (rc != cudaSuccess) {
        err = std::string("residue kernel launch: ") + cudaGetErrorString(rc);
        return CTD_ERR_CUDA;
    }
    note_kernel_launch();
    return CTD_OK;
}

template <uint32_t FAM>
static int occupancy(int block)
{
    int n = 0;
    const size_t sm = smem_bytes<FAM>(block);
    if (allow_smem(residue_kernel<FAM>, sm) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, residue_kernel<FAM>, block, sm) != cudaSuccess)
        return 0;
    return n;
}

int residue_blocks_per_sm(uint32_t family, int block)
{
    switch (family) {
    case MERSENNE: return occupancy<MERSENNE>(block);
    case PROTH: return occupancy<PROTH>(block);
    case RIESEL: return occupancy<RIESEL>(block);
    case SMARANDACHE: return occupancy<SMARANDACHE>(block);
    case FIBONACCI: return occupancy<FIBONACCI>(block);
    case LUCAS: return occupancy<LUCAS>(block);
    case PROTH_FIXED_N: return occupancy<PROTH_FIXED_N>(block);
    case RIESEL_FIXED_N: return occupancy<RIESEL_FIXED_N>(block);
    case TRIBONACCI: return occupancy<TRIBONACCI>(block);
    case PEANO: return occupancy<PEANO>(block);
    default: return 0;
    }
}

int launch_mod2(const JobView &view, cudaStream_t stream, std::string &err)
{
    if (view.n1 <= view.n0)
        return CTD_OK;
    mod2_kernel<<<1, 1, 0, stream>>>(view);
    cudaError_t rc = cudaGetLastError();
    if (rc != cudaSuccess) {
        err = std::string("mod-2 kernel launch: ") + cudaGetErrorString(rc);
        return CTD_ERR_CUDA;
    }
    note_kernel_launch();
    return CTD_OK;
}

}  // namespace ctd
