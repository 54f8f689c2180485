// Host-side check of the doubling families' power-residue classes
// (ctd_powres.cuh is __host__ __device__).  Reads "p wt" lines on stdin
// (odd prime p, 0 < wt < p) and prints "M r M2 r2": every n with
// 2^-n = wt (mod p) satisfies n = r (mod M), and n = r2 (mod M2) after the
// refinement by the smallest rare prime q = 11 .. 127 dividing p - 1 and by
// the 9th-power character when 9 | p - 1; M = 0 (M2 = 0)
// when no n does; then "x" (1 when the quadratic screen excludes p) and the
// Jacobi symbol (wt/p); last 1 when the classes through the narrow
// Montgomery product (p < 2^40) and the class for p's divisibility pattern
// (doubling_class_pat) equal these.
#include <cinttypes>
#include <cstdio>

#include "../cutrialdive_gb300/csrc/ctd_powres.cuh"

// doubling_class_pat for p's own pattern
template <class MT>
ctd::PowerClass doubling_class_by_pattern(const MT &m, uint64_t k, bool negate)
{
    switch (ctd::powres_pattern(m.p)) {
    case 0: return ctd::doubling_class_pat<0>(m, k, negate);
    case 1: return ctd::doubling_class_pat<1>(m, k, negate);
    case 2: return ctd::doubling_class_pat<2>(m, k, negate);
    case 3: return ctd::doubling_class_pat<3>(m, k, negate);
    case 4: return ctd::doubling_class_pat<4>(m, k, negate);
    case 5: return ctd::doubling_class_pat<5>(m, k, negate);
    case 6: return ctd::doubling_class_pat<6>(m, k, negate);
    default: return ctd::doubling_class_pat<7>(m, k, negate);
    }
}

int main()
{
    unsigned long long p, wt;
    while (std::scanf("%llu %llu", &p, &wt) == 2) {
        ctd::Mont m;
        m.init(p);
        // wt as -k with k = p - wt (the Proth form); the test covers every wt
        const ctd::PowerClass c = ctd::doubling_class(m, p - wt, true);
        ctd::PowerClass f = ctd::refine_class(m, p - wt, true, c, ctd::rare_q_of(p, 127));
        if ((p - 1) % 9 == 0)
            f = ctd::nine_class(m, p - wt, true, f);
        const int x = ctd::quadratic_excluded(p, p - wt, true) ? 1 : 0;
        const ctd::PowerClass cp = doubling_class_by_pattern(m, p - wt, true);
        int same = cp.M == c.M && cp.r == c.r;
        if (p < ctd::MONT_NARROW_LIMIT) {
            ctd::MontN n;
            n.init(p);
            const ctd::PowerClass cn = ctd::doubling_class(n, p - wt, true);
            ctd::PowerClass fn = ctd::refine_class(n, p - wt, true, cn, ctd::rare_q_of(p, 127));
            if ((p - 1) % 9 == 0)
                fn = ctd::nine_class(n, p - wt, true, fn);
            const ctd::PowerClass cpn = doubling_class_by_pattern(n, p - wt, true);
            same = same && cn.M == c.M && cn.r == c.r && fn.M == f.M && fn.r == f.r && cpn.M == c.M && cpn.r == c.r;
        }
        std::printf("%u %u %u %u %d %d %d\n", c.M, c.r, f.M, f.r, x, ctd::jacobi(wt, p), same);
    }
    return 0;
}
