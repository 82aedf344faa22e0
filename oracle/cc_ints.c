/* ORACLE (test infrastructure only) -- the synthetic antisymmetrised
 * two-electron integrals <pq||rs> of the coupled-cluster oracle, over the
 * outer product of four orbital index lists, in C with OpenMP.
 *
 * The same definition as oracle/cc.py System.integral_values (which is the
 * readable statement and the check: tests/test_cc_blocks.py compares the two
 * bit for bit):
 *   pair (p,q) -> (a,b) = sorted, sign -1 per swap; likewise (r,s) -> (c,d);
 *   P = a n + b, R = c n + d, key = seed ^ (min(P,R) * GOLD + max(P,R) * C2),
 *   z = splitmix64 finaliser of key, value = (z >> 63 ? -1 : 1) * mag[(b-a)+(d-c)]
 *   times the pair signs; zero when p == q, r == s or the irreps of p, q, r, s
 *   do not multiply (XOR) to the totally symmetric irrep.
 * The reference has no integrals of its own (its tensors are filled by
 * Tensor::initialize, tensor.cc:744-758, or by the drivers). */
#include <stdint.h>

static uint64_t orc_mix(uint64_t z) {
    z ^= z >> 30;
    z *= 0xBF58476D1CE4E5B9ull;
    z ^= z >> 27;
    z *= 0x94D049BB133111EBull;
    z ^= z >> 31;
    return z;
}

void orc_cc_integrals(uint64_t seed_int, int64_t n, const double* mag, const int64_t* irrep,
                      int64_t np_, const int64_t* P, int64_t nq, const int64_t* Q,
                      int64_t nr, const int64_t* R, int64_t ns, const int64_t* S, double* out) {
    const uint64_t GOLD = 0x9E3779B97F4A7C15ull, C2 = 0xC2B2AE3D27D4EB4Full;
    #pragma omp parallel for collapse(2) schedule(static)
    for (int64_t i = 0; i < np_; ++i)
        for (int64_t j = 0; j < nq; ++j) {
            double* o = out + (i * nq + j) * nr * ns;
            const uint64_t p = (uint64_t)P[i], q = (uint64_t)Q[j];
            const double s1 = p > q ? -1.0 : 1.0;
            const uint64_t a = p > q ? q : p, b = p > q ? p : q;
            for (int64_t k = 0; k < nr; ++k)
                for (int64_t l = 0; l < ns; ++l) {
                    const uint64_t r = (uint64_t)R[k], s = (uint64_t)S[l];
                    double v = 0.0;
                    const int zero = p == q || r == s ||
                                     (irrep[p] ^ irrep[q] ^ irrep[r] ^ irrep[s]) != 0;
                    if (!zero) {
                        const double s2 = r > s ? -1.0 : 1.0;
                        const uint64_t c = r > s ? s : r, d = r > s ? r : s;
                        const uint64_t PP = a * (uint64_t)n + b, RR = c * (uint64_t)n + d;
                        const uint64_t lo = PP < RR ? PP : RR, hi = PP < RR ? RR : PP;
                        const uint64_t z = orc_mix(seed_int ^ (lo * GOLD + hi * C2));
                        const double m = mag[(b - a) + (d - c)];
                        v = ((z >> 63) ? -m : m) * s1 * s2;
                    }
                    o[k * ns + l] = v;
                }
        }
}
