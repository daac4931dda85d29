// Exact emulation of sequential IEEE double summation, for sums the reference takes one term at a
// time in a fixed order.
//
// seq_repeat_add(s, w, c) returns what `repeat(c) { s += w }` leaves in s with round-to-nearest-
// even, for s >= 0 and w > 0, in O(binades crossed) steps instead of O(c). Within one binade
// [2^e, 2^(e+1)) every double is a multiple of U = 2^(e-52), so s = m*U and one addition gives
// m' = m + rne(q + f), where w/U = q + f (q integer, 0 <= f < 1): the increment is q or q+1 and
// depends on m only through a tie (f = 1/2), where it is q + ((m + q) & 1). After one tie step m is
// even, and from then on every step adds q + (q & 1). So, while the exact sum stays below
// 2^(e+1), a run of steps adds one fixed increment and can be taken at once; the step that leaves
// the binade is taken as a plain hardware addition. Nothing here is approximate.
#pragma once

#include <stdint.h>

#ifdef __CUDACC__
#define CG_HD __host__ __device__ __forceinline__
#else
#define CG_HD inline
#include <cmath>
#endif

namespace cg {

CG_HD double seq_repeat_add(double s, double w, int64_t c) {
    const int64_t TOP = (int64_t)1 << 53;   // m ranges over [2^52, 2^53) within a binade
    while (c > 0) {
        if (s == 0.0) {   // fl(0 + w) = w
            s = s + w;
            --c;
            continue;
        }
        int e;
#ifdef __CUDA_ARCH__
        e = ilogb(s);
        double U = ldexp(1.0, e - 52);
#else
        e = std::ilogb(s);
        double U = std::ldexp(1.0, e - 52);
#endif
        int64_t m = (int64_t)(s / U);   // exact: s is a multiple of U
        double x = w / U;               // exact: scaling by a power of two
        if (x >= 9.0e15) {              // the term alone reaches past the binade: one plain step
            s = s + w;
            --c;
            continue;
        }
        int64_t q = (int64_t)x;
        double f = x - (double)q;       // exact
        if (m + q > TOP - 1) {          // this step leaves the binade: take it in hardware
            s = s + w;
            --c;
            continue;
        }
        int64_t d;
        if (f == 0.5) {
            if ((m & 1) != 0) {         // one tie step from an odd m, which lands on an even m
                s = (double)(m + q + ((m + q) & 1)) * U;
                --c;
                continue;
            }
            d = q + (q & 1);            // from an even m every tie step adds this and keeps m even
        } else {
            d = q + (f > 0.5 ? 1 : 0);
        }
        if (d == 0) return s;           // every remaining step rounds back to s
        // Steps j = 0..t-1 stay inside the binade while m + j*d + q <= TOP - 1.
        int64_t tmax = (TOP - 1 - q - m) / d + 1;
        int64_t t = c < tmax ? c : tmax;
        m += t * d;
        c -= t;
        s = (double)m * U;               // exact (m <= 2^53)
    }
    return s;
}

}  // namespace cg
