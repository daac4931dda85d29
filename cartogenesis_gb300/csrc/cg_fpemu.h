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

#ifdef __CUDACC__
// One warp, 32 terms: each lane adds `count` copies of its term `w` (> 0) to a running sum `s` that
// is the same in every lane, lanes in order. When s > 0 and every addition of the chunk stays inside
// s's binade with no tie at half an ulp, every addition adds a fixed whole number of ulps d, so the
// chunk is an integer prefix sum. Then it returns true with, per lane, the sum before that lane's
// first addition (*before) and the sum after the whole chunk (*after, same in all lanes); otherwise
// it returns false and the caller replays the chunk one addition at a time.
__device__ __forceinline__ bool warp_chunk_sum(double s, double w, int64_t count, double* before, double* after) {
    const unsigned FULL = 0xFFFFFFFFu;
    const int64_t TOP = (int64_t)1 << 53;
    const int lane = threadIdx.x & 31;
    if (!(s > 0.0)) return false;
    int e = ilogb(s);
    double U = ldexp(1.0, e - 52);
    int64_t m = (int64_t)(s / U);
    bool ok = true;
    int64_t inc = 0, q = 0, d = 0;
    if (count > 0) {
        double x = ldexp(w, 52 - e);   // w / U, exact
        if (!(x < 9.0e15)) {
            ok = false;
        } else {
            q = (int64_t)x;
            double f = x - (double)q;
            if (f == 0.5) ok = false;
            d = q + (f > 0.5 ? 1 : 0);
            if (d > 0 && count > TOP / d) ok = false;
            else inc = count * d;
        }
    }
    // Exclusive prefix of the increments across the warp.
    int64_t incl = inc;
    for (int o = 1; o < 32; o <<= 1) {
        int64_t t = __shfl_up_sync(FULL, incl, o);
        if (lane >= o) incl += t;
    }
    int64_t excl = incl - inc;
    // Every step of this lane stays in the binade: the last one starts at m + excl + (count-1) d.
    if (ok && count > 0 && m + excl + (count - 1) * d + q > TOP - 1) ok = false;
    if (!__all_sync(FULL, ok)) return false;
    int64_t total = __shfl_sync(FULL, incl, 31);
    *before = (double)(m + excl) * U;
    *after = (double)(m + total) * U;
    return true;
}
#endif

}  // namespace cg
