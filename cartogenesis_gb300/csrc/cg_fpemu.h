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
// The double m * 2^(e-52) for 2^52 <= m <= 2^53 (the top of the binade [2^e, 2^(e+1)) included).
__device__ __forceinline__ double from_binade(int64_t m, int e) {
    if (m == ((int64_t)1 << 53)) return __longlong_as_double((long long)(e + 1 + 1023) << 52);
    return __longlong_as_double(((long long)(e + 1023) << 52) | (long long)(m - ((int64_t)1 << 52)));
}

// One warp's share of a sequential double sum: lane j adds `count` copies of its term w > 0 (count
// may be 0), lanes in order, to a running sum s >= 0 that is the same in every lane. Returns the
// sum after the whole warp (the same in every lane) and sets *before, per lane, to the sum before
// the lane's first addition. Exact, and on the integer pipes: while the sum stays in one binade
// [2^e, 2^(e+1)) and no addition falls on a tie, every addition adds a whole number d of units
// U = 2^(e-52) (d = w / U rounded to nearest, read off the bits of w), so a run of lanes is an
// integer prefix sum of count * d. The first lane whose additions would leave the binade or meet a
// tie is taken alone by seq_repeat_add, and the scan resumes after it.
__device__ double warp_seq_sum(double s, double w, int64_t count, double* before) {
    const unsigned FULL = 0xFFFFFFFFu;
    const int64_t TOP = (int64_t)1 << 53;
    const int lane = threadIdx.x & 31;
    const long long wb = __double_as_longlong(w);
    const int ew = (int)((wb >> 52) & 0x7FF) - 1023;
    const int64_t mw = (int64_t)((wb & ((1LL << 52) - 1)) | (1LL << 52));
    const bool w_normal = ((wb >> 52) & 0x7FF) != 0 && wb > 0;
    int start = 0;
    while (start < 32) {
        const long long sb = __double_as_longlong(s);
        const int es = (int)((sb >> 52) & 0x7FF);
        int first_bad;
        int64_t m = 0, excl = 0, total = 0;
        int e = 0;
        if (sb > 0 && es != 0 && es != 0x7FF) {   // s positive and normal: it has a binade
            e = es - 1023;
            m = (int64_t)((sb & ((1LL << 52) - 1)) | (1LL << 52));
            int64_t q = 0, d = 0, inc = 0;
            bool ok = true;
            if (lane >= start && count > 0) {
                const int shift = e - ew;
                if (!w_normal || shift < 0) {
                    ok = false;   // the term alone reaches the next binade
                } else if (shift == 0) {
                    q = d = mw;
                } else if (shift < 63) {
                    q = mw >> shift;
                    const int64_t rem = mw & (((int64_t)1 << shift) - 1), half = (int64_t)1 << (shift - 1);
                    if (rem == half) ok = false;   // a tie: the parity of the sum decides
                    d = q + (rem > half ? 1 : 0);
                }   // shift >= 63: w is below half a unit, every addition rounds back (d = 0)
                if (ok && d > 0 && count > TOP / d) ok = false;
                if (ok) inc = count * d;
            }
            int64_t incl = inc;
            for (int o = 1; o < 32; o <<= 1) {
                const int64_t t = __shfl_up_sync(FULL, incl, o);
                if (lane >= o) incl += t;
            }
            excl = incl - inc;
            total = __shfl_sync(FULL, incl, 31);
            // Every addition of this lane stays in the binade: the last one starts at m + excl + (count-1) d.
            if (ok && lane >= start && count > 0 && m + excl + (count - 1) * d + q > TOP - 1) ok = false;
            const unsigned bad = __ballot_sync(FULL, !ok);
            first_bad = bad ? __ffs(bad) - 1 : 32;
            if (lane >= start && lane < first_bad) *before = from_binade(m + excl, e);
            if (first_bad == 32) return from_binade(m + total, e);
            s = from_binade(m + __shfl_sync(FULL, excl, first_bad), e);
        } else {
            first_bad = start;   // no binade (zero or subnormal sum): one lane at a time
        }
        // Lane first_bad alone, in closed form.
        const double wj = __shfl_sync(FULL, w, first_bad);
        const int64_t cj = __shfl_sync(FULL, count, first_bad);
        if (lane == first_bad) *before = s;
        if (cj > 0) s = seq_repeat_add(s, wj, cj);
        start = first_bad + 1;
    }
    return s;
}
#endif

}  // namespace cg
