// BeltErosion.replay (BeltErosion.kt:96-425) on the device, and GaussianBlur.apply
// (GaussianBlur.kt:44-111) beside it.
//
// Before the hydraulic rounds, each young belt is lowered to where its crust stood when the exposure
// window opened, raised again round by round at the rate its own thickening came at, and cut as it
// rises: about a hundred rounds over the belt cells alone. Every step keeps the reference's bits:
//  - a round's spill levels are FlowRouting.fillDepressions over the belt's inner land (belt cells
//    above the shoreline, off the polar rows, whose eight neighbours all lie in the belt): every other
//    belt cell seeds the belt's flood at its own height and never rises, and no cell off the belt
//    neighbours an inner one, so the fill pops the inner cells in the belt flood's order (its keys'
//    local indices run in cell order) and gives them the same levels;
//  - the facet rule (FlowRouting.facetReceiver) routes the belt's land over the caller-shaped surface;
//  - the run order is the Kahn FIFO of FlowRouting.drainageOrder over the belt, so the tree walk's
//    drainage keys (level, deepest source) order it; a cell's discharge and spoil flux add its donors
//    in key order, and one cooperative kernel runs the Kahn levels with a grid barrier between them,
//    upward for the sums and downward for the cut, which reads each receiver's final height;
//  - the books (uplift, cut, export to the sea and to the land, the slopes' shed) are the reference's
//    running double sums: each round lays its terms out in the reference's order, the running total
//    first, and sums them exactly in parallel (seq_sum_f64_dev); a term the reference skips is +0,
//    which leaves a sum that started at +0 unchanged;
//  - the sweeps give from belt cells only and visit neighbours rows first, then columns
//    (forEachNeighborWithLimit); every cell of a sweep reads the heights before it;
//  - the rebound's blur sums its taps in order in double; the taps are computed on the host with
//    std::exp, like a plan's twiddles.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cooperative_groups.h>
#include <vector>

#include "cg_common.cuh"
#include "cg_internal.h"
#include "cg_params.h"
#include "cg_util.h"

namespace cg {
namespace {

namespace cgr = cooperative_groups;

constexpr int kReboundRounds = 10;                   // BeltErosion.REBOUND_ROUNDS
constexpr double kCrustKernelSpreadSpacings = 0.6;   // CrustMap.KERNEL_SPREAD_SPACINGS (CrustMap.kt:521)
constexpr float kCoverShielding = 0.5f;              // BeltErosion.COVER_SHIELDING
constexpr float kPondDepthMetres = 24.0f;            // HydraulicErosion.POND_DEPTH_METRES

// The replay's scalars, as the reference forms them.
struct BeltConsts {
    float freeboard;       // (mantle - crust) / mantle * 1000, metres per km of crust
    float mpfu;            // WorldScale.reliefSpanMetres
    float pond;            // POND_DEPTH_METRES / mpfu
    float courant;         // HydraulicErosion.Rates.courantCoefficient
    float land_cells;      // the opening's land cells as a Float, at least 1
    float shoreline;       // the opening's shoreline
    float rate;            // ErosionConfig.rate
    float lim_ew, lim_ns, lim_diag, settled;
    float step_ns, step_diag;
    float rebound_share;   // crust / mantle
    double area;           // square metres per cell
    double round_years, round_myr, window_myr;
    int rounds, hydraulic_rounds;
};

__device__ __forceinline__ size_t tid() { return blockIdx.x * (size_t)blockDim.x + threadIdx.x; }
__device__ __forceinline__ size_t nthreads() { return (size_t)gridDim.x * blockDim.x; }

// Kotlin's Double.toInt(): toward zero, NaN to 0, saturating.
__host__ __device__ __forceinline__ int jvm_d2i(double x) {
    if (x != x) return 0;
    if (x >= 2147483647.0) return INT_MAX;
    if (x <= -2147483648.0) return INT_MIN;
    return (int)x;
}

// Math.min(float, float) on the JVM: NaN if either is, -0 below +0.
__device__ __forceinline__ float jvm_min(float a, float b) {
    if (a != a) return a;
    if (b != b) return b;
    if (a == 0.0f && b == 0.0f) return signbit(a) ? a : b;
    return a < b ? a : b;
}

__device__ __forceinline__ float limit_of(int rs, int cs, const BeltConsts& k) {
    return (rs != 0 && cs != 0) ? k.lim_diag : (rs != 0 ? k.lim_ns : k.lim_ew);
}

__global__ void k_fill_f(float* __restrict__ a, size_t N, float v) {
    for (size_t i = tid(); i < N; i += nthreads()) a[i] = v;
}

__global__ void k_widen(const float* __restrict__ h, size_t N, double* __restrict__ out) {
    for (size_t i = tid(); i < N; i += nthreads()) out[i] = (double)h[i];
}

// The belt (onset >= 0, BeltErosion.kt:127) and its scan flags.
__global__ void k_belt_mark(const float* __restrict__ onset, size_t N, uint8_t* __restrict__ belt,
                            int* __restrict__ flag) {
    for (size_t i = tid(); i < N; i += nthreads()) {
        const bool b = onset[i] >= 0.0f;
        belt[i] = b ? 1 : 0;
        flag[i] = b ? 1 : 0;
    }
}

// The belt's cells in index order, and each cell's local index (-1 off the belt).
__global__ void k_belt_list(const uint8_t* __restrict__ belt, const int* __restrict__ pos, size_t N,
                            int* __restrict__ list, int* __restrict__ local) {
    for (size_t i = tid(); i < N; i += nthreads()) {
        if (belt[i]) {
            list[pos[i]] = (int)i;
            local[i] = pos[i];
        } else {
            local[i] = -1;
        }
    }
}

// Each belt cell lowered to the window's start, its first round and its rise a round
// (BeltErosion.kt:132-144).
__global__ void k_belt_lower(const int* __restrict__ list, int B, const float* __restrict__ tectonic,
                             const float* __restrict__ wear, const float* __restrict__ onset,
                             const float* __restrict__ uplift, BeltConsts k, float* __restrict__ h,
                             int* __restrict__ first, float* __restrict__ rise) {
    for (size_t l = tid(); l < (size_t)B; l += nthreads()) {
        const int c = list[l];
        h[c] = __fsub_rn(h[c], __fdiv_rn(__fmul_rn(k.freeboard, __fsub_rn(tectonic[c], wear[c])), k.mpfu));
        const double share =
            uplift ? __ddiv_rn(__dmul_rn((double)__fmul_rn(uplift[c], (float)k.hydraulic_rounds), k.round_years), 1000.0)
                   : 0.0;
        const double rise_m = __dsub_rn((double)__fmul_rn(k.freeboard, tectonic[c]), share);
        int f = jvm_d2i(ceil(__dsub_rn(__ddiv_rn(__dsub_rn(k.window_myr, (double)onset[c]), k.round_myr), 1e-9)));
        f = f < 0 ? 0 : (f > k.rounds - 1 ? k.rounds - 1 : f);
        first[l] = f;
        rise[l] = __double2float_rn(__ddiv_rn(__ddiv_rn(rise_m, (double)(k.rounds - f)), (double)k.mpfu));
    }
}

// The rain's weights and the cover's and rock's factor over the opening's land means
// (BeltErosion.kt:151-163): sums[0] and sums[1] hold the means in double.
__global__ void k_belt_weights(const float* __restrict__ rain, const float* __restrict__ cover,
                               const float* __restrict__ rock, const double* __restrict__ sums, int shield,
                               size_t N, float* __restrict__ weights, float* __restrict__ factor) {
    const float rain_mean = __double2float_rn(sums[0]);
    const float cover_mean = __double2float_rn(sums[1]);
    for (size_t i = tid(); i < N; i += nthreads()) {
        weights[i] = rain_mean > 0.0f ? __fdiv_rn(rain[i], rain_mean) : 1.0f;
        const float cv = (shield && cover_mean > 0.0f)
                             ? __fdiv_rn(__fsub_rn(1.0f, __fmul_rn(kCoverShielding, cover[i])), cover_mean)
                             : 1.0f;
        factor[i] = __fmul_rn(cv, rock ? rock[i] : 1.0f);
    }
}

// The water reaching each belt cell from off the belts over the opening routing, its donors added in
// the order of their cell indices (BeltErosion.kt:174-180).
__global__ void k_belt_inflow(const int* __restrict__ list, int B, const int* __restrict__ local,
                              const int32_t* __restrict__ recv0, const float* __restrict__ area, int W, int H,
                              double* __restrict__ inflow) {
    for (size_t l = tid(); l < (size_t)B; l += nthreads()) {
        const int c = list[l];
        const int row = pdiv(c, W), col = pmod(c, W);
        int nb[8];
        int k = 0;
        for (int rs = -1; rs <= 1; ++rs) {
            const int nr = row + rs;
            if (nr < 0 || nr >= H) continue;
            for (int cs = -1; cs <= 1; ++cs) {
                if (rs == 0 && cs == 0) continue;
                const int n = nr * W + wrap_col(col + cs, W);
                if (local[n] >= 0 || recv0[n] != c) continue;
                int j = k++;
                while (j > 0 && nb[j - 1] > n) {
                    nb[j] = nb[j - 1];
                    --j;
                }
                nb[j] = n;
            }
        }
        double v = 0.0;
        for (int j = 0; j < k; ++j) v = __dadd_rn(v, (double)area[nb[j]]);
        inflow[c] = v;
    }
}

// The frontier (BeltErosion.kt:184-195): off-belt cells with a belt neighbour, as scan flags.
__global__ void k_frontier_flag(const int* __restrict__ local, int W, int H, int* __restrict__ flag) {
    const size_t N = (size_t)W * H;
    for (size_t i = tid(); i < N; i += nthreads()) {
        int f = 0;
        if (local[i] < 0) {
            const int row = pdiv((int)i, W), col = pmod((int)i, W);
            for (int rs = -1; rs <= 1 && !f; ++rs) {
                const int nr = row + rs;
                if (nr < 0 || nr >= H) continue;
                for (int cs = -1; cs <= 1; ++cs)
                    if (!(rs == 0 && cs == 0) && local[nr * W + wrap_col(col + cs, W)] >= 0) f = 1;
            }
        }
        flag[i] = f;
    }
}

__global__ void k_frontier_list(const int* __restrict__ flag, const int* __restrict__ pos, size_t N,
                                int* __restrict__ out) {
    for (size_t i = tid(); i < N; i += nthreads())
        if (flag[i]) out[pos[i]] = (int)i;
}

// The rise where the belt has begun to (BeltErosion.kt:240-248); xs[1 + l] the uplift book's term.
__global__ void k_belt_rise(const int* __restrict__ list, int B, const int* __restrict__ first,
                            const float* __restrict__ rise, int round, BeltConsts k, float* __restrict__ h,
                            float* __restrict__ uplifted_m, double* __restrict__ xs) {
    for (size_t l = tid(); l < (size_t)B; l += nthreads()) {
        double term = 0.0;
        if (round >= first[l]) {
            const int c = list[l];
            const float r = rise[l];
            h[c] = __fadd_rn(h[c], r);
            if (uplifted_m) uplifted_m[c] = __fadd_rn(uplifted_m[c], __fmul_rn(r, k.mpfu));
            term = __dmul_rn(__dmul_rn((double)r, (double)k.mpfu), k.area);
        }
        xs[1 + l] = term;
    }
}

__global__ void k_route_cells(const int* __restrict__ cells, int n, const float* __restrict__ h,
                              double* __restrict__ routing) {
    for (size_t j = tid(); j < (size_t)n; j += nthreads()) {
        const int c = cells[j];
        routing[c] = (double)h[c];
    }
}

// The belt flood's inner land and the facet rule's cells (BeltErosion.kt:257-292).
__global__ void k_belt_masks(const int* __restrict__ list, int B, const int* __restrict__ local,
                             const uint8_t* __restrict__ land, const float* __restrict__ h, BeltConsts k, int W,
                             int H, uint8_t* __restrict__ inner, uint8_t* __restrict__ routed) {
    for (size_t l = tid(); l < (size_t)B; l += nthreads()) {
        const int c = list[l];
        const int row = pdiv(c, W), col = pmod(c, W);
        const bool sea = !land[c] || h[c] <= k.shoreline;
        bool edge = row == 0 || row == H - 1;
        for (int rs = -1; rs <= 1 && !edge && !sea; ++rs) {
            const int nr = row + rs;
            for (int cs = -1; cs <= 1; ++cs)
                if (!(rs == 0 && cs == 0) && local[nr * W + wrap_col(col + cs, W)] < 0) edge = true;
        }
        inner[c] = (!sea && !edge) ? 1 : 0;
        routed[c] = sea ? 0 : 1;
    }
}

// The routing surface of the belt's land above the shoreline: its flood levels (BeltErosion.kt:285-288).
__global__ void k_route_filled(const int* __restrict__ list, int B, const uint8_t* __restrict__ routed,
                               const float* __restrict__ filled, double* __restrict__ routing) {
    for (size_t l = tid(); l < (size_t)B; l += nthreads()) {
        const int c = list[l];
        if (routed[c]) routing[c] = (double)filled[c];
    }
}

enum { LV_DISCHARGE = 0, LV_CUT = 1, LV_FLUX = 2 };

struct LevelArgs {
    int W, H, levels, mode;
    const int* bucket;          // belt cells by Kahn level
    const int* start;           // each level's first slot (levels + 1)
    const uint8_t* belt;
    const int32_t* recv;
    const long long* key;       // drainage keys
    const float* weights;
    const double* inflow;
    double* disc;
    const uint8_t* land;
    const float* filled;
    const float* unresolved;    // or null
    const float* factor;
    float* h;
    float* eroded;
    double* flux;
    double* cutv;
    BeltConsts k;
};

// v plus the donors' values of cell c (val), added in drainage-key order: the order the reference's
// FIFO hands them to c. Donors sit on lower levels, final before c's level runs.
__device__ double add_donors(const LevelArgs& a, int c, double v, const double* val) {
    const int row = pdiv(c, a.W), col = pmod(c, a.W);
    long long kk[8];
    int nn[8];
    int k = 0;
    for (int rs = -1; rs <= 1; ++rs) {
        const int nr = row + rs;
        if (nr < 0 || nr >= a.H) continue;
        for (int cs = -1; cs <= 1; ++cs) {
            if (rs == 0 && cs == 0) continue;
            const int n = nr * a.W + wrap_col(col + cs, a.W);
            if (!a.belt[n] || a.recv[n] != c) continue;
            const long long kn = a.key[n];
            int j = k++;
            while (j > 0 && kk[j - 1] > kn) {
                kk[j] = kk[j - 1];
                nn[j] = nn[j - 1];
                --j;
            }
            kk[j] = kn;
            nn[j] = n;
        }
    }
    for (int j = 0; j < k; ++j) v = __dadd_rn(v, __ldcg(&val[nn[j]]));
    return v;
}

// One cell of the cut, from the outlets up (BeltErosion.kt:327-351): its receiver's height is final.
__device__ void cut_cell(const LevelArgs& a, int c) {
    const BeltConsts& k = a.k;
    double t = 0.0;
    const int d = a.recv[c];
    if (d >= 0) {
        const float h = __ldcg(&a.h[c]);
        if (!(__fsub_rn(a.filled[c], h) > k.pond)) {
            const float own = a.unresolved ? a.unresolved[c] : 0.0f;
            const float hd = __ldcg(&a.h[d]);
            float base;
            if (!a.land[d] || hd <= k.shoreline) base = __fadd_rn(k.shoreline, own);
            else if (a.belt[d] && __fsub_rn(a.filled[d], hd) > k.pond) base = __fadd_rn(a.filled[d], own);
            else base = __fsub_rn(__fadd_rn(hd, own), a.unresolved ? a.unresolved[d] : 0.0f);
            if (!(h <= base)) {
                const double share = __ddiv_rn(__ldcg(&a.disc[c]), (double)k.land_cells);
                const bool same_row = pdiv(c, a.W) == pdiv(d, a.W), same_col = pmod(c, a.W) == pmod(d, a.W);
                const float step = (!same_row && !same_col) ? k.step_diag : (!same_row ? k.step_ns : 1.0f);
                const double cn = __ddiv_rn(__dmul_rn(__dmul_rn((double)k.courant, __dsqrt_rn(share)), (double)a.factor[c]),
                                            (double)step);
                const float after = __double2float_rn(
                    __dadd_rn((double)base, __ddiv_rn((double)__fsub_rn(h, base), __dadd_rn(1.0, cn))));
                __stcg(&a.h[c], after);
                const float lost = __fmul_rn(__fsub_rn(h, after), k.mpfu);
                a.eroded[c] = __fadd_rn(a.eroded[c], lost);
                t = __dmul_rn((double)lost, k.area);
            }
        }
    }
    __stcg(&a.flux[c], t);
    a.cutv[c] = t;
}

// The Kahn levels, upward for the discharge and the spoil flux, downward for the cut, one grid
// barrier between levels.
__global__ void __launch_bounds__(256) k_belt_levels(LevelArgs a) {
    cgr::grid_group g = cgr::this_grid();
    const int t = blockIdx.x * blockDim.x + threadIdx.x, nt = gridDim.x * blockDim.x;
    for (int s = 0; s < a.levels; ++s) {
        const int L = a.mode == LV_CUT ? a.levels - 1 - s : s;
        const int b1 = a.start[L + 1];
        for (int i = a.start[L] + t; i < b1; i += nt) {
            const int c = a.bucket[i];
            if (a.mode == LV_DISCHARGE) {
                const double v = add_donors(a, c, __dadd_rn((double)a.weights[c], a.inflow[c]), a.disc);
                __stcg(&a.disc[c], v);
            } else if (a.mode == LV_CUT) {
                cut_cell(a, c);
            } else {
                const double v = add_donors(a, c, __ldcg(&a.flux[c]), a.flux);
                __stcg(&a.flux[c], v);
            }
        }
        g.sync();
    }
}

// The books' terms in the reference's order after their running totals: the cut in reverse run order,
// the exports to the sea and to the land in run order (BeltErosion.kt:346-370).
__global__ void k_order_terms(const int* __restrict__ order, int B, const int32_t* __restrict__ recv,
                              const uint8_t* __restrict__ belt, const uint8_t* __restrict__ land,
                              const float* __restrict__ h, float shoreline, const double* __restrict__ flux,
                              const double* __restrict__ cutv, double* __restrict__ xcut,
                              double* __restrict__ xsea, double* __restrict__ xland) {
    for (size_t i = tid(); i < (size_t)B; i += nthreads()) {
        xcut[1 + i] = cutv[order[B - 1 - i]];
        const int c = order[i];
        const int d = recv[c];
        const double f = flux[c];
        double sea = 0.0, lnd = 0.0;
        if (d < 0) {
            if (!land[c] || h[c] <= shoreline) sea = f;
            else lnd = f;
        } else if (!belt[d]) {
            if (!land[d] || h[d] <= shoreline) sea = f;
            else lnd = f;
        }
        xsea[1 + i] = sea;
        xland[1 + i] = lnd;
    }
}

// One sweep's give rates of the belt cells (BeltErosion.kt:375-390).
__global__ void k_belt_give(const int* __restrict__ list, int B, const float* __restrict__ h, int W, int H,
                            BeltConsts k, float* __restrict__ give) {
    for (size_t l = tid(); l < (size_t)B; l += nthreads()) {
        const int c = list[l];
        const int row = pdiv(c, W), col = pmod(c, W);
        const float here = h[c];
        float excess = 0.0f, steepest = 0.0f;
        for (int rs = -1; rs <= 1; ++rs) {
            const int nr = row + rs;
            if (nr < 0 || nr >= H) continue;
            for (int cs = -1; cs <= 1; ++cs) {
                if (rs == 0 && cs == 0) continue;
                const float drop = __fsub_rn(here, h[nr * W + wrap_col(col + cs, W)]);
                if (drop > 0.0f) {
                    if (drop > steepest) steepest = drop;
                    const float limit = limit_of(rs, cs, k);
                    if (drop > limit) excess = __fadd_rn(excess, __fsub_rn(drop, limit));
                }
            }
        }
        give[c] = excess <= k.settled ? 0.0f
                                      : __fdiv_rn(jvm_min(__fmul_rn(k.rate, excess), __fmul_rn(steepest, 0.5f)), excess);
    }
}

// One sweep's new heights of the belt and its frontier (BeltErosion.kt:391-403).
__global__ void k_belt_next(const int* __restrict__ swept, int n, const int* __restrict__ local,
                            const float* __restrict__ h, const float* __restrict__ give, int W, int H, BeltConsts k,
                            float* __restrict__ next) {
    for (size_t j = tid(); j < (size_t)n; j += nthreads()) {
        const int c = swept[j];
        const int row = pdiv(c, W), col = pmod(c, W);
        const float here = h[c];
        const bool own = local[c] >= 0;
        float received = 0.0f, given = 0.0f;
        for (int rs = -1; rs <= 1; ++rs) {
            const int nr = row + rs;
            if (nr < 0 || nr >= H) continue;
            for (int cs = -1; cs <= 1; ++cs) {
                if (rs == 0 && cs == 0) continue;
                const int nb = nr * W + wrap_col(col + cs, W);
                const float limit = limit_of(rs, cs, k);
                const float incoming = __fsub_rn(h[nb], here);
                if (incoming > limit && local[nb] >= 0)
                    received = __fadd_rn(received, __fmul_rn(give[nb], __fsub_rn(incoming, limit)));
                else if (-incoming > limit && own)
                    given = __fadd_rn(given, __fmul_rn(give[c], __fsub_rn(-incoming, limit)));
            }
        }
        next[j] = __fadd_rn(__fsub_rn(here, given), received);
    }
}

// The sweep's heights written back; the frontier's change is the shed book's terms (BeltErosion.kt:404-407).
__global__ void k_belt_commit(const int* __restrict__ swept, int B, int F, const float* __restrict__ next,
                              BeltConsts k, float* __restrict__ h, double* __restrict__ xs) {
    for (size_t j = tid(); j < (size_t)(B + F); j += nthreads()) {
        const int c = swept[j];
        if (j >= (size_t)B)
            xs[j - B] = __dmul_rn(__dmul_rn((double)__fsub_rn(next[j], h[c]), (double)k.mpfu), k.area);
        h[c] = next[j];
    }
}

// The rock lost so far less the rebound already given (BeltErosion.kt:414-416).
__global__ void k_belt_loss(size_t N, const float* __restrict__ upl, const float* __restrict__ rbm,
                            const float* __restrict__ h, const float* __restrict__ ref, float mpfu,
                            float* __restrict__ loss) {
    for (size_t i = tid(); i < N; i += nthreads())
        loss[i] = __fsub_rn(__fadd_rn(upl[i], rbm[i]), __fmul_rn(__fsub_rn(h[i], ref[i]), mpfu));
}

// GaussianBlur.across: x wraps; each output a double sum over the taps in order.
__global__ void k_blur_across(const float* __restrict__ in, int W, int H, const double* __restrict__ taps,
                              int radius, float* __restrict__ out) {
    const size_t N = (size_t)W * H;
    for (size_t i = tid(); i < N; i += nthreads()) {
        const int row = pdiv((int)i, W), col = pmod((int)i, W);
        const float* line = in + (size_t)row * W;
        double sum = 0.0;
        for (int t = 0; t <= 2 * radius; ++t)
            sum = __dadd_rn(sum, __dmul_rn(taps[t], (double)line[wrap_col(col + t - radius, W)]));
        out[i] = __double2float_rn(sum);
    }
}

// GaussianBlur.down: y clamps at the poles.
__global__ void k_blur_down(const float* __restrict__ in, int W, int H, const double* __restrict__ taps, int radius,
                            float* __restrict__ out) {
    const size_t N = (size_t)W * H;
    for (size_t i = tid(); i < N; i += nthreads()) {
        const int row = pdiv((int)i, W), col = pmod((int)i, W);
        double sum = 0.0;
        for (int t = 0; t <= 2 * radius; ++t) {
            int src = row + t - radius;
            src = src < 0 ? 0 : (src > H - 1 ? H - 1 : src);
            sum = __dadd_rn(sum, __dmul_rn(taps[t], (double)in[(size_t)src * W + col]));
        }
        out[i] = __double2float_rn(sum);
    }
}

// The crust's answer (BeltErosion.kt:418-422).
__global__ void k_belt_rebound(size_t N, const float* __restrict__ loss, float share, float mpfu,
                               float* __restrict__ h, float* __restrict__ rbm) {
    for (size_t i = tid(); i < N; i += nthreads()) {
        const float rebound = __fmul_rn(share, loss[i]);
        h[i] = __fadd_rn(h[i], __fdiv_rn(__fsub_rn(rebound, rbm[i]), mpfu));
        rbm[i] = rebound;
    }
}

bool pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

cg_status check_grid(cg_ctx* ctx, int W, int H) {
    if (!pow2(W) || !pow2(H)) return fail(ctx, CG_BAD_ARG, "width/height must be powers of two (got %d x %d)", W, H);
    if ((int64_t)W * H > (int64_t)1 << 30) return fail(ctx, CG_BAD_ARG, "grid of %d x %d cells is too large", W, H);
    return CG_OK;
}

// GaussianBlur.weights (GaussianBlur.kt:53-65).
std::vector<double> gaussian_taps(double sigma) {
    int radius = jvm_d2i(std::ceil(4.0 * sigma));
    if (radius < 1) radius = 1;
    std::vector<double> taps(2 * (size_t)radius + 1);
    double total = 0.0;
    for (int off = -radius; off <= radius; ++off) {
        const double z = off / sigma;
        const double w = std::exp(-0.5 * z * z);
        taps[off + radius] = w;
        total += w;
    }
    for (double& t : taps) t /= total;
    return taps;
}

// GaussianBlur.apply on a device field, `tmp` a field of the same size.
cg_status gaussian_blur_dev(cg_ctx* ctx, int W, int H, float* d_field, float* d_tmp, double sigma_across,
                            double sigma_down) {
    const size_t N = (size_t)W * H;
    const int grid = ctx->num_sms * 8;
    cudaStream_t sm = ctx->stream;
    std::vector<double> across, down;
    if (sigma_across > 0.0) across = gaussian_taps(sigma_across);
    if (sigma_down > 0.0) down = gaussian_taps(sigma_down);
    if (across.size() > (size_t)INT_MAX / 2 || down.size() > (size_t)INT_MAX / 2)
        return fail(ctx, CG_BAD_ARG, "a blur of %g x %g cells is too wide", sigma_across, sigma_down);
    CG_BUF(double, d_taps, ctx, S_BT_TAPS, across.size() + down.size() + 1);
    if (!across.empty())
        CG_CUDA(ctx, cudaMemcpyAsync(d_taps, across.data(), across.size() * 8, cudaMemcpyHostToDevice, sm));
    if (!down.empty())
        CG_CUDA(ctx, cudaMemcpyAsync(d_taps + across.size(), down.data(), down.size() * 8, cudaMemcpyHostToDevice, sm));
    if (!across.empty()) {
        CG_LAUNCH(ctx) k_blur_across<<<grid, 256, 0, sm>>>(d_field, W, H, d_taps, (int)across.size() / 2, d_tmp);
        CG_CUDA(ctx, cudaMemcpyAsync(d_field, d_tmp, N * 4, cudaMemcpyDeviceToDevice, sm));
    }
    if (!down.empty()) {
        CG_LAUNCH(ctx) k_blur_down<<<grid, 256, 0, sm>>>(d_field, W, H, d_taps + across.size(), (int)down.size() / 2,
                                                         d_tmp);
        CG_CUDA(ctx, cudaMemcpyAsync(d_field, d_tmp, N * 4, cudaMemcpyDeviceToDevice, sm));
    }
    CG_CHECK_LAUNCH(ctx);
    // The host taps must outlive their copies.
    CG_CUDA(ctx, cudaStreamSynchronize(sm));
    return CG_OK;
}

}  // namespace

cg_status belt_replay_dev(cg_ctx* ctx, const cg_erosion_params& p, float* d_h, const BeltInputsDev& in,
                          double window_myr, const cg_belt_inputs& opt, float* d_eroded, cg_belt_books* books) {
    const int W = p.width, H = p.height;
    const size_t N = (size_t)W * H;
    const int grid = ctx->num_sms * 8;
    cudaStream_t sm = ctx->stream;
    *books = cg_belt_books{};
    CG_CUDA(ctx, cudaMemsetAsync(d_eroded, 0, N * 4, sm));

    const ScaleF sc = scale_of(p);
    BeltConsts k{};
    k.round_years = sc.years_per_round;
    k.round_myr = k.round_years / 1e6;
    const double main_myr = p.hydraulic_rounds * k.round_myr;
    k.window_myr = window_myr;
    k.rounds = jvm_d2i((window_myr - main_myr) / k.round_myr + 1e-9);   // ROUND_ROUNDING
    k.hydraulic_rounds = p.hydraulic_rounds;
    if (k.rounds <= 0 || p.hydraulic_rounds <= 0 || p.bedrock_erodibility_per_year <= 0.0f) return sync(ctx);

    // The belt (BeltErosion.kt:127-130).
    CG_BUF(uint8_t, d_belt, ctx, S_BT_BELT, N);
    CG_BUF(int, d_flag, ctx, S_BT_FLAG, N);
    CG_BUF(int, d_pos, ctx, S_BT_POS, N);
    CG_BUF(int, d_swept, ctx, S_BT_LIST, N);   // the belt, then its frontier
    CG_BUF(int, d_local, ctx, S_BT_LOCAL, N);
    CG_LAUNCH(ctx) k_belt_mark<<<grid, 256, 0, sm>>>(in.onset, N, d_belt, d_flag);
    CG_CHECK_LAUNCH(ctx);
    int B = 0;
    CG_TRY_ST(exclusive_scan(ctx, d_flag, d_pos, (int)N, &B));
    if (B == 0) return sync(ctx);
    CG_LAUNCH(ctx) k_belt_list<<<grid, 256, 0, sm>>>(d_belt, d_pos, N, d_swept, d_local);

    k.freeboard = (p.mantle_density - p.continental_crust_density) / p.mantle_density * 1000.0f;
    k.mpfu = sc.relief_span();
    CG_BUF(int, d_first, ctx, S_BT_FIRST, (size_t)B);
    CG_BUF(float, d_rise, ctx, S_BT_RISE, (size_t)B);
    CG_LAUNCH(ctx) k_belt_lower<<<grid, 256, 0, sm>>>(d_swept, B, in.tectonic, in.wear, in.onset, in.uplift, k, d_h,
                                                      d_first, d_rise);
    CG_CHECK_LAUNCH(ctx);

    // The opening's cut, weights and factors (BeltErosion.kt:147-163).
    CG_BUF(uint8_t, d_land, ctx, S_BT_LAND, N);
    CG_BUF(float, d_rel, ctx, S_BT_REL, N);
    float shoreline = 0.0f;
    int land_count = 0;
    CG_TRY_ST(percentile_cut_dev(ctx, W, H, d_h, opt.provisional_sea_level, std::fmax(sc.land_half(), 1e-6f),
                                 std::fmax(sc.sea_half(), 1e-6f), 0.0f, d_land, d_rel, &shoreline, &land_count));
    k.shoreline = shoreline;
    k.land_cells = std::fmax((float)land_count, 1.0f);
    CG_BUF(double, d_small, ctx, S_BT_SMALL, 8);   // the two means, then the five books
    double* d_books = d_small + 2;
    CG_CUDA(ctx, cudaMemsetAsync(d_books, 0, 5 * sizeof(double), sm));
    CG_TRY_ST(seq_sum_dev(ctx, in.rain, d_land, 0, N, (double)k.land_cells, d_small, nullptr));
    CG_TRY_ST(seq_sum_dev(ctx, in.cover, d_land, 1, N, (double)k.land_cells, d_small + 1, nullptr));
    CG_BUF(float, d_weights, ctx, S_BT_WEIGHTS, N);
    CG_BUF(float, d_factor, ctx, S_BT_FACTOR, N);
    CG_LAUNCH(ctx) k_belt_weights<<<grid, 256, 0, sm>>>(in.rain, in.cover, in.rock, d_small, opt.shield_cut != 0, N,
                                                        d_weights, d_factor);
    CG_CHECK_LAUNCH(ctx);

    // The water from beyond the belts over the opening's routing (BeltErosion.kt:166-181).
    const double r = sc.cell_height_km(H) / sc.cell_width_km(W);
    CG_BUF(float, d_filled, ctx, S_BT_FILLED, N);
    CG_BUF(double, d_surf, ctx, S_BT_SURF, N);
    CG_BUF(int32_t, d_recv, ctx, S_BT_RECV, N);
    CG_BUF(long long, d_key, ctx, S_BT_KEY, N);
    CG_BUF(int32_t, d_donors, ctx, S_BT_DONORS, N);
    CG_BUF(float, d_area, ctx, S_BT_AREA, N);
    CG_BUF(double, d_inflow, ctx, S_BT_INFLOW, N);
    CG_TRY_ST(fill_depressions_dev(ctx, W, H, d_land, d_rel, d_filled, nullptr, nullptr));
    FlatCounts fc{0, 0, 0};
    CG_TRY_ST(flow_directions_dev(ctx, W, H, d_land, d_rel, d_filled, p.seed, r,
                                  smooth_field_lattice_columns(sc.world_width_km), p.facet_routing != 0,
                                  p.flat_potential != 0, d_recv, d_surf, &fc));
    CG_TRY_ST(tree_walk_dev(ctx, W, H, d_land, d_recv, d_weights, d_key, d_donors, d_area, nullptr));
    CG_LAUNCH(ctx) k_belt_inflow<<<grid, 256, 0, sm>>>(d_swept, B, d_local, d_recv, d_area, W, H, d_inflow);

    // The frontier (BeltErosion.kt:184-195), laid after the belt.
    CG_LAUNCH(ctx) k_frontier_flag<<<grid, 256, 0, sm>>>(d_local, W, H, d_flag);
    CG_CHECK_LAUNCH(ctx);
    int F = 0;
    CG_TRY_ST(exclusive_scan(ctx, d_flag, d_pos, (int)N, &F));
    CG_LAUNCH(ctx) k_frontier_list<<<grid, 256, 0, sm>>>(d_flag, d_pos, N, d_swept + B);
    CG_CHECK_LAUNCH(ctx);

    const RatesF rates = rates_of(p);
    const cg_thermal_limits lim = thermal_limits(p);
    const int hr = p.hydraulic_rounds < 1 ? 1 : p.hydraulic_rounds;
    int sweeps = sweeps_for(p) / hr;
    if (sweeps < 1) sweeps = 1;
    k.pond = kPondDepthMetres / k.mpfu;
    k.courant = rates.courant_coefficient;
    k.rate = p.rate;
    k.lim_ew = lim.east_west;
    k.lim_ns = lim.north_south;
    k.lim_diag = lim.diagonal;
    k.settled = lim.east_west * 1e-3f;   // SETTLED_SHARE_OF_CRITICAL_SLOPE
    k.step_ns = (float)r;
    k.step_diag = (float)std::sqrt(1.0 + r * r);
    k.area = sc.cell_width_km(W) * sc.cell_height_km(H) * 1e6;
    k.rebound_share = p.continental_crust_density / p.mantle_density;

    // The round state.
    CG_BUF(double, d_routing, ctx, S_BT_ROUTING, N);
    CG_BUF(uint8_t, d_inner, ctx, S_BT_INNER, N);
    CG_BUF(uint8_t, d_routed, ctx, S_BT_ROUTED, N);
    CG_BUF(double, d_disc, ctx, S_BT_DISC, N);
    CG_BUF(double, d_flux, ctx, S_BT_FLUX, N);
    CG_BUF(double, d_cutv, ctx, S_BT_CUTV, N);
    CG_BUF(float, d_give, ctx, S_BT_GIVE, N);
    CG_BUF(float, d_next, ctx, S_BT_NEXT, N);
    CG_BUF(int32_t, d_order, ctx, S_BT_ORDER, (size_t)B);
    const size_t xs_len = std::max(4 * ((size_t)B + 1), 1 + (size_t)sweeps * F);
    CG_BUF(double, d_xs, ctx, S_BT_XS, xs_len);
    double* xs_rise = d_xs;
    double* xs_cut = d_xs + (B + 1);
    double* xs_sea = d_xs + 2 * ((size_t)B + 1);
    double* xs_land = d_xs + 3 * ((size_t)B + 1);
    double* xs_shed = d_xs;   // after the others are summed
    CG_LAUNCH(ctx) k_widen<<<grid, 256, 0, sm>>>(d_h, N, d_routing);
    CG_CUDA(ctx, cudaMemsetAsync(d_inner, 0, N, sm));
    CG_CUDA(ctx, cudaMemsetAsync(d_routed, 0, N, sm));
    const bool rebound = opt.rebound != 0;
    float *d_ref = nullptr, *d_uplm = nullptr, *d_rbm = nullptr, *d_loss = nullptr, *d_tmp = nullptr;
    if (rebound) {
        CG_BUF(float, a, ctx, S_BT_REF, N);
        CG_BUF(float, b, ctx, S_BT_UPLM, N);
        CG_BUF(float, c, ctx, S_BT_RBM, N);
        CG_BUF(float, d, ctx, S_BT_LOSS, N);
        CG_BUF(float, e, ctx, S_BT_TMP, N);
        d_ref = a;
        d_uplm = b;
        d_rbm = c;
        d_loss = d;
        d_tmp = e;
        CG_CUDA(ctx, cudaMemcpyAsync(d_ref, d_h, N * 4, cudaMemcpyDeviceToDevice, sm));
        CG_CUDA(ctx, cudaMemsetAsync(d_uplm, 0, N * 4, sm));
        CG_CUDA(ctx, cudaMemsetAsync(d_rbm, 0, N * 4, sm));
    }
    const double crust_spread_km = kCrustKernelSpreadSpacings * opt.history_cell_km;
    int per_sm = 0;
    CG_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_belt_levels, 256, 0));
    if (per_sm < 1) return fail(ctx, CG_CUDA, "the belt's level kernel cannot be resident");
    const int cgrid = ctx->num_sms * (per_sm < 2 ? per_sm : 2);
    const int bgrid = std::min(grid, (B + 255) / 256 + 1);

    LevelArgs la{};
    la.W = W;
    la.H = H;
    la.belt = d_belt;
    la.recv = d_recv;
    la.key = d_key;
    la.weights = d_weights;
    la.inflow = d_inflow;
    la.disc = d_disc;
    la.land = d_land;
    la.filled = d_filled;
    la.unresolved = in.unresolved;
    la.factor = d_factor;
    la.h = d_h;
    la.eroded = d_eroded;
    la.flux = d_flux;
    la.cutv = d_cutv;
    la.k = k;

    for (int round = 0; round < k.rounds; ++round) {
        if (ctx->cancel.exchange(0)) return fail(ctx, CG_CANCELLED, "cancelled");
        // The rise and its book (BeltErosion.kt:240-249).
        CG_LAUNCH(ctx) k_belt_rise<<<bgrid, 256, 0, sm>>>(d_swept, B, d_first, d_rise, round, k, d_h, d_uplm, xs_rise);
        CG_CUDA(ctx, cudaMemcpyAsync(xs_rise, d_books + 0, 8, cudaMemcpyDeviceToDevice, sm));
        CG_TRY_ST(seq_sum_f64_dev(ctx, xs_rise, (size_t)B + 1, d_books + 0));
        CG_LAUNCH(ctx) k_route_cells<<<grid, 256, 0, sm>>>(d_swept, B + F, d_h, d_routing);
        // The spill levels, the routing surface and the facet receivers (BeltErosion.kt:253-292).
        CG_LAUNCH(ctx) k_belt_masks<<<bgrid, 256, 0, sm>>>(d_swept, B, d_local, d_land, d_h, k, W, H, d_inner, d_routed);
        CG_CHECK_LAUNCH(ctx);
        CG_TRY_ST(fill_depressions_dev(ctx, W, H, d_inner, d_h, d_filled, nullptr, nullptr));
        CG_LAUNCH(ctx) k_route_filled<<<bgrid, 256, 0, sm>>>(d_swept, B, d_routed, d_filled, d_routing);
        CG_CHECK_LAUNCH(ctx);
        CG_TRY_ST(facet_receivers_dev(ctx, W, H, d_routed, d_routing, p.seed, r, d_recv));
        // The run order (BeltErosion.kt:296-311).
        int levels = 0;
        CG_TRY_ST(tree_walk_dev(ctx, W, H, d_belt, d_recv, nullptr, d_key, d_donors, nullptr, &levels));
        int *d_bucket = nullptr, *d_start = nullptr;
        CG_TRY_ST(level_buckets_dev(ctx, W, H, d_belt, d_key, levels, &d_bucket, &d_start));
        CG_TRY_ST(order_from_keys_dev(ctx, W, H, d_belt, d_key, B, d_order));
        // Discharge, the cut and the spoil's flux, level by level (BeltErosion.kt:313-370).
        la.levels = levels;
        la.bucket = d_bucket;
        la.start = d_start;
        for (int mode : {LV_DISCHARGE, LV_CUT, LV_FLUX}) {
            la.mode = mode;
            void* kargs[] = {&la};
            ctx->launches++;
            CG_CUDA(ctx, cudaLaunchCooperativeKernel((void*)k_belt_levels, cgrid, 256, kargs, 0, sm));
        }
        CG_LAUNCH(ctx) k_order_terms<<<bgrid, 256, 0, sm>>>(d_order, B, d_recv, d_belt, d_land, d_h, k.shoreline,
                                                            d_flux, d_cutv, xs_cut, xs_sea, xs_land);
        CG_CHECK_LAUNCH(ctx);
        CG_CUDA(ctx, cudaMemcpyAsync(xs_cut, d_books + 1, 8, cudaMemcpyDeviceToDevice, sm));
        CG_CUDA(ctx, cudaMemcpyAsync(xs_sea, d_books + 2, 8, cudaMemcpyDeviceToDevice, sm));
        CG_CUDA(ctx, cudaMemcpyAsync(xs_land, d_books + 3, 8, cudaMemcpyDeviceToDevice, sm));
        CG_TRY_ST(seq_sum_f64_dev(ctx, xs_cut, (size_t)B + 1, d_books + 1));
        CG_TRY_ST(seq_sum_f64_dev(ctx, xs_sea, (size_t)B + 1, d_books + 2));
        CG_TRY_ST(seq_sum_f64_dev(ctx, xs_land, (size_t)B + 1, d_books + 3));
        // The slopes (BeltErosion.kt:373-408), the frontier's changes the shed book's terms.
        for (int s = 0; s < sweeps; ++s) {
            CG_LAUNCH(ctx) k_belt_give<<<bgrid, 256, 0, sm>>>(d_swept, B, d_h, W, H, k, d_give);
            CG_LAUNCH(ctx) k_belt_next<<<grid, 256, 0, sm>>>(d_swept, B + F, d_local, d_h, d_give, W, H, k, d_next);
            CG_LAUNCH(ctx) k_belt_commit<<<grid, 256, 0, sm>>>(d_swept, B, F, d_next, k, d_h, xs_shed + 1 + (size_t)s * F);
        }
        CG_CHECK_LAUNCH(ctx);
        CG_CUDA(ctx, cudaMemcpyAsync(xs_shed, d_books + 4, 8, cudaMemcpyDeviceToDevice, sm));
        CG_TRY_ST(seq_sum_f64_dev(ctx, xs_shed, 1 + (size_t)sweeps * F, d_books + 4));
        // The crust's answer to the rock taken so far (BeltErosion.kt:413-423).
        if (rebound && ((round + 1) % kReboundRounds == 0 || round == k.rounds - 1)) {
            CG_LAUNCH(ctx) k_belt_loss<<<grid, 256, 0, sm>>>(N, d_uplm, d_rbm, d_h, d_ref, k.mpfu, d_loss);
            CG_CHECK_LAUNCH(ctx);
            CG_TRY_ST(gaussian_blur_dev(ctx, W, H, d_loss, d_tmp, crust_spread_km / sc.cell_width_km(W),
                                        crust_spread_km / sc.cell_height_km(H)));
            CG_LAUNCH(ctx) k_belt_rebound<<<grid, 256, 0, sm>>>(N, d_loss, k.rebound_share, k.mpfu, d_h, d_rbm);
            CG_CHECK_LAUNCH(ctx);
        }
    }
    double h_books[5];
    CG_CUDA(ctx, cudaMemcpyAsync(h_books, d_books, sizeof(h_books), cudaMemcpyDeviceToHost, sm));
    CG_TRY_ST(sync(ctx));
    books->rounds = k.rounds;
    books->belt_cells = B;
    books->uplifted_cubic_meters = h_books[0];
    books->cut_cubic_meters = h_books[1];
    books->exported_to_sea_cubic_meters = h_books[2];
    books->exported_to_land_cubic_meters = h_books[3];
    books->shed_beside_cubic_meters = h_books[4];
    return CG_OK;
}

cg_status belt_window_dev(cg_ctx* ctx, const cg_erosion_params& p, const cg_belt_window& w, BeltInputsDev* in) {
    const size_t N = (size_t)p.width * p.height;
    const float** dst[3] = {&in->tectonic, &in->wear, &in->onset};
    const float* src[3] = {w.tectonic_km, w.wear_km, w.onset_myr_ago};
    const int slots[3] = {S_BT_TECT, S_BT_WEAR, S_BT_ONSET};
    for (int i = 0; i < 3; ++i) {
        cg_status st = CG_OK;
        float* d = (float*)buf(ctx, slots[i], N * 4, &st);
        if (st != CG_OK) return st;
        CG_CUDA(ctx, cudaMemcpyAsync(d, src[i], N * 4, cudaMemcpyHostToDevice, ctx->stream));
        *dst[i] = d;
    }
    return CG_OK;
}

cg_status belt_weather_dev(cg_ctx* ctx, int W, int H, const float* d_rain, const float* d_cover, BeltInputsDev* in) {
    const size_t N = (size_t)W * H;
    const int grid = ctx->num_sms * 8;
    in->rain = d_rain;
    in->cover = d_cover;
    if (!in->rain) {
        CG_BUF(float, d, ctx, S_BT_RAIN, N);
        CG_LAUNCH(ctx) k_fill_f<<<grid, 256, 0, ctx->stream>>>(d, N, 1.0f);
        in->rain = d;
    }
    if (!in->cover) {
        CG_BUF(float, d, ctx, S_BT_COVER, N);
        CG_LAUNCH(ctx) k_fill_f<<<grid, 256, 0, ctx->stream>>>(d, N, 0.0f);
        in->cover = d;
    }
    CG_CHECK_LAUNCH(ctx);
    return CG_OK;
}

namespace {

// Uploads one optional host field into its slot (null stays null).
cg_status upload_optional(cg_ctx* ctx, int slot, const float* host, size_t N, const float** d) {
    *d = nullptr;
    if (!host) return CG_OK;
    cg_status st = CG_OK;
    float* p = (float*)buf(ctx, slot, N * 4, &st);
    if (st != CG_OK) return st;
    CG_CUDA(ctx, cudaMemcpyAsync(p, host, N * 4, cudaMemcpyHostToDevice, ctx->stream));
    *d = p;
    return CG_OK;
}

}  // namespace
}  // namespace cg

using namespace cg;

extern "C" cg_status cg_belt_replay(cg_ctx* ctx, const cg_erosion_params* params, float* height,
                                    const cg_belt_window* window, const cg_belt_inputs* inputs, float* eroded_meters,
                                    cg_belt_books* books) {
    if (!ctx || !params || !height || !window || !inputs || !books || !window->tectonic_km || !window->wear_km ||
        !window->onset_myr_ago)
        return CG_BAD_ARG;
    ctx->run.active = false;   // this call reuses the context's buffers
    if (params->abi_version != CG_ABI_VERSION)
        return fail(ctx, CG_BAD_ARG, "params carry ABI version %u, this library is %u", params->abi_version,
                    CG_ABI_VERSION);
    CG_TRY_ST(check_grid(ctx, params->width, params->height));
    if (params->mode != CG_MODE_REF32) return fail(ctx, CG_UNSUPPORTED, "only the REF32 mode is built");
    if (!(params->mantle_density > 0.0f)) return fail(ctx, CG_BAD_ARG, "mantle density must be positive");
    CG_CUDA(ctx, cudaSetDevice(ctx->device));
    const size_t N = (size_t)params->width * params->height;
    cudaStream_t sm = ctx->stream;
    CG_BUF(float, d_h, ctx, S_BT_H, N);
    CG_CUDA(ctx, cudaMemcpyAsync(d_h, height, N * 4, cudaMemcpyHostToDevice, sm));
    BeltInputsDev in{};
    const float *d_rain, *d_cover;
    CG_TRY_ST(belt_window_dev(ctx, *params, *window, &in));
    CG_TRY_ST(upload_optional(ctx, S_BT_UPLIFT, inputs->uplift_mm_per_year, N, &in.uplift));
    CG_TRY_ST(upload_optional(ctx, S_BT_ROCK, inputs->rock_erodibility, N, &in.rock));
    CG_TRY_ST(upload_optional(ctx, S_BT_UNRES, inputs->unresolved_relief, N, &in.unresolved));
    CG_TRY_ST(upload_optional(ctx, S_BT_RAIN, inputs->rainfall_mm, N, &d_rain));
    CG_TRY_ST(upload_optional(ctx, S_BT_COVER, inputs->cover_density, N, &d_cover));
    CG_TRY_ST(belt_weather_dev(ctx, params->width, params->height, d_rain, d_cover, &in));
    CG_BUF(float, d_eroded, ctx, S_BT_ERODED, N);
    CG_TRY_ST(belt_replay_dev(ctx, *params, d_h, in, window->window_myr, *inputs, d_eroded, books));
    CG_CUDA(ctx, cudaMemcpyAsync(height, d_h, N * 4, cudaMemcpyDeviceToHost, sm));
    if (eroded_meters) CG_CUDA(ctx, cudaMemcpyAsync(eroded_meters, d_eroded, N * 4, cudaMemcpyDeviceToHost, sm));
    CG_CUDA(ctx, cudaStreamSynchronize(sm));
    return CG_OK;
}

extern "C" cg_status cg_gaussian_blur(cg_ctx* ctx, int32_t width, int32_t height, float* field, double sigma_across,
                                      double sigma_down) {
    if (!ctx || !field) return CG_BAD_ARG;
    ctx->run.active = false;
    CG_TRY_ST(check_grid(ctx, width, height));
    CG_CUDA(ctx, cudaSetDevice(ctx->device));
    const size_t N = (size_t)width * height;
    CG_BUF(float, d_f, ctx, S_BT_LOSS, N);
    CG_BUF(float, d_t, ctx, S_BT_TMP, N);
    CG_CUDA(ctx, cudaMemcpyAsync(d_f, field, N * 4, cudaMemcpyHostToDevice, ctx->stream));
    CG_TRY_ST(gaussian_blur_dev(ctx, width, height, d_f, d_t, sigma_across, sigma_down));
    CG_CUDA(ctx, cudaMemcpyAsync(field, d_f, N * 4, cudaMemcpyDeviceToHost, ctx->stream));
    CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return CG_OK;
}

extern "C" cg_status cg_sequential_sum_f64(cg_ctx* ctx, const double* x, int64_t n, double* sum) {
    if (!ctx || !sum || n < 0 || (n > 0 && !x)) return CG_BAD_ARG;
    ctx->run.active = false;
    CG_CUDA(ctx, cudaSetDevice(ctx->device));
    const size_t N = (size_t)n;
    CG_BUF(double, d_x, ctx, S_BT_XS, N + 1);
    CG_BUF(double, d_out, ctx, S_BT_SMALL, 8);
    if (N) CG_CUDA(ctx, cudaMemcpyAsync(d_x, x, N * 8, cudaMemcpyHostToDevice, ctx->stream));
    CG_TRY_ST(seq_sum_f64_dev(ctx, d_x, N, d_out));
    CG_CUDA(ctx, cudaMemcpyAsync(sum, d_out, 8, cudaMemcpyDeviceToHost, ctx->stream));
    CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return CG_OK;
}
