// FlowRouting.flowDirections (FlowRouting.kt:179-448) with FlatRouting.surfaceOf
// (FlatRouting.kt:58-518) on the device.
//
// Routing surface: the filled field (ocean cells their own ground), except across each raised flat,
// where the potential of a Poisson problem is laid into the band between the flat's highest entry
// and its lowest raised level. Flats are 8-connected components of raised cells and never touch one
// another, so each is solved on its own: a warp per flat of up to 32 members (nearly all of them: the
// fill's small depressions), a CTA per flat of up to 512 members and a cluster of 8 CTAs per flat of
// up to 16384, with the solver's vectors in shared memory, and in global memory beyond:
//  - members are ordered by (column, row), so each column run is a contiguous segment and the
//    reduction order is fixed (results are deterministic run to run);
//  - each member's weighted degree and its Laplacian row are accumulated in the reference's
//    neighbour order, and each column run's Thomas factorisation and solves are done by one thread
//    in the reference's order, so both are bit-identical to FlatRouting's;
//  - the conjugate-gradient dot products are block reductions, where the reference sums members in
//    DFS order: the potential may differ from the reference's in its last bits (it is an
//    intermediate, laid into a band whose order the receivers read).
// The facet rule (Tarboton's D-infinity facets on ground-true legs, then the Rho8 draw from the
// SplitMix64 cell hash) is a per-cell stencil in double, bit-exact.
#include <algorithm>
#include <cfloat>
#include <cooperative_groups.h>
#include <climits>

#include "cg_common.cuh"
#include "cg_internal.h"
#include "cg_util.h"

namespace cg {

namespace {

// FlowRouting.seededNoise (FlowRouting.kt:426-436): SplitMix64 on wrapping 64-bit integers.
__device__ __forceinline__ float seeded_noise(int lc, int lr, long long seed) {
    unsigned long long m = (unsigned long long)seed ^ ((unsigned long long)(long long)lc * 0x9E3779B97F4A7C15ull) ^
                           ((unsigned long long)(long long)lr * 0x27220A951D5A2B1Full);
    m ^= m >> 30;
    m *= 0xBF58476D1CE4E5B9ull;
    m ^= m >> 27;
    m *= 0x94D049BB133111EBull;
    m ^= m >> 31;
    int top = (int)(m >> 40);
    return __fsub_rn(__fdiv_rn((float)top, 8388608.0f), 1.0f);
}

__device__ __forceinline__ float lerpf(float a, float b, float t) { return __fadd_rn(a, __fmul_rn(__fsub_rn(b, a), t)); }

// FlowRouting.smoothSeededField (FlowRouting.kt:377-397).
__device__ float smooth_seeded_field(int W, int lattice, int col, int row, long long seed) {
    int cal = col * lattice, ral = row * lattice;
    int ccol = pdiv(cal, W), crow = pdiv(ral, W);
    float ac = __fdiv_rn((float)(cal - ccol * W), (float)W);
    float ar = __fdiv_rn((float)(ral - crow * W), (float)W);
    float ec = __fmul_rn(__fmul_rn(ac, ac), __fsub_rn(3.0f, __fmul_rn(2.0f, ac)));
    float er = __fmul_rn(__fmul_rn(ar, ar), __fsub_rn(3.0f, __fmul_rn(2.0f, ar)));
    int west = ccol % lattice, east = (ccol + 1) % lattice;
    float north = lerpf(seeded_noise(west, crow, seed), seeded_noise(east, crow, seed), ec);
    float south = lerpf(seeded_noise(west, crow + 1, seed), seeded_noise(east, crow + 1, seed), ec);
    return lerpf(north, south, er);
}

constexpr long long kSubGridDrawSalt = 0x5f3a91c72b64d8e3LL;   // FlowRouting.kt:358
constexpr long long kRainReliefSalt = 0x3c6ef372fe94f82bLL;    // FlatRouting.kt:507

struct Steps {
    float ew, ns, diag;   // GroundSteps (MA/GroundSteps.kt)
    __device__ float of(int dc, int dr) const { return (dc != 0 && dr != 0) ? diag : (dr != 0 ? ns : ew); }
};

__device__ __forceinline__ int neighbour_at(int W, int H, int col, int row) {
    if (row < 0 || row >= H) return -1;
    return row * W + wrap_col(col, W);
}

// x / d, skipping the division by a leg of exactly one cell width (x / 1.0 is x in IEEE arithmetic).
__device__ __forceinline__ double div_leg(double x, double d) {
    return __double_as_longlong(d) == 0x3FF0000000000000LL ? x : __ddiv_rn(x, d);
}

// Comparisons of doubles on the integer pipes (GB300 issues FP64 instructions, compares included,
// at a small fraction of its integer rate). For values that are not NaN, dkey maps a double to a
// signed integer in IEEE order, with -0 and +0 equal; x > 0 is the sign-and-magnitude test.
__device__ __forceinline__ long long dkey(double x) {
    const long long b = __double_as_longlong(x);
    return b >= 0 ? b : -(b & 0x7FFFFFFFFFFFFFFFLL);
}
__device__ __forceinline__ bool dpos(double x) { return __double_as_longlong(x) > 0; }

// Exact early outs for a facet's slope against the steepest so far (steepest >= 0). A correctly
// rounded result can exceed steepest only if the exact one does: for fl(sqrt(s)) that needs
// s > steepest^2, for fl(df / dg) (dg > 0) df > steepest * dg. Each exact product q lies within half
// a unit in the last place of its rounded value t, hence above the double just below t, so a value
// at or below that double is below q and its slope cannot win. Non-negative doubles order as their
// bit patterns, and the double just below a positive t has the bit pattern of t minus one.
__device__ __forceinline__ bool sqrt_cannot_win(double s, double steepest) {
    const long long t = __double_as_longlong(__dmul_rn(steepest, steepest));
    return t > 0 ? __double_as_longlong(s) <= t - 1 : __double_as_longlong(s) == 0;
}
__device__ __forceinline__ bool ratio_cannot_win(double df, double dg, double steepest) {
    if (!dpos(df)) return true;   // df / dg <= 0 <= steepest
    const long long t = __double_as_longlong(__dmul_rn(steepest, dg));
    return t > 0 && __double_as_longlong(df) <= t - 1;
}

// FlowRouting.facetReceiver (FlowRouting.kt:223-310), with the same values in fewer FP64 operations:
//  - a cardinal's slope is shared by its two facets and a diagonal's by its two facets, so each is
//    computed once, and a diagonal's only if a facet is clamped to it and could be the steepest;
//  - an inside facet's square root is taken only if its slope could be the steepest (the early
//    outs above), and comparisons run on the integer pipes;
//  - the share along the far edge, a / b with a = outward tc^2 and b = cdrop od^2 (rounded products,
//    as the reference forms them), is compared with 1 as a >= b: for positive doubles fl(a/b) >= 1
//    exactly when a >= b, since a < b puts a/b at or below the double just under 1. The division is
//    taken once, for the winning facet, whose share the draw is compared with;
//  - UNIT: both legs are exactly one cell width (square cells), so the products and quotients by a
//    leg are the values themselves.
// Facets are visited and compared in the reference's order, so ties resolve identically.
template <bool UNIT>
__device__ int facet_receiver(int W, int H, const double* __restrict__ rs, int col, int row, Steps st, long long seed) {
    const int ccs_t[4] = {1, 0, -1, 0};
    const int crs_t[4] = {0, -1, 0, 1};
    const double here = rs[row * W + col];
    const double ew = (double)st.ew, ns = (double)st.ns, dg = (double)st.diag;
    // Diagonal falls and slopes, indexed by (column step, row step) = (+-1, +-1).
    double dfall[4];
    double dslope[4];
    bool dslope_done[4] = {false, false, false, false};
    int dcell[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        int dcs = (k & 1) ? 1 : -1, drs = (k & 2) ? 1 : -1;
        dcell[k] = neighbour_at(W, H, col + dcs, row + drs);
        dfall[k] = dcell[k] >= 0 ? __dsub_rn(here, rs[dcell[k]]) : 0.0;
    }
    double steepest = 0.0;
    int fcard = -1, fdiag = -1;
    int mode = 0;   // 0: cardinal, 1: diagonal, 2: inside the facet (share a / b)
    double wa = 0.0, wb = 0.0;
#pragma unroll
    for (int side = 0; side < 4; ++side) {
        const int ccs = ccs_t[side], crs = crs_t[side];
        const int card = neighbour_at(W, H, col + ccs, row + crs);
        if (card < 0) continue;
        const double cdrop = __dsub_rn(here, rs[card]);
        const double to_card = ccs != 0 ? ew : ns;     // GroundSteps.of(ccs, crs): never a diagonal here
        const double on_to_diag = ccs == 0 ? ew : ns;
        const double cslope = UNIT ? cdrop : div_leg(cdrop, to_card);
        const bool cdown = dpos(cdrop);
#pragma unroll
        for (int turn = -1; turn <= 1; turn += 2) {
            const int dcs = ccs == 0 ? turn : ccs;
            const int drs = crs == 0 ? turn : crs;
            const int k = (dcs > 0 ? 1 : 0) | (drs > 0 ? 2 : 0);
            if (dcell[k] < 0) continue;
            const double df = dfall[k];
            const double outward = __dsub_rn(df, cdrop);
            double a = 0.0, b = 0.0;
            bool wins;
            int m;
            if (cdown && !dpos(outward)) {   // to the cardinal
                wins = dkey(cslope) > dkey(steepest);
                if (wins) steepest = cslope;
                m = 0;
            } else {
                bool to_diagonal = true;   // share 1 when the cardinal is not downhill
                if (cdown) {
                    a = UNIT ? outward : __dmul_rn(__dmul_rn(outward, to_card), to_card);
                    b = UNIT ? cdrop : __dmul_rn(__dmul_rn(cdrop, on_to_diag), on_to_diag);
                    to_diagonal = dkey(a) >= dkey(b);
                }
                if (to_diagonal) {
                    wins = false;
                    if (dslope_done[k] || !ratio_cannot_win(df, dg, steepest)) {
                        if (!dslope_done[k]) {
                            dslope[k] = __ddiv_rn(df, dg);
                            dslope_done[k] = true;
                        }
                        wins = dkey(dslope[k]) > dkey(steepest);
                        if (wins) steepest = dslope[k];
                    }
                    m = 1;
                } else {
                    const double oslope = UNIT ? outward : div_leg(outward, on_to_diag);
                    const double sq = __dadd_rn(__dmul_rn(cslope, cslope), __dmul_rn(oslope, oslope));
                    wins = false;
                    if (!sqrt_cannot_win(sq, steepest)) {
                        const double fslope = __dsqrt_rn(sq);
                        wins = dkey(fslope) > dkey(steepest);
                        if (wins) steepest = fslope;
                    }
                    m = 2;
                }
            }
            if (wins) {
                fcard = card;
                fdiag = dcell[k];
                mode = m;
                wa = a;
                wb = b;
            }
        }
    }
    if (!dpos(steepest)) return -1;
    if (mode == 0) return fcard;
    if (mode == 1) return fdiag;
    const double share = __ddiv_rn(wa, wb);
    if (!dpos(share)) return fcard;
    // FlowRouting.subGridDraw (FlowRouting.kt:355-356).
    const double draw = (double)__fmul_rn(__fadd_rn(seeded_noise(col, row, seed ^ kSubGridDrawSalt), 1.0f), 0.5f);
    return dkey(draw) < dkey(share) ? fdiag : fcard;
}

// facet_receiver<true> for the 32 cells a warp holds (cell < 0: an idle lane), with the expensive
// FP64 operations taken densely. An FP64 warp instruction holds the pipe whatever its active lanes, and
// in the per-lane form each facet's division and square root run under a branch that only some lanes
// take. Here every lane first settles each facet's case (cardinal, diagonal, inside) from the falls,
// which are dense FP64 subtractions and integer comparisons; the warp then takes the diagonal
// divisions and the inside square roots as two compacted lists, every lane one request; then each
// lane compares its facets' slopes in the reference's order. The early outs of the per-lane form only
// skipped slopes that could not win, so computing every slope changes no comparison's outcome.
struct DenseFacets {
    double sq[32 * 8];    // per lane and facet: an inside facet's squared slope, then its slope
    double dv[32 * 4];    // per lane and diagonal: the fall, then the slope
    int idx[32 * 8];      // the compacted requests
};

__device__ __forceinline__ int warp_exclusive_sum(int v, int lane, int* total) {
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= o) x += y;
    }
    *total = __shfl_sync(0xFFFFFFFFu, x, 31);
    return x - v;
}

__device__ int facet_receiver_dense(int W, int H, const double* __restrict__ rs, int cell, Steps st, long long seed,
                                    DenseFacets& sh) {
    const int lane = threadIdx.x & 31;
    const int ccs_t[4] = {1, 0, -1, 0};
    const int crs_t[4] = {0, -1, 0, 1};
    const bool live = cell >= 0;
    const int row = live ? pdiv(cell, W) : 0, col = live ? pmod(cell, W) : 0;
    const double here = live ? rs[cell] : 0.0;
    const double dg = (double)st.diag;
    int dcell[4];
    double dfall[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int dcs = (k & 1) ? 1 : -1, drs = (k & 2) ? 1 : -1;
        dcell[k] = live ? neighbour_at(W, H, col + dcs, row + drs) : -1;
        dfall[k] = dcell[k] >= 0 ? __dsub_rn(here, rs[dcell[k]]) : 0.0;
    }
    int card[4];
    double cdrop[4];
    unsigned modes = 0;     // 2 bits per facet: 0 cardinal, 1 diagonal, 2 inside, 3 none
    unsigned need_div = 0, need_sq = 0;
#pragma unroll
    for (int side = 0; side < 4; ++side) {
        card[side] = live ? neighbour_at(W, H, col + ccs_t[side], row + crs_t[side]) : -1;
        cdrop[side] = card[side] >= 0 ? __dsub_rn(here, rs[card[side]]) : 0.0;
        const bool cdown = dpos(cdrop[side]);
#pragma unroll
        for (int t = 0; t < 2; ++t) {
            const int turn = t ? 1 : -1, f = side * 2 + t;
            const int dcs = ccs_t[side] == 0 ? turn : ccs_t[side];
            const int drs = crs_t[side] == 0 ? turn : crs_t[side];
            const int k = (dcs > 0 ? 1 : 0) | (drs > 0 ? 2 : 0);
            unsigned m = 3;
            if (card[side] >= 0 && dcell[k] >= 0) {
                const double outward = __dsub_rn(dfall[k], cdrop[side]);
                if (cdown && !dpos(outward)) {
                    m = 0;
                } else if (!cdown || dkey(outward) >= dkey(cdrop[side])) {   // a >= b, with unit legs
                    m = 1;
                    need_div |= 1u << k;
                } else {
                    m = 2;
                    need_sq |= 1u << f;
                    sh.sq[lane * 8 + f] = __dadd_rn(__dmul_rn(cdrop[side], cdrop[side]), __dmul_rn(outward, outward));
                }
            }
            modes |= m << (2 * f);
        }
    }
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (need_div & (1u << k)) sh.dv[lane * 4 + k] = dfall[k];
    // The diagonal divisions, densely.
    int total;
    int off = warp_exclusive_sum(__popc(need_div), lane, &total);
    for (int k = 0, j = 0; k < 4; ++k)
        if (need_div & (1u << k)) sh.idx[off + j++] = lane * 4 + k;
    __syncwarp();
    for (int base = 0; base < total; base += 32)
        if (base + lane < total) {
            const int i = sh.idx[base + lane];
            sh.dv[i] = __ddiv_rn(sh.dv[i], dg);
        }
    __syncwarp();
    // The inside facets' square roots, densely.
    off = warp_exclusive_sum(__popc(need_sq), lane, &total);
    for (int f = 0, j = 0; f < 8; ++f)
        if (need_sq & (1u << f)) sh.idx[off + j++] = lane * 8 + f;
    __syncwarp();
    for (int base = 0; base < total; base += 32)
        if (base + lane < total) {
            const int i = sh.idx[base + lane];
            sh.sq[i] = __dsqrt_rn(sh.sq[i]);
        }
    __syncwarp();
    // The facets in the reference's order; the winner's cells and falls kept as it wins.
    double steepest = 0.0;
    unsigned wmode = 3;
    int fcard = -1, fdiag = -1;
    double wout = 0.0, wdrop = 0.0;
#pragma unroll
    for (int f = 0; f < 8; ++f) {
        const unsigned m = (modes >> (2 * f)) & 3u;
        const int side = f >> 1, turn = (f & 1) ? 1 : -1;
        const int dcs = ccs_t[side] == 0 ? turn : ccs_t[side];
        const int drs = crs_t[side] == 0 ? turn : crs_t[side];
        const int k = (dcs > 0 ? 1 : 0) | (drs > 0 ? 2 : 0);
        if (m == 3) continue;
        const double v = m == 0 ? cdrop[side] : m == 1 ? sh.dv[lane * 4 + k] : sh.sq[lane * 8 + f];
        if (dkey(v) > dkey(steepest)) {
            steepest = v;
            wmode = m;
            fcard = card[side];
            fdiag = dcell[k];
            wout = dfall[k];
            wdrop = cdrop[side];
        }
    }
    __syncwarp();   // the buffers are the warp's next call's
    if (!live || wmode == 3 || !dpos(steepest)) return -1;
    if (wmode == 0) return fcard;
    if (wmode == 1) return fdiag;
    const double share = __ddiv_rn(__dsub_rn(wout, wdrop), wdrop);
    if (!dpos(share)) return fcard;
    // FlowRouting.subGridDraw (FlowRouting.kt:355-356).
    const double draw = (double)__fmul_rn(__fadd_rn(seeded_noise(col, row, seed ^ kSubGridDrawSalt), 1.0f), 0.5f);
    return dkey(draw) < dkey(share) ? fdiag : fcard;
}

// FlowRouting.steepestNeighbourOf (FlowRouting.kt:320-343).
__device__ int steepest_neighbour(int W, int H, const double* __restrict__ rs, int col, int row, Steps st) {
    int best = -1;
    double sd = 0.0;
    double here = rs[row * W + col];
    for (int r = -1; r <= 1; ++r) {
        int nr = row + r;
        if (nr < 0 || nr >= H) continue;
        for (int c = -1; c <= 1; ++c) {
            if (r == 0 && c == 0) continue;
            int n = nr * W + wrap_col(col + c, W);
            double drop = __ddiv_rn(__dsub_rn(here, rs[n]), (double)st.of(c, r));
            if (drop > sd) {
                sd = drop;
                best = n;
            }
        }
    }
    return best;
}

// Receivers of land cells (sea cells get -1). The facet rule is FP64 work, and an FP64 warp
// instruction costs the same with one lane active as with 32, so each warp compacts the land cells
// of the chunks it scans into a small queue in shared memory and runs the rule 32 land cells at a
// time. `near` splits the work around the flats: 0 every land cell; 1 the cells with no raised cell
// in their 3x3 block (their surface and their neighbours' are final before the flats are solved,
// so this pass runs beside the flat solvers) and the sea; 2 the cells with a raised cell in their
// 3x3 block, after the flats.
constexpr int RECV_THREADS = 256;

__device__ __forceinline__ int receiver_of(int cell, const double* __restrict__ surface, int W, int H, Steps st,
                                           long long seed, int by_facet, bool unit) {
    const int row = pdiv(cell, W), col = pmod(cell, W);
    return !by_facet ? steepest_neighbour(W, H, surface, col, row, st)
           : unit    ? facet_receiver<true>(W, H, surface, col, row, st, seed)
                     : facet_receiver<false>(W, H, surface, col, row, st, seed);
}

__device__ __forceinline__ bool near_raised(const uint8_t* __restrict__ raised, int cell, int W, int H) {
    const int row = pdiv(cell, W), col = pmod(cell, W);
    unsigned any = 0;
#pragma unroll
    for (int rs = -1; rs <= 1; ++rs) {
        const int nr = row + rs;
        if (nr < 0 || nr >= H) continue;
#pragma unroll
        for (int cs = -1; cs <= 1; ++cs) any |= raised[nr * W + wrap_col(col + cs, W)];
    }
    return any != 0;
}

__global__ void __launch_bounds__(RECV_THREADS) k_receivers(const uint8_t* __restrict__ land,
                                                            const double* __restrict__ surface, int W, int H,
                                                            Steps st, long long seed, int by_facet,
                                                            const uint8_t* __restrict__ raised, int near,
                                                            int32_t* __restrict__ recv) {
    const unsigned FULL = 0xFFFFFFFFu;
    __shared__ int queue[RECV_THREADS / 32][64];
    __shared__ DenseFacets dense[RECV_THREADS / 32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int* q = queue[warp];
    const bool unit = st.ew == 1.0f && st.ns == 1.0f;
    const bool warp_dense = by_facet && unit;   // square cells: the facet rule with dense FP64 requests
    const size_t N = (size_t)W * H;
    const size_t warps = (size_t)gridDim.x * (RECV_THREADS / 32);
    int n = 0;   // queued land cells (the same in every lane)
    for (size_t base = ((size_t)blockIdx.x * (RECV_THREADS / 32) + warp) * 32; base < N; base += warps * 32) {
        const size_t i = base + lane;
        const bool is_land = i < N && land[i];
        if (i < N && !is_land && near != 2) recv[i] = -1;
        const bool l = is_land && (near == 0 || near_raised(raised, (int)i, W, H) == (near == 2));
        const unsigned m = __ballot_sync(FULL, l);
        if (l) q[n + __popc(m & ((1u << lane) - 1u))] = (int)i;
        n += __popc(m);
        __syncwarp();
        if (n >= 32) {
            const int cell = q[lane];
            recv[cell] = warp_dense ? facet_receiver_dense(W, H, surface, cell, st, seed, dense[warp])
                                    : receiver_of(cell, surface, W, H, st, seed, by_facet, unit);
            __syncwarp();
            if (lane < n - 32) q[lane] = q[32 + lane];
            n -= 32;
            __syncwarp();
        }
    }
    if (warp_dense) {
        const int cell = lane < n ? q[lane] : -1;
        const int r = facet_receiver_dense(W, H, surface, cell, st, seed, dense[warp]);
        if (lane < n) recv[cell] = r;
    } else if (lane < n) {
        const int cell = q[lane];
        recv[cell] = receiver_of(cell, surface, W, H, st, seed, by_facet, unit);
    }
}

__global__ void k_surface(const uint8_t* __restrict__ land, const float* __restrict__ rel,
                          const float* __restrict__ filled, size_t N, double* __restrict__ surface,
                          uint8_t* __restrict__ raised, int* __restrict__ local) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x) {
        bool l = land[i] != 0;
        surface[i] = (double)(l ? filled[i] : rel[i]);
        if (raised) raised[i] = l && filled[i] > rel[i];
        if (local) local[i] = -1;
    }
}

__global__ void k_flat_count(const int* __restrict__ label, size_t N, int* __restrict__ count) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x)
        if (label[i] >= 0) atomicAdd(&count[label[i]], 1);
}

__global__ void k_flat_scatter(const int* __restrict__ label, size_t N, const int* __restrict__ off,
                               int* __restrict__ cursor, int* __restrict__ members) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x) {
        int l = label[i];
        if (l >= 0) members[off[l] + atomicAdd(&cursor[l], 1)] = (int)i;
    }
}

constexpr int FT = 512;   // threads per flat CTA

struct FlatArgs {
    int W, H, lattice;
    long long seed;
    double ew, ns, diag;   // FlatRouting.stencil
    const int* off;
    const int* count;
    int* members;
    int* local;
    const float* filled;
    double* surface;
    double* degree;
    double* pivot;
    double* x;
    double* r;
    double* z;
    double* d;
    double* ad;
    double* coef;   // ns / pivot per member
    short* nbr;     // per member, the member index of its 8 neighbours in stencil order (-1: none)
    const int* large;   // the flats that k_flat_solve takes
    int* kept;
};

template <class T, class Op>
__device__ T block_reduce(T v, T* sh, Op op, T identity) {
    for (int o = 16; o > 0; o >>= 1) v = op(v, __shfl_xor_sync(0xFFFFFFFFu, v, o));
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    if (warp == 0) {
        v = lane < (int)(blockDim.x >> 5) ? sh[lane] : identity;
        for (int o = 16; o > 0; o >>= 1) v = op(v, __shfl_xor_sync(0xFFFFFFFFu, v, o));
        if (lane == 0) sh[0] = v;
    }
    __syncthreads();
    T out = sh[0];
    __syncthreads();
    return out;
}

struct DAdd {
    __device__ double operator()(double a, double b) const { return __dadd_rn(a, b); }
};
struct DMax {
    __device__ double operator()(double a, double b) const { return a > b ? a : b; }
};
struct FMin {
    __device__ float operator()(float a, float b) const { return a < b ? a : b; }
};
struct IAnd {
    __device__ int operator()(int a, int b) const { return a & b; }
};

// In-CTA sort of the flat's member list, ascending cell index, in place over exactly n entries.
// The bitonic network in its all-ascending form: each merge of 2k-blocks first compares i with its
// mirror i ^ (k-1), then half-cleans with i ^ j. Every comparator puts the smaller key at the lower
// index, so a partner at or past n (an implicit +infinity) never has to move and is skipped.
__device__ void sort_members(int* m, int n) {
    int P2 = 1;
    while (P2 < n) P2 <<= 1;
    for (int k = 2; k <= P2; k <<= 1) {
        for (int j = k - 1; j > 0; j = (j == k - 1) ? (k >> 2) : (j >> 1)) {
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                int l = i ^ j;
                if (l > i && l < n) {
                    int a = m[i], b = m[l];
                    if (a > b) {
                        m[i] = b;
                        m[l] = a;
                    }
                }
            }
            __syncthreads();
            if (k == 2) break;
        }
    }
}

// x / p for a pivot p > 0 whose reciprocal r = 1 / p (correctly rounded) is kept: q0 = x r and one
// correction with fused multiply-adds, q = q0 + (x - q0 p) r. With a correctly rounded reciprocal
// this is the correctly rounded quotient (Markstein's theorem, barring overflow and underflow), so
// the bits of x / p, in three dependent operations instead of a division's sequence; the column
// runs' solves are chains of such divisions, so their latency is the CG iteration's.
__device__ __forceinline__ double div_by(double x, double p, double r) {
    const double q0 = __dmul_rn(x, r);
    return __fma_rn(__fma_rn(-q0, p, x), r, q0);
}

__device__ __forceinline__ double stencil_weight(const FlatArgs& a, int cs, int rs) {
    return (cs != 0 && rs != 0) ? a.diag : (rs != 0 ? a.ns : a.ew);
}

// Column-run preconditioner solve (FlatRouting.ColumnRuns.solve, FlatRouting.kt:399-413). Members
// are ordered by (column, row), so every run is a contiguous segment, walked by one thread down the
// column and back up with the chain carried in registers; the expressions are the reference's
// ((right + ns * above) / pivot down, += (ns / pivot) * below up, ns / pivot kept per member).
__device__ __forceinline__ bool run_continues(const int* mem, int n, int k, int W, int H) {
    return k + 1 < n && mem[k + 1] == mem[k] + W && pdiv(mem[k], W) + 1 < H;
}
__device__ __forceinline__ bool run_head(const int* mem, int k, int W) { return k == 0 || mem[k - 1] != mem[k] - W; }

__device__ void runs_solve(const FlatArgs& a, int base, int n, const double* right, double* into) {
    const int* mem = a.members + base;
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        if (!run_head(mem, k, a.W)) continue;
        int j = k;
        double v = __ddiv_rn(__dadd_rn(right[base + j], 0.0), a.pivot[base + j]);   // carried = 0.0 at a head
        into[base + j] = v;
        while (run_continues(mem, n, j, a.W, a.H)) {
            ++j;
            v = __ddiv_rn(__dadd_rn(right[base + j], __dmul_rn(a.ns, v)), a.pivot[base + j]);
            into[base + j] = v;
        }
        // Back up the run from its last member j.
        double below = v;
        for (int i = j - 1; i >= k; --i) {
            double u = __dadd_rn(into[base + i], __dmul_rn(a.coef[base + i], below));
            into[base + i] = u;
            below = u;
        }
    }
}

// Laplacian row (FlatRouting.kt:274-282): degree * x minus the member neighbours in stencil order.
__device__ void apply_laplacian(const FlatArgs& a, int base, int n, const double* xv, double* into) {
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        int cell = a.members[base + k];
        int col = pmod(cell, a.W), row = pdiv(cell, a.W);
        double sum = __dmul_rn(a.degree[base + k], xv[base + k]);
        for (int rs = -1; rs <= 1; ++rs) {
            int nr = row + rs;
            if (nr < 0 || nr >= a.H) continue;
            for (int cs = -1; cs <= 1; ++cs) {
                if (cs == 0 && rs == 0) continue;
                int nb = nr * a.W + wrap_col(col + cs, a.W);
                int l = a.local[nb];
                if (l >= 0) sum = __dsub_rn(sum, __dmul_rn(stencil_weight(a, cs, rs), xv[base + l]));
            }
        }
        into[base + k] = sum;
    }
}

// FlatRouting.layInBand (FlatRouting.kt:455-489) over one flat, by the whole CTA: the potential x,
// scaled into the band between the highest entry and the entry level, is kept only if every member
// then has a lower neighbour; otherwise the flat keeps its filled level and counts as kept.
__device__ void lay_in_band(const FlatArgs& a, const int* mem, int n, const double* x, bool positive, double highest,
                            double entry_level, double entry_height, int* shi) {
    bool laid = positive && !(highest <= 0.0 || entry_height >= entry_level);
    if (laid) {
        const double band = __dmul_rn(__dsub_rn(entry_level, entry_height), 0.9);
        for (int k = threadIdx.x; k < n; k += blockDim.x)
            a.surface[mem[k]] = __dadd_rn(entry_height, __dmul_rn(band, __ddiv_rn(x[k], highest)));
        __syncthreads();
        int ok = 1;
        for (int k = threadIdx.x; k < n; k += blockDim.x) {
            int cell = mem[k];
            int col = pmod(cell, a.W), row = pdiv(cell, a.W);
            double here = a.surface[cell];
            bool lower = false;
            for (int rs = -1; rs <= 1 && !lower; ++rs) {
                int nr = row + rs;
                if (nr < 0 || nr >= a.H) continue;
                for (int cs = -1; cs <= 1; ++cs) {
                    if (cs == 0 && rs == 0) continue;
                    if (a.surface[nr * a.W + wrap_col(col + cs, a.W)] < here) {
                        lower = true;
                        break;
                    }
                }
            }
            if (!lower) ok = 0;
        }
        ok = block_reduce(ok, shi, IAnd(), 1);
        if (!ok) {
            for (int k = threadIdx.x; k < n; k += blockDim.x) a.surface[mem[k]] = (double)a.filled[mem[k]];
            laid = false;
        }
    }
    if (!laid && threadIdx.x == 0) atomicAdd(a.kept, 1);
}

__global__ void __launch_bounds__(FT) k_flat_solve(FlatArgs a) {
    __shared__ double shd[32];
    __shared__ float shf[32];
    __shared__ int shi[32];
    const int f = a.large[blockIdx.x];
    const int base = a.off[f];
    const int n = a.count[f];
    int* mem = a.members + base;
    // Order the members by (column, row): every column run becomes a contiguous segment. The order
    // is fixed, so the block reductions below are deterministic.
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        int c = mem[k];
        mem[k] = pmod(c, a.W) * a.H + pdiv(c, a.W);
    }
    __syncthreads();
    sort_members(mem, n);
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        int key = mem[k];
        mem[k] = pmod(key, a.H) * a.W + pdiv(key, a.H);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < n; k += blockDim.x) a.local[mem[k]] = k;
    __syncthreads();

    // The entry level and the highest entry (FlatRouting.kt:93-115, 427-445).
    float lo = FLT_MAX;
    for (int k = threadIdx.x; k < n; k += blockDim.x) lo = fminf(lo, a.filled[mem[k]]);
    const float lowest = block_reduce(lo, shf, FMin(), FLT_MAX);
    const double entry_level = (double)lowest;
    double hi = -INFINITY;
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        int cell = mem[k];
        int col = pmod(cell, a.W), row = pdiv(cell, a.W);
        for (int rs = -1; rs <= 1; ++rs) {
            int nr = row + rs;
            if (nr < 0 || nr >= a.H) continue;
            for (int cs = -1; cs <= 1; ++cs) {
                if (cs == 0 && rs == 0) continue;
                int nb = nr * a.W + wrap_col(col + cs, a.W);
                double there = a.surface[nb];
                if (a.local[nb] < 0 && there < entry_level && there > hi) hi = there;
            }
        }
    }
    const double entry_height = block_reduce(hi, shd, DMax(), (double)-INFINITY);

    // Degrees (FlatRouting.kt:239-271) and the rain (:289-295).
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        int cell = mem[k];
        int col = pmod(cell, a.W), row = pdiv(cell, a.W);
        double total = 0.0;
        for (int rs = -1; rs <= 1; ++rs) {
            int nr = row + rs;
            if (nr < 0 || nr >= a.H) continue;
            for (int cs = -1; cs <= 1; ++cs) {
                if (cs == 0 && rs == 0) continue;
                int nb = nr * a.W + wrap_col(col + cs, a.W);
                double w = stencil_weight(a, cs, rs);
                if (a.local[nb] >= 0) total = __dadd_rn(total, w);
                else if (a.surface[nb] < entry_level) total = __dadd_rn(total, w);
            }
        }
        a.degree[base + k] = total;
        a.x[base + k] = 0.0;
        a.r[base + k] = __dadd_rn(1.0, __dmul_rn(0.5, (double)smooth_seeded_field(a.W, a.lattice, col, row,
                                                                                    a.seed ^ kRainReliefSalt)));
    }
    __syncthreads();
    // Thomas pivots per run (FlatRouting.kt:388-395), and ns / pivot for the solves' way back up.
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        if (!run_head(mem, k, a.W)) continue;
        int j = k;
        double p = a.degree[base + j];
        while (true) {
            a.pivot[base + j] = p;
            a.coef[base + j] = __ddiv_rn(a.ns, p);
            if (!run_continues(mem, n, j, a.W, a.H)) break;
            ++j;
            p = __dsub_rn(a.degree[base + j], __ddiv_rn(__dmul_rn(a.ns, a.ns), p));
        }
    }
    __syncthreads();

    // Preconditioned conjugate gradients (FlatRouting.kt:296-333).
    runs_solve(a, base, n, a.r, a.z);
    __syncthreads();
    double rn = 0.0, ra = 0.0;
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        double rv = a.r[base + k], zv = a.z[base + k];
        a.d[base + k] = zv;
        rn = __dadd_rn(rn, __dmul_rn(rv, rv));
        ra = __dadd_rn(ra, __dmul_rn(rv, zv));
    }
    double rnorm = block_reduce(rn, shd, DAdd(), 0.0);
    double rap = block_reduce(ra, shd, DAdd(), 0.0);
    const double stop_at = __dmul_rn(__dmul_rn(rnorm, 1e-7), 1e-7);
    const int most = 64 + (int)(8.0 * sqrt((double)n));
    for (int it = 0; rnorm > stop_at && it < most; ++it) {
        apply_laplacian(a, base, n, a.d, a.ad);
        __syncthreads();
        double e = 0.0;
        for (int k = threadIdx.x; k < n; k += blockDim.x) e = __dadd_rn(e, __dmul_rn(a.d[base + k], a.ad[base + k]));
        double energy = block_reduce(e, shd, DAdd(), 0.0);
        if (energy <= 0.0 || rap <= 0.0) break;
        double step = __ddiv_rn(rap, energy);
        double nn = 0.0;
        for (int k = threadIdx.x; k < n; k += blockDim.x) {
            a.x[base + k] = __dadd_rn(a.x[base + k], __dmul_rn(step, a.d[base + k]));
            double rv = __dsub_rn(a.r[base + k], __dmul_rn(step, a.ad[base + k]));
            a.r[base + k] = rv;
            nn = __dadd_rn(nn, __dmul_rn(rv, rv));
        }
        double next_norm = block_reduce(nn, shd, DAdd(), 0.0);
        runs_solve(a, base, n, a.r, a.z);
        __syncthreads();
        double na = 0.0;
        for (int k = threadIdx.x; k < n; k += blockDim.x) na = __dadd_rn(na, __dmul_rn(a.r[base + k], a.z[base + k]));
        double next_ap = block_reduce(na, shd, DAdd(), 0.0);
        double improvement = __ddiv_rn(next_ap, rap);
        for (int k = threadIdx.x; k < n; k += blockDim.x)
            a.d[base + k] = __dadd_rn(a.z[base + k], __dmul_rn(improvement, a.d[base + k]));
        __syncthreads();
        rnorm = next_norm;
        rap = next_ap;
    }
    int positive = 1;
    double top = 0.0;
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        double v = a.x[base + k];
        if (!(v > 0.0)) positive = 0;
        if (v > top) top = v;
    }
    positive = block_reduce(positive, shi, IAnd(), 1);
    const double highest = block_reduce(top, shd, DMax(), 0.0);

    lay_in_band(a, mem, n, a.x + base, positive, highest, entry_level, entry_height, shi);
}

// Flats of 33 to 512 members, one CTA each, with the CG's working vectors in shared memory.
// A CG iteration is latency-bound: the column runs' Thomas solves are chains of dependent
// divisions, one run per thread, and a valley floor can hold runs hundreds of cells long, so a
// chain that goes through L2 at every step costs most of the iteration. Here r, z, d, A d, the
// pivots, ns / pivot and the run table sit in shared memory; the per-member constants (degree, the
// member neighbours) and the potential x, which a thread reads only for its own members, stay in
// global memory. The arithmetic per member and per run is that of k_flat_solve. A dot product is
// each thread's partial sum in member order, then block_reduce2's fixed order, so its bits are fixed
// for a given CTA size.
constexpr int MID_FLAT = 512;    // members at most for the 128-thread CTA
constexpr int SM_BYTES_PER_MEMBER = 7 * 8 + 4;   // seven doubles and one run-table entry

struct Sum2 {
    __device__ double2 operator()(double2 a, double2 b) const { return make_double2(__dadd_rn(a.x, b.x), __dadd_rn(a.y, b.y)); }
};
struct MinMax2 {
    __device__ double2 operator()(double2 a, double2 b) const {
        return make_double2(a.x < b.x ? a.x : b.x, a.y > b.y ? a.y : b.y);
    }
};

// The CTA's combination of v (two values), returned to every thread. Every thread's partial goes to
// shared memory; the first warp folds the FT / 32 partials of each lane in thread order, then a
// butterfly over its lanes, and hands the result out. The FP64 pipe is the scarce resource: this
// takes FT / 32 - 1 + 5 FP64 operations of one warp per value, where a butterfly in every warp
// takes 5 in each. `buf` holds FT double2 and `out` one; the two barriers keep consecutive calls
// apart.
template <int FT, class Op>
__device__ __forceinline__ double2 block_reduce2(double2 v, Op op, double2* buf, double2* out) {
    buf[threadIdx.x] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        double2 s = buf[threadIdx.x];
#pragma unroll
        for (int k = 1; k < FT / 32; ++k) s = op(s, buf[threadIdx.x + 32 * k]);
        for (int o = 16; o > 0; o >>= 1) {
            double2 t;
            t.x = __shfl_xor_sync(0xFFFFFFFFu, s.x, o);
            t.y = __shfl_xor_sync(0xFFFFFFFFu, s.y, o);
            s = op(s, t);
        }
        if (threadIdx.x == 0) *out = s;
    }
    __syncthreads();
    return *out;
}

__device__ __forceinline__ int nbr_lo(int v) { return (int)(short)(v & 0xFFFF); }
__device__ __forceinline__ int nbr_hi(int v) { return v >> 16; }
__device__ __forceinline__ int nbr_pack(int lo, int hi) { return (int)(((unsigned)lo & 0xFFFFu) | ((unsigned)hi << 16)); }

template <int FT>
__global__ void __launch_bounds__(FT) k_flat_solve_sm(FlatArgs a, const int* __restrict__ list) {
    extern __shared__ double dyn[];
    __shared__ double shd[32];
    __shared__ float shf[32];
    __shared__ int shi[32];
    __shared__ double2 red[FT];
    __shared__ double2 red_out;
    __shared__ int s_nruns;
    const int f = list[blockIdx.x];
    const int base = a.off[f];
    const int n = a.count[f];
    const int W = a.W, H = a.H;
    int* mem = a.members + base;
    double* s_r = dyn;
    double* s_z = s_r + n;
    double* s_d = s_z + n;
    double* s_ad = s_d + n;
    double* s_piv = s_ad + n;
    double* s_coef = s_piv + n;
    double* s_rcp = s_coef + n;   // 1 / pivot
    unsigned* s_run = reinterpret_cast<unsigned*>(s_rcp + n);   // first | last << 16
    double* x = a.x + base;
    double* degree = a.degree + base;
    int4* nbr = reinterpret_cast<int4*>(a.nbr + (size_t)base * 8);

    // Members by (column, row), as in k_flat_solve.
    for (int k = threadIdx.x; k < n; k += FT) {
        int c = mem[k];
        mem[k] = pmod(c, W) * H + pdiv(c, W);
    }
    __syncthreads();
    sort_members(mem, n);
    for (int k = threadIdx.x; k < n; k += FT) {
        int key = mem[k];
        mem[k] = pmod(key, H) * W + pdiv(key, H);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < n; k += FT) a.local[mem[k]] = k;
    if (threadIdx.x == 0) s_nruns = 0;
    __syncthreads();

    // Entry level; then per member the highest entry, the degree, the member neighbours and the rain
    // (FlatRouting.kt:93-115, 239-295, 427-445).
    float lo = FLT_MAX;
    for (int k = threadIdx.x; k < n; k += FT) lo = fminf(lo, a.filled[mem[k]]);
    const double entry_level = (double)block_reduce(lo, shf, FMin(), FLT_MAX);
    double hi = -INFINITY;
    for (int k = threadIdx.x; k < n; k += FT) {
        const int cell = mem[k];
        const int col = pmod(cell, W), row = pdiv(cell, W);
        double total = 0.0;
        int nb8[8];
        int t = 0;
        for (int rs = -1; rs <= 1; ++rs) {
            const int nr = row + rs;
            for (int cs = -1; cs <= 1; ++cs) {
                if (cs == 0 && rs == 0) continue;
                nb8[t] = -1;
                if (nr >= 0 && nr < H) {
                    const int nb = nr * W + wrap_col(col + cs, W);
                    const double w = stencil_weight(a, cs, rs);
                    const int l = a.local[nb];
                    if (l >= 0) {
                        total = __dadd_rn(total, w);
                        nb8[t] = l;
                    } else {
                        const double there = a.surface[nb];
                        if (there < entry_level) {
                            total = __dadd_rn(total, w);
                            if (there > hi) hi = there;
                        }
                    }
                }
                ++t;
            }
        }
        degree[k] = total;
        x[k] = 0.0;
        nbr[k] = make_int4(nbr_pack(nb8[0], nb8[1]), nbr_pack(nb8[2], nb8[3]), nbr_pack(nb8[4], nb8[5]),
                           nbr_pack(nb8[6], nb8[7]));
        s_r[k] = __dadd_rn(1.0, __dmul_rn(0.5, (double)smooth_seeded_field(W, a.lattice, col, row,
                                                                             a.seed ^ kRainReliefSalt)));
        if (run_head(mem, k, W)) {
            int j = k;
            while (run_continues(mem, n, j, W, H)) ++j;
            s_run[atomicAdd(&s_nruns, 1)] = (unsigned)k | ((unsigned)j << 16);
        }
    }
    const double entry_height = block_reduce(hi, shd, DMax(), (double)-INFINITY);
    const int runs = s_nruns;

    // Thomas pivots down each run (FlatRouting.kt:388-395) and ns / pivot for the way back up.
    for (int i = threadIdx.x; i < runs; i += FT) {
        const int first = (int)(s_run[i] & 0xFFFFu), last = (int)(s_run[i] >> 16);
        double p = degree[first];
        for (int j = first;; ++j) {
            s_piv[j] = p;
            s_coef[j] = __ddiv_rn(a.ns, p);
            s_rcp[j] = __ddiv_rn(1.0, p);
            if (j == last) break;
            p = __dsub_rn(degree[j + 1], __ddiv_rn(__dmul_rn(a.ns, a.ns), p));
        }
    }
    __syncthreads();

    // z = M^-1 r through the runs (FlatRouting.ColumnRuns.solve, FlatRouting.kt:399-413).
    auto precondition = [&]() {
        for (int i = threadIdx.x; i < runs; i += FT) {
            const int first = (int)(s_run[i] & 0xFFFFu), last = (int)(s_run[i] >> 16);
            double v = div_by(__dadd_rn(s_r[first], 0.0), s_piv[first], s_rcp[first]);
            s_z[first] = v;
            for (int j = first + 1; j <= last; ++j) {
                v = div_by(__dadd_rn(s_r[j], __dmul_rn(a.ns, v)), s_piv[j], s_rcp[j]);
                s_z[j] = v;
            }
            double below = v;
            for (int j = last - 1; j >= first; --j) {
                below = __dadd_rn(s_z[j], __dmul_rn(s_coef[j], below));
                s_z[j] = below;
            }
        }
    };
    const double w8[8] = {a.diag, a.ns, a.diag, a.ew, a.ew, a.diag, a.ns, a.diag};   // stencil order

    // Preconditioned conjugate gradients (FlatRouting.kt:296-333).
    precondition();
    __syncthreads();
    double rn = 0.0, ra = 0.0;
    for (int k = threadIdx.x; k < n; k += FT) {
        const double rv = s_r[k], zv = s_z[k];
        s_d[k] = zv;
        rn = __dadd_rn(rn, __dmul_rn(rv, rv));
        ra = __dadd_rn(ra, __dmul_rn(rv, zv));
    }
    double2 sums = block_reduce2<FT>(make_double2(rn, ra), Sum2(), red, &red_out);
    double rnorm = sums.x, rap = sums.y;
    const double stop_at = __dmul_rn(__dmul_rn(rnorm, 1e-7), 1e-7);
    const int most = 64 + (int)(8.0 * sqrt((double)n));
    for (int it = 0; rnorm > stop_at && it < most; ++it) {
        // A d (FlatRouting.kt:274-282) and d . A d.
        double e = 0.0;
        for (int k = threadIdx.x; k < n; k += FT) {
            const int4 q = nbr[k];
            const int l8[8] = {nbr_lo(q.x), nbr_hi(q.x), nbr_lo(q.y), nbr_hi(q.y),
                               nbr_lo(q.z), nbr_hi(q.z), nbr_lo(q.w), nbr_hi(q.w)};
            const double dk = s_d[k];
            double sum = __dmul_rn(degree[k], dk);
#pragma unroll
            for (int t = 0; t < 8; ++t)
                if (l8[t] >= 0) sum = __dsub_rn(sum, __dmul_rn(w8[t], s_d[l8[t]]));
            s_ad[k] = sum;
            e = __dadd_rn(e, __dmul_rn(dk, sum));
        }
        const double energy = block_reduce2<FT>(make_double2(e, 0.0), Sum2(), red, &red_out).x;
        if (energy <= 0.0 || rap <= 0.0) break;
        const double step = __ddiv_rn(rap, energy);
        for (int k = threadIdx.x; k < n; k += FT) {
            x[k] = __dadd_rn(x[k], __dmul_rn(step, s_d[k]));
            s_r[k] = __dsub_rn(s_r[k], __dmul_rn(step, s_ad[k]));
        }
        __syncthreads();
        precondition();
        __syncthreads();
        double nn = 0.0, na = 0.0;
        for (int k = threadIdx.x; k < n; k += FT) {
            const double rv = s_r[k];
            nn = __dadd_rn(nn, __dmul_rn(rv, rv));
            na = __dadd_rn(na, __dmul_rn(rv, s_z[k]));
        }
        sums = block_reduce2<FT>(make_double2(nn, na), Sum2(), red, &red_out);
        const double improvement = __ddiv_rn(sums.y, rap);
        for (int k = threadIdx.x; k < n; k += FT) s_d[k] = __dadd_rn(s_z[k], __dmul_rn(improvement, s_d[k]));
        __syncthreads();
        rnorm = sums.x;
        rap = sums.y;
    }
    int positive = 1;
    double top = 0.0;
    for (int k = threadIdx.x; k < n; k += FT) {
        const double v = x[k];
        if (!(v > 0.0)) positive = 0;
        if (v > top) top = v;
    }
    positive = block_reduce(positive, shi, IAnd(), 1);
    const double highest = block_reduce(top, shd, DMax(), 0.0);
    lay_in_band(a, mem, n, x, positive, highest, entry_level, entry_height, shi);
}

// Flats of 513 to CL_FLAT members, one thread-block cluster of CL CTAs each. On GB300 a CG
// iteration of a large flat is bound by one SM's FP64 pipe, so the flat's members are split over
// the cluster's SMs: CTA q owns the members [bound[q], bound[q + 1]), bounds placed at column-run
// heads so that every Thomas chain stays in one CTA. Each CTA keeps its members' vectors in its own
// shared memory; the Laplacian reads a neighbour owned by another CTA from that CTA's shared memory
// (distributed shared memory), and every dot product is a CTA partial (as in k_flat_solve_sm) sent
// to all CTAs of the cluster and summed there in rank order, so each CTA holds the same bits. A flat
// whose ranges do not fit the shared memory this launch was given (a column run longer than the
// slack) is handed to k_flat_solve, through its list.
constexpr int CL = 8;                          // CTAs per cluster
constexpr int CL_THREADS = 256;
constexpr int CL_FLAT = 16384;                 // members at most for the cluster kernel
constexpr int CL_RANGE_MAX = 8191;             // members per CTA: the neighbour code keeps 13 bits of offset
constexpr int CL_SMEM_MEMBERS = (227 * 1024 - 8192) / SM_BYTES_PER_MEMBER;   // members per CTA that fit beside the static arrays

namespace cgc = cooperative_groups;


// The CTA's combination of (u, v) (block_reduce2), sent to slot q of every CTA's `slots[par]`; after
// the cluster barrier each CTA's first warp combines the CL slots in rank order and hands the result
// to the CTA through shared memory (the FP64 pipe is the scarce resource: the other warps need not
// repeat it). `par` alternates between calls: the next call's barrier keeps this call's readers
// ahead of the call after it.
template <class Op>
__device__ double2 cluster_combine(double2 v, Op op, double2* warps, double2 (*slots)[CL], double2* result, int& par,
                                   int q) {
    const double2 cta = block_reduce2<CL_THREADS>(v, op, warps, result + 2);
    if (threadIdx.x < CL) {
        double2* dst = cgc::this_cluster().map_shared_rank(&slots[par][q], (int)threadIdx.x);
        *dst = cta;
    }
    cgc::this_cluster().sync();
    if (threadIdx.x < 32) {
        double2 s = slots[par][0];
#pragma unroll
        for (int r = 1; r < CL; ++r) s = op(s, slots[par][r]);
        if (threadIdx.x == 0) result[par] = s;
    }
    __syncthreads();
    const double2 s = result[par];
    par ^= 1;
    return s;
}

// A member neighbour as owner rank (3 bits) and offset in the owner's range (13 bits); 0xFFFF is
// none (an offset is at most CL_RANGE_MAX - 1, so rank 7 never packs to it).
constexpr int CL_NONE = 0xFFFF;
__device__ __forceinline__ int cl_lo(int v) { return v & 0xFFFF; }
__device__ __forceinline__ int cl_hi(int v) { return (int)((unsigned)v >> 16); }
__device__ __forceinline__ int cl_pack(const int* bound, int l) {
    if (l < 0) return -1;
    int r = 0;
#pragma unroll
    for (int t = 1; t < CL; ++t) r = l >= bound[t] ? t : r;
    return (r << 13) | (l - bound[r]);
}

template <bool UNITW>
__global__ void __cluster_dims__(CL, 1, 1) __launch_bounds__(CL_THREADS)
    k_flat_solve_cl(FlatArgs a, const int* __restrict__ list, int range_cap, int* __restrict__ spill_list,
                    int* __restrict__ spill_count) {
    constexpr int FT = CL_THREADS;
    extern __shared__ double dyn[];
    __shared__ double2 warps[FT];   // block_reduce2's partials
    __shared__ double2 slots[2][CL];
    __shared__ double2 result[3];   // two for the cluster's results, one for the CTA's
    __shared__ int bound[CL + 1];
    __shared__ int s_nruns;
    __shared__ double* s_dptr[CL];
    cgc::cluster_group cluster = cgc::this_cluster();
    const int q = (int)cluster.block_rank();
    const int f = list[blockIdx.x / CL];
    const int base = a.off[f];
    const int n = a.count[f];
    const int W = a.W, H = a.H;
    int* mem = a.members + base;
    int par = 0;

    // Members by (column, row), sorted by the first CTA.
    if (q == 0) {
        for (int k = threadIdx.x; k < n; k += FT) {
            int c = mem[k];
            mem[k] = pmod(c, W) * H + pdiv(c, W);
        }
        __syncthreads();
        sort_members(mem, n);
        for (int k = threadIdx.x; k < n; k += FT) {
            int key = mem[k];
            mem[k] = pmod(key, H) * W + pdiv(key, H);
        }
    }
    cluster.sync();
    // Range bounds: the first run head at or after q n / CL (every CTA computes all of them).
    if (threadIdx.x <= CL) {
        int t = (int)((long long)n * threadIdx.x / CL);
        while (t < n && !run_head(mem, t, W)) ++t;
        bound[threadIdx.x] = t;
    }
    if (threadIdx.x == 0) s_nruns = 0;
    __syncthreads();
    int widest = 0;
    for (int r = 0; r < CL; ++r) widest = max(widest, bound[r + 1] - bound[r]);
    if (widest > range_cap) {   // the same decision in every CTA, before any shared memory is shared
        if (q == 0 && threadIdx.x == 0) spill_list[atomicAdd(spill_count, 1)] = f;
        return;
    }
    const int lo = bound[q], m = bound[q + 1] - lo;
    // d first: the other CTAs read it at the same offset in this CTA's shared memory.
    double* s_d = dyn;
    double* s_r = s_d + m;
    double* s_z = s_r + m;
    double* s_ad = s_z + m;
    double* s_piv = s_ad + m;
    double* s_coef = s_piv + m;
    double* s_rcp = s_coef + m;   // 1 / pivot
    unsigned* s_run = reinterpret_cast<unsigned*>(s_rcp + m);   // first | last << 16, CTA-local
    if (threadIdx.x < CL) s_dptr[threadIdx.x] = cluster.map_shared_rank(s_d, (int)threadIdx.x);
    double* x = a.x + base + lo;
    double* degree = a.degree + base + lo;
    int4* nbr = reinterpret_cast<int4*>(a.nbr + (size_t)(base + lo) * 8);
    for (int j = threadIdx.x; j < m; j += FT) a.local[mem[lo + j]] = lo + j;
    cluster.sync();   // every member's index is in place

    // Entry level and highest entry (FlatRouting.kt:93-115, 427-445), degrees, member neighbours and
    // the rain (:239-295), as k_flat_solve_sm does for its members.
    float lo_f = FLT_MAX;
    for (int j = threadIdx.x; j < m; j += FT) lo_f = fminf(lo_f, a.filled[mem[lo + j]]);
    const double entry_level =
        cluster_combine(make_double2((double)lo_f, 0.0), MinMax2(), warps, slots, result, par, q).x;
    double hi = -INFINITY;
    for (int j = threadIdx.x; j < m; j += FT) {
        const int k = lo + j;
        const int cell = mem[k];
        const int col = pmod(cell, W), row = pdiv(cell, W);
        double total = 0.0;
        int nb8[8];
        int t = 0;
        for (int rs = -1; rs <= 1; ++rs) {
            const int nr = row + rs;
            for (int cs = -1; cs <= 1; ++cs) {
                if (cs == 0 && rs == 0) continue;
                nb8[t] = -1;
                if (nr >= 0 && nr < H) {
                    const int nb = nr * W + wrap_col(col + cs, W);
                    const double w = stencil_weight(a, cs, rs);
                    const int l = a.local[nb];
                    if (l >= 0) {
                        total = __dadd_rn(total, w);
                        nb8[t] = cl_pack(bound, l);
                    } else {
                        const double there = a.surface[nb];
                        if (there < entry_level) {
                            total = __dadd_rn(total, w);
                            if (there > hi) hi = there;
                        }
                    }
                }
                ++t;
            }
        }
        degree[j] = total;
        x[j] = 0.0;
        nbr[j] = make_int4(nbr_pack(nb8[0], nb8[1]), nbr_pack(nb8[2], nb8[3]), nbr_pack(nb8[4], nb8[5]),
                           nbr_pack(nb8[6], nb8[7]));
        s_r[j] = __dadd_rn(1.0, __dmul_rn(0.5, (double)smooth_seeded_field(W, a.lattice, col, row,
                                                                             a.seed ^ kRainReliefSalt)));
        if (run_head(mem, k, W)) {
            int e = k;
            while (run_continues(mem, n, e, W, H)) ++e;
            s_run[atomicAdd(&s_nruns, 1)] = (unsigned)j | ((unsigned)(e - lo) << 16);
        }
    }
    const double entry_height = cluster_combine(make_double2(0.0, hi), MinMax2(), warps, slots, result, par, q).y;
    const int runs = s_nruns;

    // Thomas pivots down each run (FlatRouting.kt:388-395) and ns / pivot for the way back up.
    for (int i = threadIdx.x; i < runs; i += FT) {
        const int first = (int)(s_run[i] & 0xFFFFu), last = (int)(s_run[i] >> 16);
        double p = degree[first];
        for (int j = first;; ++j) {
            s_piv[j] = p;
            s_coef[j] = __ddiv_rn(a.ns, p);
            s_rcp[j] = __ddiv_rn(1.0, p);
            if (j == last) break;
            p = __dsub_rn(degree[j + 1], __ddiv_rn(UNITW ? 1.0 : __dmul_rn(a.ns, a.ns), p));
        }
    }
    __syncthreads();

    auto precondition = [&]() {
        for (int i = threadIdx.x; i < runs; i += FT) {
            const int first = (int)(s_run[i] & 0xFFFFu), last = (int)(s_run[i] >> 16);
            double v = div_by(__dadd_rn(s_r[first], 0.0), s_piv[first], s_rcp[first]);
            s_z[first] = v;
            for (int j = first + 1; j <= last; ++j) {
                v = div_by(__dadd_rn(s_r[j], UNITW ? v : __dmul_rn(a.ns, v)), s_piv[j], s_rcp[j]);
                s_z[j] = v;
            }
            double below = v;
            for (int j = last - 1; j >= first; --j) {
                below = __dadd_rn(s_z[j], __dmul_rn(s_coef[j], below));
                s_z[j] = below;
            }
        }
    };
    const double w8[8] = {a.diag, a.ns, a.diag, a.ew, a.ew, a.diag, a.ns, a.diag};   // stencil order

    // Preconditioned conjugate gradients (FlatRouting.kt:296-333).
    precondition();
    __syncthreads();
    double rn = 0.0, ra = 0.0;
    for (int j = threadIdx.x; j < m; j += FT) {
        const double rv = s_r[j], zv = s_z[j];
        s_d[j] = zv;
        rn = __dadd_rn(rn, __dmul_rn(rv, rv));
        ra = __dadd_rn(ra, __dmul_rn(rv, zv));
    }
    double2 sums = cluster_combine(make_double2(rn, ra), Sum2(), warps, slots, result, par, q);   // also publishes d
    double rnorm = sums.x, rap = sums.y;
    const double stop_at = __dmul_rn(__dmul_rn(rnorm, 1e-7), 1e-7);
    const int most = 64 + (int)(8.0 * sqrt((double)n));
    for (int it = 0; rnorm > stop_at && it < most; ++it) {
        double e = 0.0;
        for (int j = threadIdx.x; j < m; j += FT) {
            const int4 qv = nbr[j];
            const int l8[8] = {cl_lo(qv.x), cl_hi(qv.x), cl_lo(qv.y), cl_hi(qv.y),
                               cl_lo(qv.z), cl_hi(qv.z), cl_lo(qv.w), cl_hi(qv.w)};
            const double dk = s_d[j];
            double sum = __dmul_rn(degree[j], dk);
#pragma unroll
            for (int t = 0; t < 8; ++t) {
                if (l8[t] == CL_NONE) continue;
                const int owner = l8[t] >> 13, off = l8[t] & 8191;
                const double dn = owner == q ? s_d[off] : s_dptr[owner][off];
                sum = __dsub_rn(sum, UNITW ? dn : __dmul_rn(w8[t], dn));
            }
            s_ad[j] = sum;
            e = __dadd_rn(e, __dmul_rn(dk, sum));
        }
        const double energy = cluster_combine(make_double2(e, 0.0), Sum2(), warps, slots, result, par, q).x;
        if (energy <= 0.0 || rap <= 0.0) break;
        const double step = __ddiv_rn(rap, energy);
        for (int j = threadIdx.x; j < m; j += FT) {
            x[j] = __dadd_rn(x[j], __dmul_rn(step, s_d[j]));
            s_r[j] = __dsub_rn(s_r[j], __dmul_rn(step, s_ad[j]));
        }
        __syncthreads();
        precondition();
        __syncthreads();
        double nn = 0.0, na = 0.0;
        for (int j = threadIdx.x; j < m; j += FT) {
            const double rv = s_r[j];
            nn = __dadd_rn(nn, __dmul_rn(rv, rv));
            na = __dadd_rn(na, __dmul_rn(rv, s_z[j]));
        }
        sums = cluster_combine(make_double2(nn, na), Sum2(), warps, slots, result, par, q);
        const double improvement = __ddiv_rn(sums.y, rap);
        for (int j = threadIdx.x; j < m; j += FT) s_d[j] = __dadd_rn(s_z[j], __dmul_rn(improvement, s_d[j]));
        cluster.sync();   // every CTA's new d before the next Laplacian reads it
        rnorm = sums.x;
        rap = sums.y;
    }
    int positive = 1;
    double top = 0.0;
    for (int j = threadIdx.x; j < m; j += FT) {
        const double v = x[j];
        if (!(v > 0.0)) positive = 0;
        if (v > top) top = v;
    }
    const double2 pt = cluster_combine(make_double2(positive ? 1.0 : 0.0, top), MinMax2(), warps, slots, result, par, q);
    const double highest = pt.y;

    // FlatRouting.layInBand (FlatRouting.kt:455-489) over the cluster.
    bool laid = pt.x > 0.0 && !(highest <= 0.0 || entry_height >= entry_level);
    if (laid) {
        const double band = __dmul_rn(__dsub_rn(entry_level, entry_height), 0.9);
        for (int j = threadIdx.x; j < m; j += FT)
            a.surface[mem[lo + j]] = __dadd_rn(entry_height, __dmul_rn(band, __ddiv_rn(x[j], highest)));
        cluster.sync();
        double ok = 1.0;
        for (int j = threadIdx.x; j < m; j += FT) {
            const int cell = mem[lo + j];
            const int col = pmod(cell, W), row = pdiv(cell, W);
            const double here = a.surface[cell];
            bool lower = false;
            for (int rs = -1; rs <= 1 && !lower; ++rs) {
                const int nr = row + rs;
                if (nr < 0 || nr >= H) continue;
                for (int cs = -1; cs <= 1; ++cs) {
                    if (cs == 0 && rs == 0) continue;
                    if (a.surface[nr * W + wrap_col(col + cs, W)] < here) {
                        lower = true;
                        break;
                    }
                }
            }
            if (!lower) ok = 0.0;
        }
        ok = cluster_combine(make_double2(ok, 0.0), MinMax2(), warps, slots, result, par, q).x;
        if (ok <= 0.0) {
            for (int j = threadIdx.x; j < m; j += FT) a.surface[mem[lo + j]] = (double)a.filled[mem[lo + j]];
            laid = false;
        }
    }
    if (!laid && q == 0 && threadIdx.x == 0) atomicAdd(a.kept, 1);
}

// Flats of at most 32 members (nearly all flats: the fill's small depressions), packed 32 / S to a
// warp by size class, S in {4, 8, 16, 32}: a flat takes a segment of S lanes, one member per lane.
// An FP64 warp instruction costs the same however few lanes are busy, so packing the small flats
// divides their cost. The per-member arithmetic (degree, Laplacian row, the column runs' Thomas
// solves) is the reference's, done by the member's lane or the run head's lane; the dot products
// are butterflies within the segment, which give every lane of the segment the same bits; each
// segment runs its own CG iterations and stops on its own test (the warp loops while any segment
// is still going, a stopped segment's state no longer changes).
constexpr int WF = 8;   // warps per block

template <int S>
__device__ __forceinline__ double seg_sum(double v) {
#pragma unroll
    for (int o = S / 2; o > 0; o >>= 1) v = __dadd_rn(v, __shfl_xor_sync(0xFFFFFFFFu, v, o));
    return v;
}

template <int S>
__global__ void __launch_bounds__(32 * WF) k_flat_solve_seg(FlatArgs a, const int* __restrict__ list, int count) {
    constexpr int G = 32 / S;   // flats per warp
    const unsigned FULL = 0xFFFFFFFFu;
    __shared__ double s_right[WF][32], s_into[WF][32], s_piv[WF][32], s_coef[WF][32], s_rcp[WF][32], s_d[WF][32];
    __shared__ int s_cont[WF][32];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int seg = lane / S, sl = lane % S;
    const unsigned seg_mask = (S == 32 ? FULL : ((1u << S) - 1u)) << (seg * S);
    const int slot = (blockIdx.x * WF + w) * G + seg;
    if ((blockIdx.x * WF + w) * G >= count) return;   // the whole warp is past the list
    const int f = slot < count ? list[slot] : -1;
    const int n = f >= 0 ? a.count[f] : 0;
    const int base = f >= 0 ? a.off[f] : 0;
    const bool act = sl < n;
    const int W = a.W, H = a.H;

    // Members by (column, row): a bitonic sort across the segment's lanes.
    int key = act ? pmod(a.members[base + sl], W) * H + pdiv(a.members[base + sl], W) : INT_MAX;
#pragma unroll
    for (int k = 2; k <= S; k <<= 1)
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
            const int other = __shfl_xor_sync(FULL, key, j);
            const bool up = (sl & k) == 0;
            const bool lower = (sl & j) == 0;
            const int lo = min(key, other), hi = max(key, other);
            key = (lower == up) ? lo : hi;
        }
    const int cell = act ? pmod(key, H) * W + pdiv(key, H) : -1;
    if (act) {
        a.members[base + sl] = cell;
        a.local[cell] = sl;
    }
    __syncwarp();
    const int col = act ? pmod(cell, W) : 0, row = act ? pdiv(cell, W) : 0;

    // Entry level, highest entry, member neighbours (their lanes), degree and rain.
    float lo = act ? a.filled[cell] : FLT_MAX;
#pragma unroll
    for (int o = S / 2; o > 0; o >>= 1) lo = fminf(lo, __shfl_xor_sync(FULL, lo, o));
    const double entry_level = (double)lo;
    double hi = -INFINITY, deg = 0.0, rv = 0.0;
    int nb_lane[8];
    double nb_w[8];
#pragma unroll
    for (int t = 0; t < 8; ++t) nb_lane[t] = -1, nb_w[t] = 0.0;
    if (act) {
        int t = 0;
        for (int rs = -1; rs <= 1; ++rs) {
            const int nr = row + rs;
            for (int cs = -1; cs <= 1; ++cs) {
                if (cs == 0 && rs == 0) continue;
                if (nr >= 0 && nr < H) {
                    const int nb = nr * W + wrap_col(col + cs, W);
                    const double wgt = stencil_weight(a, cs, rs);
                    const int l = a.local[nb];
                    const double there = a.surface[nb];
                    if (l < 0 && there < entry_level && there > hi) hi = there;
                    if (l >= 0) {
                        deg = __dadd_rn(deg, wgt);
                        nb_lane[t] = seg * S + l;
                        nb_w[t] = wgt;
                    } else if (there < entry_level) {
                        deg = __dadd_rn(deg, wgt);
                    }
                }
                ++t;
            }
        }
        rv = __dadd_rn(1.0, __dmul_rn(0.5, (double)smooth_seeded_field(W, a.lattice, col, row,
                                                                         a.seed ^ kRainReliefSalt)));
    }
#pragma unroll
    for (int o = S / 2; o > 0; o >>= 1) hi = fmax(hi, __shfl_xor_sync(FULL, hi, o));
    const double entry_height = hi;

    // Column runs: contiguous lanes of the segment. Pivots and ns / pivot down each run by its head.
    const int prev_cell = __shfl_up_sync(FULL, cell, 1);
    const int next_cell = __shfl_down_sync(FULL, cell, 1);
    const bool head = act && (sl == 0 || prev_cell != cell - W);
    s_cont[w][lane] = (act && sl + 1 < n && next_cell == cell + W) ? 1 : 0;
    s_right[w][lane] = deg;
    __syncwarp();
    if (head) {
        int j = lane;
        double p = s_right[w][j];
        while (true) {
            s_piv[w][j] = p;
            s_coef[w][j] = __ddiv_rn(a.ns, p);
            s_rcp[w][j] = __ddiv_rn(1.0, p);
            if (!s_cont[w][j]) break;
            ++j;
            p = __dsub_rn(s_right[w][j], __ddiv_rn(__dmul_rn(a.ns, a.ns), p));
        }
    }
    __syncwarp();

    // z = M^-1 r through the runs (FlatRouting.ColumnRuns.solve).
    auto precondition = [&](double right) -> double {
        s_right[w][lane] = right;
        __syncwarp();
        if (head) {
            int j = lane;
            double v = div_by(__dadd_rn(s_right[w][j], 0.0), s_piv[w][j], s_rcp[w][j]);
            s_into[w][j] = v;
            while (s_cont[w][j]) {
                ++j;
                v = div_by(__dadd_rn(s_right[w][j], __dmul_rn(a.ns, v)), s_piv[w][j], s_rcp[w][j]);
                s_into[w][j] = v;
            }
            double below = v;
            for (int i = j - 1; i >= lane; --i) {
                const double u = __dadd_rn(s_into[w][i], __dmul_rn(s_coef[w][i], below));
                s_into[w][i] = u;
                below = u;
            }
        }
        __syncwarp();
        const double z = act ? s_into[w][lane] : 0.0;
        __syncwarp();
        return z;
    };
    auto laplacian = [&](double dv) -> double {
        s_d[w][lane] = dv;
        __syncwarp();
        double sum = __dmul_rn(deg, dv);
#pragma unroll
        for (int t = 0; t < 8; ++t)
            if (nb_lane[t] >= 0) sum = __dsub_rn(sum, __dmul_rn(nb_w[t], s_d[w][nb_lane[t]]));
        __syncwarp();
        return act ? sum : 0.0;
    };

    // Preconditioned conjugate gradients (FlatRouting.kt:296-333), per segment.
    double x = 0.0, r = act ? rv : 0.0;
    double z = precondition(r);
    double d = z;
    double rnorm = seg_sum<S>(act ? __dmul_rn(r, r) : 0.0);
    double rap = seg_sum<S>(act ? __dmul_rn(r, z) : 0.0);
    const double stop_at = __dmul_rn(__dmul_rn(rnorm, 1e-7), 1e-7);
    const int most = 64 + (int)(8.0 * sqrt((double)(n > 0 ? n : 1)));
    bool stopped = f < 0;
    for (int it = 0;; ++it) {
        if (!stopped && !(rnorm > stop_at && it < most)) stopped = true;
        if (!__any_sync(FULL, !stopped)) break;
        const double ad = laplacian(d);
        const double energy = seg_sum<S>(act ? __dmul_rn(d, ad) : 0.0);
        if (!stopped && (energy <= 0.0 || rap <= 0.0)) stopped = true;
        const bool go = !stopped;
        const double step = __ddiv_rn(rap, energy);
        if (go && act) {
            x = __dadd_rn(x, __dmul_rn(step, d));
            r = __dsub_rn(r, __dmul_rn(step, ad));
        }
        const double next_norm = seg_sum<S>(act ? __dmul_rn(r, r) : 0.0);
        const double zn = precondition(r);
        const double next_ap = seg_sum<S>(act ? __dmul_rn(r, zn) : 0.0);
        if (go) {
            const double improvement = __ddiv_rn(next_ap, rap);
            if (act) d = __dadd_rn(zn, __dmul_rn(improvement, d));
            rnorm = next_norm;
            rap = next_ap;
        }
    }
    // Every collective below runs with the whole warp; a segment's decisions are read from its bits.
    const bool positive = (__ballot_sync(FULL, act && !(x > 0.0)) & seg_mask) == 0;
    double top = act ? x : 0.0;
#pragma unroll
    for (int o = S / 2; o > 0; o >>= 1) top = fmax(top, __shfl_xor_sync(FULL, top, o));
    const double highest = top > 0.0 ? top : 0.0;

    // FlatRouting.layInBand (FlatRouting.kt:455-489).
    bool laid = f >= 0 && positive && !(highest <= 0.0 || entry_height >= entry_level);
    if (laid && act) {
        const double band = __dmul_rn(__dsub_rn(entry_level, entry_height), 0.9);
        a.surface[cell] = __dadd_rn(entry_height, __dmul_rn(band, __ddiv_rn(x, highest)));
    }
    __syncwarp();
    bool lower = !act;
    if (laid && act) {
        const double here = a.surface[cell];
        for (int rs = -1; rs <= 1 && !lower; ++rs) {
            const int nr = row + rs;
            if (nr < 0 || nr >= H) continue;
            for (int cs = -1; cs <= 1; ++cs) {
                if (cs == 0 && rs == 0) continue;
                if (a.surface[nr * W + wrap_col(col + cs, W)] < here) {
                    lower = true;
                    break;
                }
            }
        }
    }
    const bool all_lower = (__ballot_sync(FULL, lower) & seg_mask) == seg_mask;
    if (laid && !all_lower) {
        if (act) a.surface[cell] = (double)a.filled[cell];
        laid = false;
    }
    if (f >= 0 && !laid && sl == 0) atomicAdd(a.kept, 1);
}

// Every flat, listed by the kernel that takes it: lists[0] the 128-thread shared-memory kernel
// (33-512 members), lists[1] the cluster kernel (513-CL_FLAT), lists[2] k_flat_solve (larger),
// lists[3..6] k_flat_solve_seg with segments of 4, 8, 16 and 32 lanes. ctr[0..2] count the first
// three, ctr[3..4] hold the largest flat of the first two (their shared-memory size), ctr[5..8]
// count lists 3-6. A warp's flats of one class take one atomic.
constexpr int FLAT_CLASSES = 7;

__device__ __forceinline__ int flat_class(int n) {
    return n <= 4 ? 3 : n <= 8 ? 4 : n <= 16 ? 5 : n <= 32 ? 6 : n <= MID_FLAT ? 0 : n <= CL_FLAT ? 1 : 2;
}

__global__ void k_flat_lists(const int* __restrict__ count, int flats, int* __restrict__ lists, int* __restrict__ ctr) {
    const unsigned FULL = 0xFFFFFFFFu;
    const int lane = threadIdx.x & 31;
    const int stride = gridDim.x * blockDim.x;
    for (int base = blockIdx.x * blockDim.x; base < flats; base += stride) {
        const int f = base + threadIdx.x;
        const int n = f < flats ? count[f] : 0;
        const int c = f < flats ? flat_class(n) : -1;
        const unsigned group = __match_any_sync(FULL, c);
        const int leader = __ffs(group) - 1;
        int* counter = c >= 3 ? &ctr[2 + c] : &ctr[c < 0 ? 0 : c];
        int slot = 0;
        if (c >= 0 && lane == leader) slot = atomicAdd(counter, __popc(group));
        slot = __shfl_sync(FULL, slot, leader) + __popc(group & ((1u << lane) - 1u));
        if (c >= 0) {
            lists[(size_t)c * flats + slot] = f;
            if (c < 2) atomicMax(&ctr[3 + c], n);
        }
    }
}

}  // namespace

// FlowRouting.facetReceiver over a caller's routing surface (FlowRouting.kt:218-310, the rule
// BeltErosion's rounds route the belts by): the facet receiver of every cell of d_mask, -1 elsewhere.
cg_status facet_receivers_dev(cg_ctx* ctx, int W, int H, const uint8_t* d_mask, const double* d_surface,
                              int64_t seed, double r, int32_t* d_recv) {
    Steps steps;
    steps.ew = 1.0f;
    steps.ns = (float)r;
    steps.diag = (float)std::sqrt(1.0 + r * r);
    CG_LAUNCH(ctx) k_receivers<<<ctx->num_sms * 8, RECV_THREADS, 0, ctx->stream>>>(d_mask, d_surface, W, H, steps,
                                                                                  (long long)seed, 1, nullptr, 0,
                                                                                  d_recv);
    CG_CHECK_LAUNCH(ctx);
    return CG_OK;
}

cg_status flow_directions_dev(cg_ctx* ctx, int W, int H, const uint8_t* d_land, const float* d_rel,
                              const float* d_filled, int64_t seed, double r, int lattice, bool by_facet,
                              bool over_potential, int32_t* d_recv, double* d_surface, FlatCounts* counts) {
    size_t N = (size_t)W * H;
    cudaStream_t sm = ctx->stream;
    int grid = ctx->num_sms * 8;
    FlatCounts fc{0, 0, 0};
    Steps steps;
    steps.ew = 1.0f;
    steps.ns = (float)r;
    steps.diag = (float)std::sqrt(1.0 + r * r);
    const int by = by_facet ? 1 : 0;
    bool routed = false;   // receivers already written (in two passes around the flats)
    if (!over_potential) {
        CG_LAUNCH(ctx) k_surface<<<grid, 256, 0, sm>>>(d_land, d_rel, d_filled, N, d_surface, nullptr, nullptr);
        CG_CHECK_LAUNCH(ctx);
    } else {
        CG_BUF(uint8_t, d_raised, ctx, S_FLATS, N);
        CG_BUF(int, d_local, ctx, S_FLATIDX, N);
        CG_BUF(int, d_root, ctx, S_LABEL, N);
        CG_BUF(int, d_label, ctx, S_SCRATCH2, N);
        CG_LAUNCH(ctx) k_surface<<<grid, 256, 0, sm>>>(d_land, d_rel, d_filled, N, d_surface, d_raised, d_local);
        CG_CHECK_LAUNCH(ctx);
        int flats = 0;
        cg_status st = component_labels(ctx, W, H, d_raised, d_root, d_label, &flats);
        if (st != CG_OK) return st;
        if (flats > 0) {
            CG_BUF(int, d_cnt, ctx, S_CG0, 3 * (size_t)flats + 1);
            int* d_off = d_cnt + flats;
            int* d_cur = d_off + flats;
            int* d_kept = d_cur + flats;
            CG_CUDA(ctx, cudaMemsetAsync(d_cnt, 0, sizeof(int) * (3 * (size_t)flats + 1), sm));
            CG_LAUNCH(ctx) k_flat_count<<<grid, 256, 0, sm>>>(d_label, N, d_cnt);
            CG_CHECK_LAUNCH(ctx);
            int raised = 0;
            if ((st = exclusive_scan(ctx, d_cnt, d_off, flats, &raised)) != CG_OK) return st;
            CG_BUF(int, d_members, ctx, S_FLATMEM, raised);
            CG_BUF(double, d_dbl, ctx, S_CG1, 10 * (size_t)raised);
            CG_LAUNCH(ctx) k_flat_scatter<<<grid, 256, 0, sm>>>(d_label, N, d_off, d_cur, d_members);
            CG_CHECK_LAUNCH(ctx);
            FlatArgs a;
            a.W = W;
            a.H = H;
            a.lattice = lattice;
            a.seed = seed;
            // FlatRouting.stencil (FlatRouting.kt:177-186).
            if (r <= 1.0) {
                double dg = 2.0 / (1.0 + r * r);
                a.ew = 1.0;
                a.ns = (1.0 + 2.0 * dg) / (r * r) - 2.0 * dg;
                a.diag = dg;
            } else {
                double dg = 2.0 / (1.0 + 1.0 / (r * r));
                a.ew = r * r * (1.0 + 2.0 * dg) - 2.0 * dg;
                a.ns = 1.0;
                a.diag = dg;
            }
            a.off = d_off;
            a.count = d_cnt;
            a.members = d_members;
            a.local = d_local;
            a.filled = d_filled;
            a.surface = d_surface;
            a.degree = d_dbl;
            a.pivot = d_dbl + raised;
            a.x = d_dbl + 2 * (size_t)raised;
            a.r = d_dbl + 3 * (size_t)raised;
            a.z = d_dbl + 4 * (size_t)raised;
            a.d = d_dbl + 5 * (size_t)raised;
            a.ad = d_dbl + 6 * (size_t)raised;
            a.coef = d_dbl + 7 * (size_t)raised;
            a.nbr = reinterpret_cast<short*>(d_dbl + 8 * (size_t)raised);   // 8 shorts per member
            a.kept = d_kept;
            // Flats of at most 32 members one warp each; larger ones one CTA each, by size class.
            CG_BUF(int, d_lists, ctx, S_CG5, FLAT_CLASSES * (size_t)flats + 9);
            int* d_ctr = d_lists + FLAT_CLASSES * (size_t)flats;
            CG_CUDA(ctx, cudaMemsetAsync(d_ctr, 0, 9 * sizeof(int), sm));
            CG_LAUNCH(ctx) k_flat_lists<<<(flats + 255) / 256, 256, 0, sm>>>(d_cnt, flats, d_lists, d_ctr);
            CG_CHECK_LAUNCH(ctx);
            int ctr[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
            CG_CUDA(ctx, cudaMemcpyAsync(ctr, d_ctr, sizeof(ctr), cudaMemcpyDeviceToHost, sm));
            CG_CUDA(ctx, cudaStreamSynchronize(sm));
            // The small and mid-sized flats on the auxiliary stream, beside the few large ones, whose
            // CTAs hold an SM each for the whole solve.
            CG_CUDA(ctx, cudaEventRecord(ctx->fork, sm));
            CG_CUDA(ctx, cudaStreamWaitEvent(ctx->aux, ctx->fork, 0));
            CG_CUDA(ctx, cudaStreamWaitEvent(ctx->aux2, ctx->fork, 0));
            // The receivers away from the flats on the third stream, beside the flat solvers.
            CG_LAUNCH(ctx) k_receivers<<<grid, RECV_THREADS, 0, ctx->aux2>>>(d_land, d_surface, W, H, steps,
                                                                            (long long)seed, by, d_raised, 1, d_recv);
            CG_CHECK_LAUNCH(ctx);
            CG_CUDA(ctx, cudaEventRecord(ctx->join2, ctx->aux2));
            {
                const int* small = d_lists + 3 * (size_t)flats;
                if (ctr[5] > 0)
                    CG_LAUNCH(ctx) k_flat_solve_seg<4><<<(ctr[5] + 8 * WF - 1) / (8 * WF), 32 * WF, 0, ctx->aux>>>(a, small, ctr[5]);
                if (ctr[6] > 0)
                    CG_LAUNCH(ctx) k_flat_solve_seg<8><<<(ctr[6] + 4 * WF - 1) / (4 * WF), 32 * WF, 0, ctx->aux>>>(
                        a, small + flats, ctr[6]);
                if (ctr[7] > 0)
                    CG_LAUNCH(ctx) k_flat_solve_seg<16><<<(ctr[7] + 2 * WF - 1) / (2 * WF), 32 * WF, 0, ctx->aux>>>(
                        a, small + 2 * (size_t)flats, ctr[7]);
                if (ctr[8] > 0)
                    CG_LAUNCH(ctx) k_flat_solve_seg<32><<<(ctr[8] + WF - 1) / WF, 32 * WF, 0, ctx->aux>>>(
                        a, small + 3 * (size_t)flats, ctr[8]);
            }
            if (ctr[0] > 0)
                CG_LAUNCH(ctx) k_flat_solve_sm<128><<<ctr[0], 128, (size_t)ctr[3] * SM_BYTES_PER_MEMBER, ctx->aux>>>(
                    a, d_lists);
            CG_CHECK_LAUNCH(ctx);
            if (ctr[1] > 0) {
                // Per CTA a share of the largest flat with room for the run-head rounding of its bounds;
                // a flat whose ranges need more goes to k_flat_solve.
                const int cap = std::min(std::min(CL_RANGE_MAX, CL_SMEM_MEMBERS),
                                         std::min(ctr[4], 2 * ((ctr[4] + CL - 1) / CL) + 64));
                // More than half an SM's shared memory, so that no two CTAs of a cluster share an SM (and
                // its FP64 pipe, which bounds the solve).
                const size_t bytes = std::max((size_t)cap * SM_BYTES_PER_MEMBER, (size_t)116 * 1024);
                const bool unit = a.ew == 1.0 && a.ns == 1.0 && a.diag == 1.0;
                auto kernel = unit ? k_flat_solve_cl<true> : k_flat_solve_cl<false>;
                // The attribute is the kernel's, shared by every context of the process: set it to the
                // most any launch asks for, so that a context on another thread lowering it between this
                // call and the launch below cannot make the launch fail.
                const size_t most = std::max((size_t)std::min(CL_RANGE_MAX, CL_SMEM_MEMBERS) * SM_BYTES_PER_MEMBER,
                                             (size_t)116 * 1024);
                CG_CUDA(ctx, cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)most));
                CG_LAUNCH(ctx) kernel<<<ctr[1] * CL, CL_THREADS, bytes, sm>>>(a, d_lists + flats, cap,
                                                                              d_lists + 2 * (size_t)flats, d_ctr + 2);
                CG_CHECK_LAUNCH(ctx);
                CG_CUDA(ctx, cudaMemcpyAsync(&ctr[2], d_ctr + 2, sizeof(int), cudaMemcpyDeviceToHost, sm));
                CG_CUDA(ctx, cudaStreamSynchronize(sm));
            }
            if (ctr[2] > 0) {
                a.large = d_lists + 2 * (size_t)flats;
                CG_LAUNCH(ctx) k_flat_solve<<<ctr[2], FT, 0, sm>>>(a);
                CG_CHECK_LAUNCH(ctx);
            }
            CG_CUDA(ctx, cudaEventRecord(ctx->join, ctx->aux));
            CG_CUDA(ctx, cudaStreamWaitEvent(sm, ctx->join, 0));
            CG_CUDA(ctx, cudaStreamWaitEvent(sm, ctx->join2, 0));
            // The receivers next to raised cells, now that the flats' surfaces are laid.
            CG_LAUNCH(ctx) k_receivers<<<grid, RECV_THREADS, 0, sm>>>(d_land, d_surface, W, H, steps, (long long)seed,
                                                                     by, d_raised, 2, d_recv);
            CG_CHECK_LAUNCH(ctx);
            routed = true;
            CG_CUDA(ctx, cudaMemcpyAsync(&fc.kept, d_kept, sizeof(int), cudaMemcpyDeviceToHost, sm));
            CG_CUDA(ctx, cudaStreamSynchronize(sm));
            fc.flats = flats;
            fc.raised = raised;
        }
    }
    if (!routed) {
        CG_LAUNCH(ctx) k_receivers<<<grid, RECV_THREADS, 0, sm>>>(d_land, d_surface, W, H, steps, (long long)seed, by,
                                                                  nullptr, 0, d_recv);
        CG_CHECK_LAUNCH(ctx);
    }
    if (counts) *counts = fc;
    return CG_OK;
}

}  // namespace cg
