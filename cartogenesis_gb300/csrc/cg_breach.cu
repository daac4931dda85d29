// The outlet notch on the device: HydraulicErosion.breach (HydraulicErosion.kt:1931-2171) as the
// rounds and the closing pass of profile P1 run it (belowSea false, nothing carried), reproducing the
// reference's result exactly.
//
// The reference cuts the basins one after another, in the order FlowRouting.spillways found them,
// and a basin reads what the basins before it cut. What one basin can touch is fixed before any
// cutting starts: its channel is the chain of receivers from the lip for as long as the summed ground
// steps stay under the reach (the walk may stop earlier, never later), and its margin is the chain
// from the entry to the lip, whatever the heights. So the footprints are listed once, and the basins
// are cut in waves: in each wave every basin still waiting claims the cells of its footprint with an
// atomic maximum of (wave, lowest basin index first), and a basin that holds every one of its claims
// has no earlier waiting basin sharing a cell with it. Those basins are pairwise disjoint, and every
// earlier basin they overlap has already been cut, so cutting them all at once gives the sequential
// result. The lowest waiting basin always holds its claims, so the waves end.
//
// One cooperative kernel runs the waves with two grid barriers each. Most footprints are a few cells
// (3.5 on average at 8192 x 4096): a thread takes such a basin, loads its cells and their heights
// up front (all loads in flight at once), places and checks its claims and replays the reference's
// walks in registers. A footprint longer than SHORT goes to a warp: the lanes load 32
// cells at a time, find where each walk stops with a ballot, carry the walks' float sums of steps
// lane by lane in the reference's order through shuffles, and cut the cells before the stop in
// parallel (each cut reads and writes only its own cell). Heights that an earlier wave may have cut
// on another SM are read through L2 (ld.cg) and written through it.
#include <cooperative_groups.h>

#include "cg_common.cuh"
#include "cg_internal.h"
#include "cg_util.h"

namespace cg {

namespace cgr = cooperative_groups;

namespace {

constexpr unsigned FULL = 0xFFFFFFFFu;
// Footprints of up to this many cells are cut by a thread, longer ones by a warp.
constexpr int SHORT = 8;

// Per-call control words at the end of the breach block.
enum { Q_SHORT0 = 0, Q_SHORT1 = 1, Q_LONG0 = 2, Q_LONG1 = 3, Q_ERROR = 4, Q_CELLS = 5, Q_WAVES = 6, Q_WORDS = 8 };

struct BreachDev {
    int W;
    int count;
    long long N;
    const int* spill;
    const int* entry;
    const float* level;
    const float* floor_;
    const uint8_t* land;
    const int32_t* recv;
    const float* area;
    float* rel;
    float* ground;
    float* surface;
    float* settled;      // profile P2's settled heights, or NULL
    double* load;        // profile P2's load in transit, or NULL
    float land_cells;
    float land_range;
    float pond_depth;
    float coefficient;   // relativeIncisionCoefficient * outletIncisionRatio (1.125), as the reference's first product
    float gradient;      // notchFallPerCell
    float reach;         // outletReachCells, compared as a float
    float step_ns;
    float step_diag;
    int* n;              // footprint cells per basin (count + 1, the last 0)
    int* start;          // exclusive scan of n
    int* n1;             // of those, the channel's
    int* foot;           // the channel from the lip, then the margin from the entry
    unsigned long long* claim;
    int* queue;          // four lists of `count` waiting basins: short (two waves), then long
    int* q;              // Q_* words
};

// GroundSteps.between (GroundSteps.kt:20-59) for cells of a grid `W` wide.
__device__ __forceinline__ float ground_step(const BreachDev& a, int from, int to) {
    const bool same_row = pdiv(from, a.W) == pdiv(to, a.W);
    const bool same_col = pmod(from, a.W) == pmod(to, a.W);
    return (!same_row && !same_col) ? a.step_diag : (!same_row ? a.step_ns : 1.0f);
}

// The step a walk adds leaving `cell` for `next` (east-west where there is no receiver).
__device__ __forceinline__ float walk_step(const BreachDev& a, int cell, int next) {
    return next >= 0 ? ground_step(a, cell, next) : 1.0f;
}

// Math.min(float, float) on the JVM: NaN if either is, -0 below +0.
__device__ __forceinline__ float jvm_min(float x, float y) {
    if (x != x) return x;
    if (y != y) return y;
    if (x == 0.0f && y == 0.0f) return __float_as_uint(x) & 0x80000000u ? x : y;
    return x < y ? x : y;
}

__device__ __forceinline__ bool notch_candidate(const BreachDev& a, int b) {
    return a.spill[b] >= 0 && __fsub_rn(a.level[b], a.floor_[b]) > 0.0f;
}

// The channel: cells from the lip while on land and under the reach (the reference's two walks
// down from the lip visit a prefix of these). Writes them to dst if given; returns their count.
__device__ int channel(const BreachDev& a, int spill, int* dst) {
    int n = 0;
    int cell = spill;
    float length = 0.0f;
    while (cell >= 0 && a.land[cell] && length < a.reach && n < a.N) {
        if (dst) dst[n] = cell;
        ++n;
        const int next = a.recv[cell];
        length = __fadd_rn(length, walk_step(a, cell, next));
        cell = next;
    }
    return n;
}

// The margin: cells from the entry to the lip, if that walk (bounded by the reach) arrives there.
__device__ int margin(const BreachDev& a, int spill, int entry, int* dst) {
    if (entry < 0 || entry == spill) return 0;
    int m = 0;
    int walker = entry;
    float widths = 0.0f;
    while (walker >= 0 && walker != spill && a.land[walker] && widths <= a.reach && m < a.N) {
        if (dst) dst[m] = walker;
        ++m;
        const int next = a.recv[walker];
        widths = __fadd_rn(widths, walk_step(a, walker, next));
        walker = next;
    }
    return walker == spill ? m : 0;
}

__global__ void k_footprint_count(BreachDev a) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b > a.count) return;
    if (b == a.count) {
        a.n[b] = 0;
        return;
    }
    int n1 = 0, n2 = 0;
    if (notch_candidate(a, b)) {
        n1 = channel(a, a.spill[b], nullptr);
        // A basin whose channel is empty walks nothing and cuts nothing.
        if (n1 > 0) n2 = margin(a, a.spill[b], a.entry[b], nullptr);
    }
    a.n1[b] = n1;
    a.n[b] = n1 + n2;
}

__global__ void k_footprint_fill(BreachDev a) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= a.count || a.n[b] == 0) return;
    int* dst = a.foot + a.start[b];
    const int n1 = channel(a, a.spill[b], dst);
    if (a.n[b] > n1) margin(a, a.spill[b], a.entry[b], dst + n1);
}

// Basins with a footprint of at most SHORT cells go to the short queue (a thread each), the rest
// to the long one (a warp each).
__global__ void k_queue_init(BreachDev a) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= a.count || a.n[b] == 0) return;
    if (a.n[b] <= SHORT) a.queue[atomicAdd(&a.q[Q_SHORT0], 1)] = b;
    else a.queue[2 * (size_t)a.count + atomicAdd(&a.q[Q_LONG0], 1)] = b;
}

// HydraulicErosion.raise with the amount `-take`, and the cut it makes in the shoreline-relative
// fields (HydraulicErosion.kt:2035-2050, 2084-2097). r, g and prior are relative[cell], ground[cell]
// and surface[cell] as read before this basin's cut (each cell is cut at most once per basin).
__device__ __forceinline__ int take(const BreachDev& a, int cell, float r, float g, float prior, float cut_level) {
    const double amount = __dmul_rn((double)__fsub_rn(r, cut_level), (double)a.land_range);
    const bool ponded = __fsub_rn(g, r) > a.pond_depth;
    const float now = (float)__dadd_rn((double)prior, -amount);
    __stcg(a.surface + cell, now);
    const double removed = -__dsub_rn((double)now, (double)prior);
    if (removed > 0.0) {
        const float as_relative = (float)__ddiv_rn(removed, (double)a.land_range);
        __stcg(a.rel + cell, __fsub_rn(r, as_relative));
        if (!ponded) __stcg(a.ground + cell, __fsub_rn(g, as_relative));
        // HydraulicErosion.kt:2045-2048: what the notch takes is carried on, and the settled
        // surface falls with the rock (a cell is cut by one basin at a time, in basin order).
        if (a.settled) __stcg(a.settled + cell, __fsub_rn(__ldcg(a.settled + cell), as_relative));
        if (a.load) __stcg(a.load + cell, __dadd_rn(__ldcg(a.load + cell), removed));
        return 1;
    }
    return 0;
}

__device__ __forceinline__ int take_down_to(const BreachDev& a, int cell, float r, float cut_level) {
    return take(a, cell, r, __ldcg(a.ground + cell), __ldcg(a.surface + cell), cut_level);
}

// walk 1's outcome, shared by both cutters: the new level of the lip, or false where the basin cuts
// nothing (HydraulicErosion.kt:2001-2027).
__device__ __forceinline__ bool new_level_of(const BreachDev& a, int spill, float level, float depth, float fall,
                                             float length, float last_step, int walked, int cell, float* out) {
    if (fall <= __fmul_rn(1e-6f, (float)walked) && cell >= 0 && !a.land[cell]) {
        fall = __fsub_rn(level, __ldcg(a.rel + cell));   // water: no basin cuts it
        length = __fadd_rn(length, last_step);
    }
    if (walked == 0) return false;
    float slope = __fmul_rn(__fdiv_rn(fall, length), (float)a.W);
    if (slope < 0.0f) slope = 0.0f;
    const float power = __fmul_rn(__fmul_rn(a.coefficient, __fsqrt_rn(__fdiv_rn(a.area[spill], a.land_cells))), slope);
    const float drop = jvm_min(power, jvm_min(depth, level));
    if (drop <= 0.0f) return false;
    *out = __fsub_rn(level, drop);
    return true;
}

__device__ __forceinline__ unsigned long long claim_key(int wave, int b) {
    return ((unsigned long long)wave << 32) | (unsigned long long)(0xFFFFFFFFu - (unsigned)b);
}

// A short basin's footprint cells, all loads in flight at once.
__device__ __forceinline__ int short_cells(const BreachDev& a, int b, int (&c)[SHORT]) {
    const int s0 = a.start[b];
    const int n = a.start[b + 1] - s0;
#pragma unroll
    for (int k = 0; k < SHORT; ++k) c[k] = k < n ? a.foot[s0 + k] : 0;
    return n;
}

// One short basin's notch by one thread (HydraulicErosion.kt:1958-2100): the footprint's heights
// are read up front, then the walks run in registers. Returns the cells cut.
__device__ int cut_short(const BreachDev& a, int b, const int (&c)[SHORT], int n) {
    const int n1 = a.n1[b];
    int nx[SHORT];
    float r[SHORT], g[SHORT], su[SHORT];
#pragma unroll
    for (int k = 0; k < SHORT; ++k) {
        if (k < n) {
            r[k] = __ldcg(a.rel + c[k]);
            g[k] = __ldcg(a.ground + c[k]);
            su[k] = __ldcg(a.surface + c[k]);
            nx[k] = a.recv[c[k]];
        } else {
            r[k] = g[k] = su[k] = 0.0f;
            nx[k] = -1;
        }
    }
    const float level = a.level[b];
    const float depth = __fsub_rn(level, a.floor_[b]);
    // Walk 1: the channel's fall and length.
    float fall = 0.0f, length = 0.0f, last_step = 1.0f;
    int walked = 0, cell = -1;
    bool going = true;
#pragma unroll
    for (int k = 0; k < SHORT; ++k) {
        if (going && k < n1) {
            fall = __fsub_rn(level, r[k]);
            if (fall > depth) {
                going = false;
                cell = c[k];
            } else {
                last_step = walk_step(a, c[k], nx[k]);
                length = __fadd_rn(length, last_step);
                ++walked;
                cell = nx[k];   // where the walk goes next, or left the land, or ran out of reach
            }
        }
    }
    float new_level;
    if (!new_level_of(a, c[0], level, depth, fall, length, last_step, walked, cell, &new_level)) return 0;
    int cut = 0;
    // Walk 2: down the channel, falling `gradient` a cell width, never below the shoreline.
    float from_lip = 0.0f;
    going = true;
#pragma unroll
    for (int k = 0; k < SHORT; ++k) {
        if (going && k < n1) {
            const float falling = __fsub_rn(new_level, __fmul_rn(from_lip, a.gradient));
            const float cut_level = falling < 0.0f ? 0.0f : falling;
            if (r[k] <= cut_level) {
                going = false;
            } else {
                cut += take(a, c[k], r[k], g[k], su[k], cut_level);
                from_lip = __fadd_rn(from_lip, walk_step(a, c[k], nx[k]));
            }
        }
    }
    // Back across the margin from the lip (margin cell k drains into k + 1, the last into the lip).
    float back = 0.0f;
    going = true;
#pragma unroll
    for (int k = SHORT - 1; k >= 0; --k) {
        if (going && k < n && k >= n1) {
            back = __fadd_rn(back, ground_step(a, c[k], nx[k]));
            const float cut_level = __fadd_rn(new_level, __fmul_rn(back, a.gradient));
            if (r[k] <= cut_level) going = false;
            else cut += take(a, c[k], r[k], g[k], su[k], cut_level);
        }
    }
    return cut;
}

// One long basin's notch by a whole warp (every lane calls it; all control flow is warp-uniform). The
// same walks as cut_short: walk 1 stops at the first cell whose fall exceeds the basin's depth, so a
// ballot finds it in each chunk of 32, and its length is the steps before it summed in order; walk 2
// and the margin stop at the first cell already at or below its cut level, which needs each lane's
// own running sum of steps (the reference's float additions, in its order) before the ballot. Returns
// this lane's count of cut cells.
__device__ int cut_long(const BreachDev& a, int b, int lane) {
    const int* list = a.foot + a.start[b];
    const int n1 = a.n1[b];
    const int n = a.n[b];
    const int spill = list[0];
    const float level = a.level[b];
    const float depth = __fsub_rn(level, a.floor_[b]);
    float fall = 0.0f, length = 0.0f, last_step = 1.0f;
    int walked = 0;
    int cell = -1;
    for (int k0 = 0; k0 < n1; k0 += 32) {
        const int j = k0 + lane;
        const bool valid = j < n1;
        int c = 0, next = -1;
        float f = 0.0f, step = 0.0f;
        if (valid) {
            c = list[j];
            f = __fsub_rn(level, __ldcg(a.rel + c));
            next = a.recv[c];
            step = walk_step(a, c, next);
        }
        const unsigned stop = __ballot_sync(FULL, valid && f > depth);
        const int m = stop ? __ffs(stop) - 1 : min(32, n1 - k0);   // cells walked in this chunk
        for (int t = 0; t < m; ++t) length = __fadd_rn(length, __shfl_sync(FULL, step, t));
        if (m > 0) last_step = __shfl_sync(FULL, step, m - 1);
        walked += m;
        if (stop) {
            fall = __shfl_sync(FULL, f, m);
            cell = __shfl_sync(FULL, c, m);
            break;
        }
        fall = __shfl_sync(FULL, f, m - 1);
        cell = __shfl_sync(FULL, next, m - 1);   // where the walk left the land or ran out of reach
    }
    float new_level;
    if (!new_level_of(a, spill, level, depth, fall, length, last_step, walked, cell, &new_level)) return 0;
    int cut = 0;
    float base = 0.0f;
    for (int k0 = 0; k0 < n1; k0 += 32) {
        const int j = k0 + lane;
        const bool valid = j < n1;
        int c = 0;
        float r = 0.0f, step = 0.0f;
        if (valid) {
            c = list[j];
            r = __ldcg(a.rel + c);
            step = walk_step(a, c, a.recv[c]);
        }
        float from_lip = base;
        for (int t = 0; t < 31; ++t) {
            const float v = __shfl_sync(FULL, step, t);
            if (t < lane) from_lip = __fadd_rn(from_lip, v);
        }
        const float falling = __fsub_rn(new_level, __fmul_rn(from_lip, a.gradient));
        const float cut_level = falling < 0.0f ? 0.0f : falling;
        const unsigned stop = __ballot_sync(FULL, valid && r <= cut_level);
        const int m = stop ? __ffs(stop) - 1 : 32;
        if (valid && lane < m) cut += take_down_to(a, c, r, cut_level);
        if (stop) break;
        base = __shfl_sync(FULL, __fadd_rn(from_lip, step), 31);
    }
    float back = 0.0f;
    for (int top = n - 1; top >= n1; top -= 32) {
        const int i = top - lane;
        const bool valid = i >= n1;
        int c = 0;
        float r = 0.0f, step = 0.0f;
        if (valid) {
            c = list[i];
            r = __ldcg(a.rel + c);
            step = ground_step(a, c, a.recv[c]);
        }
        float acc = back;
        for (int t = 0; t < 32; ++t) {
            const float v = __shfl_sync(FULL, step, t);
            if (t <= lane) acc = __fadd_rn(acc, v);
        }
        const float cut_level = __fadd_rn(new_level, __fmul_rn(acc, a.gradient));
        const unsigned stop = __ballot_sync(FULL, valid && r <= cut_level);
        const int m = stop ? __ffs(stop) - 1 : 32;
        if (valid && lane < m) cut += take_down_to(a, c, r, cut_level);
        if (stop) break;
        back = __shfl_sync(FULL, acc, 31);
    }
    return cut;
}

__global__ void __launch_bounds__(256) k_breach_waves(BreachDev a) {
    cgr::grid_group grid = cgr::this_grid();
    const int lane = threadIdx.x & 31;
    const int thread = blockIdx.x * blockDim.x + threadIdx.x;
    const int threads = gridDim.x * blockDim.x;
    const int warp = thread >> 5;
    const int warps = threads >> 5;
    const bool first = thread == 0;
    int cells = 0;
    int cur = 0;
    int wave = 1;
    for (;; ++wave) {
        const int shorts = __ldcg(a.q + Q_SHORT0 + cur);
        const int longs = __ldcg(a.q + Q_LONG0 + cur);
        if (shorts + longs == 0) break;
        if (wave > a.count + 1) {   // the lowest waiting basin cuts in every wave: cannot happen
            if (first) a.q[Q_ERROR] = 1;
            break;
        }
        const int* short_list = a.queue + (size_t)cur * a.count;
        const int* long_list = a.queue + (size_t)(2 + cur) * a.count;
        int* next_short = a.queue + (size_t)(cur ^ 1) * a.count;
        int* next_long = a.queue + (size_t)(2 + (cur ^ 1)) * a.count;
        int* next_shorts = a.q + Q_SHORT0 + (cur ^ 1);
        int* next_longs = a.q + Q_LONG0 + (cur ^ 1);
        // Claims. The atomics need no answer, so they do not wait.
        for (int i = warp; i < longs; i += warps) {
            const int b = __ldcg(long_list + i);
            const unsigned long long key = claim_key(wave, b);
            for (int j = a.start[b] + lane; j < a.start[b + 1]; j += 32) atomicMax(a.claim + a.foot[j], key);
        }
        for (int i = thread; i < shorts; i += threads) {
            const int b = __ldcg(short_list + i);
            const unsigned long long key = claim_key(wave, b);
            int c[SHORT];
            const int n = short_cells(a, b, c);
#pragma unroll
            for (int k = 0; k < SHORT; ++k)
                if (k < n) atomicMax(a.claim + c[k], key);
        }
        if (first) {
            *next_shorts = 0;
            *next_longs = 0;
        }
        grid.sync();
        // A basin holding every claim it placed cuts; the others wait for the next wave.
        for (int i = warp; i < longs; i += warps) {
            const int b = __ldcg(long_list + i);
            const unsigned long long key = claim_key(wave, b);
            bool held = true;
            for (int j = a.start[b] + lane; j < a.start[b + 1]; j += 32) held &= __ldcg(a.claim + a.foot[j]) == key;
            if (__all_sync(FULL, held)) cells += cut_long(a, b, lane);
            else if (lane == 0) __stcg(next_long + atomicAdd(next_longs, 1), b);
        }
        for (int i = thread; i < shorts; i += threads) {
            const int b = __ldcg(short_list + i);
            const unsigned long long key = claim_key(wave, b);
            int c[SHORT];
            const int n = short_cells(a, b, c);
            bool held = true;
#pragma unroll
            for (int k = 0; k < SHORT; ++k)
                if (k < n) held &= __ldcg(a.claim + c[k]) == key;
            if (held) cells += cut_short(a, b, c, n);
            else __stcg(next_short + atomicAdd(next_shorts, 1), b);
        }
        grid.sync();
        cur ^= 1;
    }
    if (cells) atomicAdd(a.q + Q_CELLS, cells);
    if (first) a.q[Q_WAVES] = wave - 1;
}

}  // namespace

cg_status breach_dev(cg_ctx* ctx, int W, int H, const uint8_t* d_land, float* d_rel, float* d_ground,
                     const int32_t* d_recv, const float* d_area, float land_cells, float land_range,
                     const BreachRates& rates, float* d_surface, int* h_cells, float* d_settled, double* d_load) {
    const size_t N = (size_t)W * H;
    cudaStream_t sm = ctx->stream;
    if (h_cells) *h_cells = 0;
    CG_BUF(int32_t, d_label, ctx, S_BASIN2, N);
    BasinArrays bas;
    int count = 0;
    cg_status st = basins_dev(ctx, W, H, d_land, d_rel, d_ground, d_recv, rates.pond_depth, d_label, &bas, &count);
    if (st != CG_OK) return st;
    if (count == 0) return CG_OK;
    // n (count + 1) | start (count + 1) | n1 (count) | four queues (4 count) | control words.
    CG_BUF(int, d_block, ctx, S_BREACH, 7 * (size_t)count + 2 + Q_WORDS);
    BreachDev a;
    a.W = W;
    a.count = count;
    a.N = (long long)N;
    a.spill = bas.spill;
    a.entry = bas.entry;
    a.level = bas.level;
    a.floor_ = bas.floor_;
    a.land = d_land;
    a.recv = d_recv;
    a.area = d_area;
    a.rel = d_rel;
    a.ground = d_ground;
    a.surface = d_surface;
    a.settled = d_settled;
    a.load = d_load;
    a.land_cells = land_cells;
    a.land_range = land_range;
    a.pond_depth = rates.pond_depth;
    a.coefficient = rates.relative_incision_coefficient * 1.125f;   // ErosionConfig.outletIncisionRatio
    a.gradient = rates.notch_fall_per_cell;
    a.reach = (float)rates.outlet_reach_cells;
    a.step_ns = rates.step_ns;
    a.step_diag = rates.step_diag;
    a.n = d_block;
    a.start = a.n + count + 1;
    a.n1 = a.start + count + 1;
    a.queue = a.n1 + count;
    a.q = a.queue + 4 * (size_t)count;
    a.foot = nullptr;
    a.claim = nullptr;
    const int blocks = (count + 1 + 255) / 256;
    CG_LAUNCH(ctx) k_footprint_count<<<blocks, 256, 0, sm>>>(a);
    CG_CHECK_LAUNCH(ctx);
    int total = 0;
    st = exclusive_scan(ctx, a.n, a.start, count + 1, &total);
    if (st != CG_OK) return st;
    if (total == 0) return CG_OK;
    CG_BUF(int, d_foot, ctx, S_FOOT, (size_t)total);
    CG_BUF(unsigned long long, d_claim, ctx, S_CLAIM, N);
    a.foot = d_foot;
    a.claim = d_claim;
    CG_CUDA(ctx, cudaMemsetAsync(d_claim, 0, N * sizeof(unsigned long long), sm));
    CG_CUDA(ctx, cudaMemsetAsync(a.q, 0, Q_WORDS * sizeof(int), sm));
    CG_LAUNCH(ctx) k_footprint_fill<<<blocks, 256, 0, sm>>>(a);
    CG_LAUNCH(ctx) k_queue_init<<<blocks, 256, 0, sm>>>(a);
    CG_CHECK_LAUNCH(ctx);
    int per_sm = 0;
    CG_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_breach_waves, 256, 0));
    if (per_sm < 1) return fail(ctx, CG_CUDA, "breach kernel cannot be resident");
    // Up to two CTAs per SM: the first waves hold most of the basins, a thread each.
    const int cgrid = ctx->num_sms * (per_sm < 2 ? per_sm : 2);
    void* kargs[] = {&a};
    ctx->launches++;
    CG_CUDA(ctx, cudaLaunchCooperativeKernel((void*)k_breach_waves, cgrid, 256, kargs, 0, sm));
    int q[Q_WORDS];
    CG_CUDA(ctx, cudaMemcpyAsync(q, a.q, sizeof(q), cudaMemcpyDeviceToHost, sm));
    CG_CUDA(ctx, cudaStreamSynchronize(sm));
    if (q[Q_ERROR]) return fail(ctx, CG_CUDA, "outlet notch: waves did not converge over %d basins", count);
    if (h_cells) *h_cells = q[Q_CELLS];
    return CG_OK;
}

}  // namespace cg
