// The drainage tree on the device: FlowRouting.drainageOrder and accumulate
// (FlowRouting.kt:485-511, 695-729), HydraulicErosion.incise (HydraulicErosion.kt:2298-2390) and
// FlowRouting.spillways (FlowRouting.kt:573-677), each reproducing the reference's result exactly.
//
// Kahn order without a queue. The reference seeds a FIFO with the land sources in index order and
// appends a cell when its last donor leaves the queue, so the queue is sorted by level (the longest
// donor chain into a cell) and, within a level, by the position of the last donor to leave. By
// induction that is the order of the chain of "deepest latest" donors back to a source, i.e. of
// that source's index. So a cell's place is the key (level, s), s the largest source index among the
// sources farthest upstream of it, and key(r) = max over donors of key(d) + (1, 0): a tree
// reduction from the leaves. It runs as a last-arriver walk: one thread per source climbs down its
// receivers; at each cell the thread that brings the donor count to zero computes the cell's key and
// its accumulation (its weight plus its donors' areas in key order, the reference's float
// additions in the reference's order) and carries on; the others stop. No barrier, O(N) work.
//
// Incision needs each receiver final before its donors: cells are bucketed by their Kahn level (a
// receiver's level is always higher than its donors') and one cooperative kernel sweeps the levels
// from the top down with a grid barrier between them. Every order with receivers first gives the
// same bits, because a cell reads only its receiver's final state.
#include <cooperative_groups.h>
#include <cuda/atomic>

#include <cfloat>
#include <climits>
#include <utility>
#include <vector>

#include "cg_common.cuh"
#include "cg_internal.h"
#include "cg_util.h"

namespace cg {

namespace cgr = cooperative_groups;

namespace {

constexpr long long LEVEL_ONE = 1LL << 32;

__device__ __forceinline__ bool is_land_receiver(const uint8_t* land, int r) { return r >= 0 && land[r]; }

// Neighbour directions in stencil order (rows -1..1, then columns -1..1, the cell itself left out).
__device__ __forceinline__ int dir_row(int t) { return t < 3 ? -1 : (t < 5 ? 0 : 1); }
__device__ __forceinline__ int dir_col(int t) { return t < 3 ? t - 1 : (t < 5 ? (t == 3 ? -1 : 1) : t - 6); }
__device__ __forceinline__ int dir_of(int rs, int cs) { return (rs + 1) * 3 + (cs + 1) - ((rs > 0 || (rs == 0 && cs > 0)) ? 1 : 0); }
__device__ __forceinline__ int step_to(int W, int c, int t) {
    const int row = pdiv(c, W), col = pmod(c, W);
    return (row + dir_row(t)) * W + wrap_col(col + dir_col(t), W);
}

// The tree's links, one byte each per cell: down[c] the direction from c to its receiver when that
// receiver is land (0xFF otherwise), and mask[r] bit t set when the neighbour of r in direction t
// drains into r. The mask bytes are set with a 32-bit atomicOr on the word holding them.
__global__ void k_links(const uint8_t* __restrict__ land, const int32_t* __restrict__ recv, int W, int H,
                        uint8_t* __restrict__ down, uint8_t* __restrict__ mask) {
    const size_t N = (size_t)W * H;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x) {
        uint8_t d = 0xFF;
        if (land[i]) {
            const int r = recv[i];
            if (is_land_receiver(land, r)) {
                const int c = (int)i;
                int rs = pdiv(r, W) - pdiv(c, W);
                int cs = pmod(r, W) - pmod(c, W);
                if (cs > 1) cs -= W;
                if (cs < -1) cs += W;
                d = (uint8_t)dir_of(rs, cs);
                const int up = dir_of(-rs, -cs);   // from r back to c
                atomicOr(reinterpret_cast<unsigned*>(mask + (r & ~3)), 1u << (up + 8 * (r & 3)));
            }
        }
        down[i] = d;
    }
}

// Donor counts, the pending counts of the walk, and the list of land sources (cells no land cell
// drains into). A CTA takes SRC_PER cells per thread at a time and reserves its sources' slots with
// one atomic (a per-warp atomic on the one counter was the kernel's cost); the list's order does not
// matter, since the walk's results do not depend on which thread reaches a cell first.
constexpr int SRC_PER = 8;

__global__ void __launch_bounds__(256) k_sources(const uint8_t* __restrict__ land, const uint8_t* __restrict__ mask,
                                                 size_t N, int32_t* __restrict__ donors,
                                                 int32_t* __restrict__ pending, int* __restrict__ sources,
                                                 int* __restrict__ n_sources) {
    const unsigned FULL = 0xFFFFFFFFu;
    __shared__ int warp_tot[8];
    __shared__ int s_base;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const size_t chunk = (size_t)blockDim.x * SRC_PER;
    for (size_t cb = (size_t)blockIdx.x * chunk; cb < N; cb += (size_t)gridDim.x * chunk) {
        unsigned bits = 0;
        int cnt = 0;
#pragma unroll
        for (int k = 0; k < SRC_PER; ++k) {
            const size_t i = cb + (size_t)k * blockDim.x + threadIdx.x;
            if (i >= N) continue;
            const int n = __popc((unsigned)mask[i]);
            donors[i] = n;
            pending[i] = n;
            if (land[i] && n == 0) {
                bits |= 1u << k;
                ++cnt;
            }
        }
        int incl = cnt;
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(FULL, incl, o);
            if (lane >= o) incl += t;
        }
        if (lane == 31) warp_tot[warp] = incl;
        __syncthreads();
        if (threadIdx.x == 0) {
            int run = 0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
                const int t = warp_tot[w];
                warp_tot[w] = run;
                run += t;
            }
            s_base = run ? atomicAdd(n_sources, run) : 0;
        }
        __syncthreads();
        int slot = s_base + warp_tot[warp] + incl - cnt;
#pragma unroll
        for (int k = 0; k < SRC_PER; ++k)
            if (bits & (1u << k)) sources[slot++] = (int)(cb + (size_t)k * blockDim.x + threadIdx.x);
        __syncthreads();
    }
}

struct WalkArgs {
    int W, H;
    const uint8_t* down;
    const uint8_t* mask;
    int32_t* pending;
    long long* key;
    const float* weights;   // null: keys only
    float* area;
    const int* sources;
    const int* n_sources;
    unsigned long long* max_key;
};

// One thread per source climbs down its receivers while it is the last donor into each. At a cell
// r it already holds the key and area of the cell it came from; r's donor mask and weight are
// loaded beside the atomic that decides whether it goes on, so a step costs the atomic and one
// round of loads of the other donors' keys and areas.
__global__ void __launch_bounds__(64) k_walk(WalkArgs a) {
    const unsigned FULL = 0xFFFFFFFFu;
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long local_max = 0;
    if (idx < *a.n_sources) {
        int c = a.sources[idx];
        long long kc = (long long)c;   // a source: level 0, its own index
        float ac = a.weights ? a.weights[c] : 0.0f;
        a.key[c] = kc;
        if (a.weights) a.area[c] = ac;
        local_max = (unsigned long long)kc;
        while (true) {
            const int d = a.down[c];
            if (d == 0xFF) break;
            const int r = step_to(a.W, c, d);
            const unsigned m = a.mask[r];
            const float wr = a.weights ? a.weights[r] : 0.0f;
            // Release: this cell's key and area are visible before its arrival is counted. Acquire:
            // the last donor in sees every other donor's.
            cuda::atomic_ref<int, cuda::thread_scope_device> pend(a.pending[r]);
            if (pend.fetch_sub(1, cuda::memory_order_acq_rel) != 1) break;   // not the last donor in
            // The donors' keys and areas (the cell just left from registers). Keys are distinct, so
            // each donor's rank is the number of smaller keys; the areas are added in rank order.
            long long kt[8];
            float at[8];
            long long kmax = LLONG_MIN;
#pragma unroll
            for (int t = 0; t < 8; ++t) {
                kt[t] = LLONG_MAX;
                at[t] = 0.0f;
                if (!(m & (1u << t))) continue;
                const int dn = step_to(a.W, r, t);
                if (dn == c) {
                    kt[t] = kc;
                    at[t] = ac;
                } else {
                    kt[t] = *((volatile long long*)&a.key[dn]);
                    if (a.weights) at[t] = *((volatile float*)&a.area[dn]);
                }
                kmax = kt[t] > kmax ? kt[t] : kmax;
            }
            kc = kmax + LEVEL_ONE;
            a.key[r] = kc;
            if (a.weights) {
                int rank[8];
#pragma unroll
                for (int t = 0; t < 8; ++t) {
                    rank[t] = 0;
#pragma unroll
                    for (int u = 0; u < 8; ++u) rank[t] += (kt[u] < kt[t]) ? 1 : 0;
                }
                const int n = __popc(m);
                float sum = wr;
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    if (j >= n) break;
                    float pick = 0.0f;
#pragma unroll
                    for (int t = 0; t < 8; ++t) pick = rank[t] == j && (m & (1u << t)) ? at[t] : pick;
                    sum = __fadd_rn(sum, pick);
                }
                ac = sum;
                a.area[r] = sum;
            }
            if ((unsigned long long)kc > local_max) local_max = (unsigned long long)kc;
            c = r;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long other = __shfl_xor_sync(FULL, local_max, o);
        if (other > local_max) local_max = other;
    }
    if ((threadIdx.x & 31) == 0 && local_max) atomicMax(a.max_key, local_max);
}

// Areas of land cells are the weights where no walk reached (sea cells hold 0).
__global__ void k_area_sea(const uint8_t* __restrict__ land, size_t N, float* __restrict__ area) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x)
        if (!land[i]) area[i] = 0.0f;
}

__global__ void k_land_flags(const uint8_t* __restrict__ land, size_t N, int* __restrict__ flag) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x)
        flag[i] = land[i] ? 1 : 0;
}

// The drainage order as a stable LSD radix sort of the land cells' compact keys, level N + deepest
// source (distinct, ordered as the drainage keys are), 8 bits a pass over the bits they use. A CTA
// takes a tile of kRsTile cells: it counts its digits, the counts are scanned digit-major over the
// tiles, and the CTA scatters its tile in order, 256 cells at a time, each cell's place among the
// chunk's cells of its digit found with __match_any_sync within its warp and per-warp counts across
// warps, so cells of one digit keep their order.
constexpr int kRsTile = 4096;

__global__ void k_land_compact_ck(const uint8_t* __restrict__ land, const int* __restrict__ pos,
                                  const long long* __restrict__ key, size_t N, unsigned long long* __restrict__ ck,
                                  int* __restrict__ vals, unsigned long long* __restrict__ kmax) {
    unsigned long long m = 0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x)
        if (land[i]) {
            const unsigned long long k = (unsigned long long)key[i];
            const unsigned long long c = (k >> 32) * (unsigned long long)N + (k & 0xFFFFFFFFull);
            ck[pos[i]] = c;
            vals[pos[i]] = (int)i;
            m = c > m ? c : m;
        }
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long t = __shfl_down_sync(0xFFFFFFFFu, m, o);
        m = t > m ? t : m;
    }
    if ((threadIdx.x & 31) == 0 && m) atomicMax(kmax, m);
}

__global__ void __launch_bounds__(256) k_rs_hist(const unsigned long long* __restrict__ keys, int n, int shift,
                                                 int tiles, int* __restrict__ hist) {
    __shared__ int h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int lo = blockIdx.x * kRsTile, hi = min(n, lo + kRsTile);
    for (int i = lo + (int)threadIdx.x; i < hi; i += 256) atomicAdd(&h[(int)((keys[i] >> shift) & 255ull)], 1);
    __syncthreads();
    hist[threadIdx.x * tiles + blockIdx.x] = h[threadIdx.x];
}

__global__ void __launch_bounds__(256) k_rs_scatter(const unsigned long long* __restrict__ kin,
                                                    const int* __restrict__ vin, int n, int shift, int tiles,
                                                    const int* __restrict__ off, unsigned long long* __restrict__ kout,
                                                    int* __restrict__ vout) {
    __shared__ int base[256];
    __shared__ int wcnt[8][256];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    base[tid] = off[tid * tiles + blockIdx.x];
#pragma unroll
    for (int w = 0; w < 8; ++w) wcnt[w][tid] = 0;
    __syncthreads();
    const int lo = blockIdx.x * kRsTile, hi = min(n, lo + kRsTile);
    for (int c = lo; c < hi; c += 256) {
        const int i = c + tid;
        const bool valid = i < hi;
        const unsigned long long k = valid ? kin[i] : 0ull;
        const int v = valid ? vin[i] : 0;
        const int d = valid ? (int)((k >> shift) & 255ull) : 256;
        const unsigned peers = __match_any_sync(0xFFFFFFFFu, d);
        const int rank = __popc(peers & ((1u << lane) - 1u));
        if (valid && rank == 0) wcnt[warp][d] = __popc(peers);
        __syncthreads();
        if (valid) {
            int before = 0;
            for (int w = 0; w < warp; ++w) before += wcnt[w][d];
            const int p = base[d] + before + rank;
            kout[p] = k;
            vout[p] = v;
        }
        __syncthreads();
        int sum = 0;
#pragma unroll
        for (int w = 0; w < 8; ++w) {
            sum += wcnt[w][tid];
            wcnt[w][tid] = 0;
        }
        base[tid] += sum;
        __syncthreads();
    }
}

// ---- incise

// Cells bucketed by their Kahn level (the high half of their drainage key). A cell's receiver sits
// on a strictly higher level, so sweeping the levels from the top down reaches every receiver
// before its donors. Warp-aggregated atomics: lanes sharing a level take one atomic between them.
// Cells per Kahn level, and the cells bucketed by level. A CTA counts its cells per level in shared
// memory and adds each nonzero count to the global one with a single atomic; the scatter does the
// same per chunk of LVL_PER cells per thread, a cell's slot being its rank within the chunk's level
// (a shared-memory atomic) after the chunk's base for that level. Level 0 holds millions of cells,
// so atomics per warp on its cursor were the kernels' cost. Worlds with more than LVL_SMEM levels
// take the per-warp kernels.
constexpr int LVL_SMEM = 4096;
constexpr int LVL_PER = 8;

__device__ __forceinline__ int level_of(const uint8_t* land, const long long* key, size_t i, size_t N, int levels) {
    if (i >= N || !land[i]) return -1;
    const int L = (int)(key[i] >> 32);
    return (L < 0 || L >= levels) ? -1 : L;   // never out of range for a forest's keys
}

__global__ void __launch_bounds__(256) k_level_count_cta(const uint8_t* __restrict__ land,
                                                         const long long* __restrict__ key, size_t N, int levels,
                                                         int* __restrict__ count) {
    __shared__ int hist[LVL_SMEM];
    for (int l = threadIdx.x; l < levels; l += blockDim.x) hist[l] = 0;
    __syncthreads();
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x) {
        const int L = level_of(land, key, i, N, levels);
        if (L >= 0) atomicAdd(&hist[L], 1);
    }
    __syncthreads();
    for (int l = threadIdx.x; l < levels; l += blockDim.x)
        if (hist[l]) atomicAdd(&count[l], hist[l]);
}

__global__ void __launch_bounds__(256) k_level_scatter_cta(const uint8_t* __restrict__ land,
                                                           const long long* __restrict__ key, size_t N, int levels,
                                                           const int* __restrict__ start, int* __restrict__ cursor,
                                                           int* __restrict__ bucket) {
    __shared__ int hist[LVL_SMEM];
    const size_t chunk = (size_t)blockDim.x * LVL_PER;
    for (size_t cb = (size_t)blockIdx.x * chunk; cb < N; cb += (size_t)gridDim.x * chunk) {
        for (int l = threadIdx.x; l < levels; l += blockDim.x) hist[l] = 0;
        __syncthreads();
        int lv[LVL_PER], rank[LVL_PER];
#pragma unroll
        for (int k = 0; k < LVL_PER; ++k) {
            lv[k] = level_of(land, key, cb + (size_t)k * blockDim.x + threadIdx.x, N, levels);
            rank[k] = lv[k] >= 0 ? atomicAdd(&hist[lv[k]], 1) : 0;
        }
        __syncthreads();
        for (int l = threadIdx.x; l < levels; l += blockDim.x)
            if (hist[l]) hist[l] = start[l] + atomicAdd(&cursor[l], hist[l]);
        __syncthreads();
#pragma unroll
        for (int k = 0; k < LVL_PER; ++k)
            if (lv[k] >= 0) bucket[hist[lv[k]] + rank[k]] = (int)(cb + (size_t)k * blockDim.x + threadIdx.x);
        __syncthreads();
    }
}

__global__ void k_level_count(const uint8_t* __restrict__ land, const long long* __restrict__ key, size_t N,
                              int levels, int* __restrict__ count) {
    const unsigned FULL = 0xFFFFFFFFu;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t base = (size_t)blockIdx.x * blockDim.x; base < N; base += stride) {
        const int L = level_of(land, key, base + threadIdx.x, N, levels);
        unsigned group = __match_any_sync(FULL, L);
        if (L >= 0 && (threadIdx.x & 31) == __ffs(group) - 1) atomicAdd(&count[L], __popc(group));
    }
}
__global__ void k_level_scatter(const uint8_t* __restrict__ land, const long long* __restrict__ key, size_t N,
                                int levels, const int* __restrict__ start, int* __restrict__ cursor,
                                int* __restrict__ bucket) {
    const unsigned FULL = 0xFFFFFFFFu;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    const int lane = threadIdx.x & 31;
    for (size_t base = (size_t)blockIdx.x * blockDim.x; base < N; base += stride) {
        const size_t i = base + threadIdx.x;
        const int L = level_of(land, key, i, N, levels);
        unsigned group = __match_any_sync(FULL, L);
        int leader = __ffs(group) - 1;
        int slot = 0;
        if (L >= 0 && lane == leader) slot = atomicAdd(&cursor[L], __popc(group));
        slot = __shfl_sync(FULL, slot, leader);
        if (L >= 0) bucket[start[L] + slot + __popc(group & ((1u << lane) - 1u))] = (int)i;
    }
}

struct InciseDev {
    InciseArgs a;
    int W;
    const uint8_t* land;
    const int32_t* recv;
    const float* ground;
    const float* rel;
    const float* area;
    const float* erod;
    float* surface;
    float* water;
    double* incised_at; // or NULL
    const int* start;   // depth buckets, [levels + 1]
    const int* bucket;
    int levels;
    int* split;         // the highest level left to the whole grid
};

// HydraulicErosion.baseLevel (HydraulicErosion.kt:2380-2390).
__device__ __forceinline__ float base_level(const InciseDev& d, int r) {
    if (!d.land[r]) return d.a.shoreline;
    float w = d.water[r];
    if (!isnan(w)) return fmaxf(d.surface[r], w);
    return d.surface[r];
}

// One cell of HydraulicErosion.incise (HydraulicErosion.kt:2322-2359).
__device__ void incise_cell(const InciseDev& d, int cell) {
    int r = d.recv[cell];
    bool under = __fsub_rn(d.ground[cell], d.rel[cell]) > d.a.pond_depth;
    if (r < 0) {
        if (under) d.water[cell] = __fadd_rn(d.a.shoreline, __fmul_rn(d.ground[cell], d.a.land_range));
        return;
    }
    float base_after = base_level(d, r);
    if (under) {
        float filled_level = __fadd_rn(d.a.shoreline, __fmul_rn(d.ground[cell], d.a.land_range));
        float wr = d.land[r] ? d.water[r] : NAN;
        float downstream = (d.land[r] && !isnan(wr)) ? wr : base_after;
        d.water[cell] = fminf(filled_level, downstream);
    }
    float height = d.surface[cell];
    // GroundSteps.between (MA/GroundSteps.kt:45-53).
    bool same_row = cell / d.W == r / d.W, same_col = cell % d.W == r % d.W;
    float step = (!same_row && !same_col) ? d.a.step_diag : (!same_row ? d.a.step_ns : 1.0f);
    float courant = __fdiv_rn(__fmul_rn(__fmul_rn(d.a.courant_coefficient,
                                                   __fsqrt_rn(__fdiv_rn(d.area[cell], d.a.land_cells))),
                                        d.erod[cell]),
                              step);
    float grades_to = base_after;   // no unresolved relief in this profile
    bool submerged = under && height <= d.water[cell];
    float after;
    if (submerged || (height <= grades_to && d.a.only_above_base)) {
        after = height;
    } else {
        double g = (double)grades_to;
        after = (float)__dadd_rn(g, __ddiv_rn((double)__fsub_rn(height, grades_to), __dadd_rn(1.0, (double)courant)));
    }
    if (after != height) {
        d.surface[cell] = after;
        if (d.incised_at && after < height) d.incised_at[cell] = __dsub_rn((double)height, (double)after);
    }
}

// Levels from the top down. The highest levels are the main stems of the largest rivers, a few
// cells each: while a level fits one pass of a CTA, the first CTA takes it alone, with a CTA barrier
// between levels (its own writes are visible to it); the rest of the grid waits at one grid barrier
// and then sweeps the lower, larger levels with a grid barrier per level.
__global__ void __launch_bounds__(256) k_incise_levels(InciseDev d) {
    cgr::grid_group grid = cgr::this_grid();
    if (blockIdx.x == 0) {
        int level = d.levels - 1;
        for (; level >= 0; --level) {
            const int lo = d.start[level], hi = d.start[level + 1];
            if (hi - lo > (int)blockDim.x) break;
            if (lo + (int)threadIdx.x < hi) incise_cell(d, d.bucket[lo + threadIdx.x]);
            __syncthreads();
        }
        if (threadIdx.x == 0) *d.split = level;
    }
    grid.sync();
    const int stride = gridDim.x * blockDim.x;
    for (int level = *(volatile int*)d.split; level >= 0; --level) {
        const int lo = d.start[level], hi = d.start[level + 1];
        for (int i = lo + blockIdx.x * blockDim.x + threadIdx.x; i < hi; i += stride) incise_cell(d, d.bucket[i]);
        grid.sync();
    }
}

__global__ void k_water_init(float* __restrict__ water, size_t N) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x)
        water[i] = NAN;
}

// ---- spillways

__device__ __forceinline__ unsigned ordered_key(float f) {
    if (f == 0.0f) f = 0.0f;   // -0 and +0 compare equal in the reference
    unsigned b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float from_ordered_key(unsigned u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}

__global__ void k_ponded(const uint8_t* __restrict__ land, const float* __restrict__ filled,
                         const float* __restrict__ rel, float pond, size_t N, uint8_t* __restrict__ ponded) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x)
        ponded[i] = land[i] && __fsub_rn(filled[i], rel[i]) > pond;
}

struct BasinDev {
    int* cells;
    unsigned* floor_key;
    unsigned long long* spill_key;
};

__global__ void k_basin_init(BasinDev b, int count) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    b.cells[i] = 0;
    b.floor_key[i] = 0xFFFFFFFFu;
    b.spill_key[i] = 0xFFFFFFFFFFFFFFFFull;
}

__global__ void k_basin_gather(const int* __restrict__ label, const uint8_t* __restrict__ ponded,
                               const uint8_t* __restrict__ land, const float* __restrict__ rel,
                               const float* __restrict__ filled, const int32_t* __restrict__ recv, size_t N,
                               BasinDev b) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x) {
        int l = label[i];
        if (l < 0) continue;
        atomicAdd(&b.cells[l], 1);
        atomicMin(&b.floor_key[l], ordered_key(rel[i]));
        int r = recv[i];
        if (r >= 0 && land[r] && !ponded[r]) {
            unsigned long long k = ((unsigned long long)ordered_key(filled[r]) << 32) | (unsigned)r;
            atomicMin(&b.spill_key[l], k);
        }
    }
}

// Per basin: the pour point down the outflow's path, the level and the fill depth
// (FlowRouting.kt:637-671).
__global__ void k_basin_finish(BasinDev b, int count, const uint8_t* __restrict__ land,
                               const float* __restrict__ rel, const float* __restrict__ filled,
                               const int32_t* __restrict__ recv, long long N, int* __restrict__ entry,
                               int* __restrict__ spill, float* __restrict__ level, float* __restrict__ floor_out,
                               float* __restrict__ depth) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    float basin_floor = from_ordered_key(b.floor_key[i]);
    unsigned long long sk = b.spill_key[i];
    int sp = -1;
    float spill_level = FLT_MAX;
    if (sk != 0xFFFFFFFFFFFFFFFFull) {
        sp = (int)(sk & 0xFFFFFFFFull);
        spill_level = filled[sp];
    }
    int pour = sp;
    if (sp >= 0) {
        int cell = sp;
        long long steps = 0;
        while (cell >= 0 && land[cell] && filled[cell] > rel[cell] && steps < N) {
            cell = recv[cell];
            ++steps;
        }
        if (cell >= 0 && land[cell]) pour = cell;
    }
    float pour_level = pour >= 0 ? filled[pour] : spill_level;
    entry[i] = sp;
    spill[i] = pour;
    level[i] = pour >= 0 ? pour_level : basin_floor;
    floor_out[i] = basin_floor;
    depth[i] = pour >= 0 ? __fsub_rn(pour_level, basin_floor) : 0.0f;
}

}  // namespace

cg_status tree_walk_dev(cg_ctx* ctx, int W, int H, const uint8_t* d_land, const int32_t* d_recv,
                        const float* d_weights, long long* d_key, int32_t* d_donors, float* d_area, int* h_levels) {
    size_t N = (size_t)W * H;
    cudaStream_t sm = ctx->stream;
    int grid = ctx->num_sms * 8;
    CG_BUF(int32_t, d_pending, ctx, S_DEPTH, N);
    CG_BUF(unsigned long long, d_max, ctx, S_STATS, 1);
    CG_BUF(uint8_t, d_links, ctx, S_LINKS, 2 * N);
    CG_BUF(int, d_sources, ctx, S_SOURCES, N + 1);
    uint8_t* d_down = d_links;
    uint8_t* d_mask = d_links + N;
    int* d_nsrc = d_sources + N;
    CG_CUDA(ctx, cudaMemsetAsync(d_mask, 0, N, sm));
    CG_CUDA(ctx, cudaMemsetAsync(d_nsrc, 0, sizeof(int), sm));
    CG_CUDA(ctx, cudaMemsetAsync(d_max, 0, sizeof(unsigned long long), sm));
    CG_LAUNCH(ctx) k_links<<<grid, 256, 0, sm>>>(d_land, d_recv, W, H, d_down, d_mask);
    CG_LAUNCH(ctx) k_sources<<<grid, 256, 0, sm>>>(d_land, d_mask, N, d_donors, d_pending, d_sources, d_nsrc);
    if (d_area) CG_LAUNCH(ctx) k_area_sea<<<grid, 256, 0, sm>>>(d_land, N, d_area);
    CG_CHECK_LAUNCH(ctx);
    int n_sources = 0;
    CG_CUDA(ctx, cudaMemcpyAsync(&n_sources, d_nsrc, sizeof(int), cudaMemcpyDeviceToHost, sm));
    CG_CUDA(ctx, cudaStreamSynchronize(sm));
    WalkArgs a{W, H, d_down, d_mask, d_pending, d_key, d_weights, d_area, d_sources, d_nsrc, d_max};
    if (n_sources > 0) CG_LAUNCH(ctx) k_walk<<<(n_sources + 63) / 64, 64, 0, sm>>>(a);
    CG_CHECK_LAUNCH(ctx);
    if (h_levels) {
        unsigned long long mk;
        CG_CUDA(ctx, cudaMemcpyAsync(&mk, d_max, sizeof(mk), cudaMemcpyDeviceToHost, sm));
        CG_CUDA(ctx, cudaStreamSynchronize(sm));
        *h_levels = (int)(mk >> 32) + 1;
    }
    return CG_OK;
}

cg_status order_from_keys_dev(cg_ctx* ctx, int W, int H, const uint8_t* d_land, const long long* d_key,
                              int land_cells, int32_t* d_order) {
    size_t N = (size_t)W * H;
    cudaStream_t sm = ctx->stream;
    int grid = ctx->num_sms * 8;
    if (land_cells <= 0) return CG_OK;
    CG_BUF(int, d_flag, ctx, S_SCRATCH0, N);
    CG_BUF(int, d_pos, ctx, S_SCRATCH1, N);
    const int n = land_cells;
    const int tiles = (n + kRsTile - 1) / kRsTile;
    CG_BUF(unsigned long long, d_keys, ctx, S_RS_KEYS, 2 * (size_t)n + 1);
    CG_BUF(int, d_vals, ctx, S_RS_VALS, 2 * (size_t)n);
    CG_BUF(int, d_hist, ctx, S_RS_HIST, 2 * (size_t)tiles * 256);
    unsigned long long* kmax = d_keys + 2 * (size_t)n;
    unsigned long long* ka = d_keys;
    unsigned long long* kb = d_keys + n;
    int* va = d_vals;
    int* vb = d_vals + n;
    int* d_off = d_hist + (size_t)tiles * 256;
    CG_LAUNCH(ctx) k_land_flags<<<grid, 256, 0, sm>>>(d_land, N, d_flag);
    CG_CHECK_LAUNCH(ctx);
    cg_status st = exclusive_scan(ctx, d_flag, d_pos, (int)N, nullptr);
    if (st != CG_OK) return st;
    CG_CUDA(ctx, cudaMemsetAsync(kmax, 0, sizeof(unsigned long long), sm));
    CG_LAUNCH(ctx) k_land_compact_ck<<<grid, 256, 0, sm>>>(d_land, d_pos, d_key, N, ka, va, kmax);
    CG_CHECK_LAUNCH(ctx);
    unsigned long long hmax = 0;
    CG_CUDA(ctx, cudaMemcpyAsync(&hmax, kmax, sizeof(hmax), cudaMemcpyDeviceToHost, sm));
    CG_CUDA(ctx, cudaStreamSynchronize(sm));
    int bits = 0;
    while (bits < 64 && (hmax >> bits) != 0) ++bits;
    for (int shift = 0; shift < bits; shift += 8) {
        CG_LAUNCH(ctx) k_rs_hist<<<tiles, 256, 0, sm>>>(ka, n, shift, tiles, d_hist);
        CG_CHECK_LAUNCH(ctx);
        st = exclusive_scan(ctx, d_hist, d_off, tiles * 256, nullptr);
        if (st != CG_OK) return st;
        CG_LAUNCH(ctx) k_rs_scatter<<<tiles, 256, 0, sm>>>(ka, va, n, shift, tiles, d_off, kb, vb);
        CG_CHECK_LAUNCH(ctx);
        std::swap(ka, kb);
        std::swap(va, vb);
    }
    CG_CUDA(ctx, cudaMemcpyAsync(d_order, va, sizeof(int) * (size_t)n, cudaMemcpyDeviceToDevice, sm));
    return CG_OK;
}

cg_status level_buckets_dev(cg_ctx* ctx, int W, int H, const uint8_t* d_land, const long long* d_key, int levels,
                            int** out_bucket, int** out_start) {
    size_t N = (size_t)W * H;
    cudaStream_t sm = ctx->stream;
    int grid = ctx->num_sms * 8;
    CG_BUF(int, d_bucket, ctx, S_SCRATCH2, N);
    CG_BUF(int, d_cnt, ctx, S_DEPTH, (size_t)levels + 1);
    CG_BUF(int, d_start, ctx, S_CG2, 2 * (size_t)levels + 2);
    int* d_cursor = d_start + levels + 1;
    CG_CUDA(ctx, cudaMemsetAsync(d_cnt, 0, ((size_t)levels + 1) * sizeof(int), sm));
    CG_CUDA(ctx, cudaMemsetAsync(d_cursor, 0, ((size_t)levels + 1) * sizeof(int), sm));
    const bool cta_hist = levels <= LVL_SMEM;
    if (cta_hist) CG_LAUNCH(ctx) k_level_count_cta<<<grid, 256, 0, sm>>>(d_land, d_key, N, levels, d_cnt);
    else CG_LAUNCH(ctx) k_level_count<<<grid, 256, 0, sm>>>(d_land, d_key, N, levels, d_cnt);
    CG_CHECK_LAUNCH(ctx);
    cg_status st = exclusive_scan(ctx, d_cnt, d_start, levels + 1, nullptr);
    if (st != CG_OK) return st;
    if (cta_hist) CG_LAUNCH(ctx) k_level_scatter_cta<<<grid, 256, 0, sm>>>(d_land, d_key, N, levels, d_start, d_cursor, d_bucket);
    else CG_LAUNCH(ctx) k_level_scatter<<<grid, 256, 0, sm>>>(d_land, d_key, N, levels, d_start, d_cursor, d_bucket);
    CG_CHECK_LAUNCH(ctx);
    *out_bucket = d_bucket;
    *out_start = d_start;
    return CG_OK;
}

cg_status incise_dev(cg_ctx* ctx, int W, int H, const uint8_t* d_land, const int32_t* d_recv, const long long* d_key,
                     int levels, const float* d_ground, const float* d_rel, const float* d_area, const float* d_erod,
                     float* d_surface, const InciseArgs& args, double* d_incised_at) {
    size_t N = (size_t)W * H;
    cudaStream_t sm = ctx->stream;
    int grid = ctx->num_sms * 8;
    if (levels <= 0) return CG_OK;
    CG_BUF(int, d_bucket, ctx, S_SCRATCH2, N);
    CG_BUF(float, d_water, ctx, S_WATER, N);
    CG_BUF(int, d_cnt, ctx, S_DEPTH, (size_t)levels + 1);
    CG_BUF(int, d_start, ctx, S_CG2, 2 * (size_t)levels + 2);
    int* d_cursor = d_start + levels + 1;
    CG_CUDA(ctx, cudaMemsetAsync(d_cnt, 0, ((size_t)levels + 1) * sizeof(int), sm));
    CG_CUDA(ctx, cudaMemsetAsync(d_cursor, 0, ((size_t)levels + 1) * sizeof(int), sm));
    const bool cta_hist = levels <= LVL_SMEM;
    if (cta_hist) CG_LAUNCH(ctx) k_level_count_cta<<<grid, 256, 0, sm>>>(d_land, d_key, N, levels, d_cnt);
    else CG_LAUNCH(ctx) k_level_count<<<grid, 256, 0, sm>>>(d_land, d_key, N, levels, d_cnt);
    CG_CHECK_LAUNCH(ctx);
    // The exclusive scan of levels + 1 counts (the last is zero) ends with the total at start[levels].
    cg_status st = exclusive_scan(ctx, d_cnt, d_start, levels + 1, nullptr);
    if (st != CG_OK) return st;
    if (cta_hist) CG_LAUNCH(ctx) k_level_scatter_cta<<<grid, 256, 0, sm>>>(d_land, d_key, N, levels, d_start, d_cursor, d_bucket);
    else CG_LAUNCH(ctx) k_level_scatter<<<grid, 256, 0, sm>>>(d_land, d_key, N, levels, d_start, d_cursor, d_bucket);
    CG_LAUNCH(ctx) k_water_init<<<grid, 256, 0, sm>>>(d_water, N);
    CG_CHECK_LAUNCH(ctx);
    InciseDev d;
    d.a = args;
    d.W = W;
    d.land = d_land;
    d.recv = d_recv;
    d.ground = d_ground;
    d.rel = d_rel;
    d.area = d_area;
    d.erod = d_erod;
    d.surface = d_surface;
    d.water = d_water;
    d.incised_at = d_incised_at;
    d.start = d_start;
    d.bucket = d_bucket;
    d.levels = levels;
    d.split = d_cursor;   // the scatter's cursors are free by now
    int per_sm = 0;
    CG_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_incise_levels, 256, 0));
    if (per_sm < 1) return fail(ctx, CG_CUDA, "incise kernel cannot be resident");
    // Two CTAs per SM: the lower levels still fill the GPU, and a grid barrier over fewer CTAs is shorter.
    int cgrid = ctx->num_sms * (per_sm < 2 ? per_sm : 2);
    void* kargs[] = {&d};
    ctx->launches++;
    CG_CUDA(ctx, cudaLaunchCooperativeKernel((void*)k_incise_levels, cgrid, 256, kargs, 0, sm));
    return CG_OK;
}

cg_status basins_dev(cg_ctx* ctx, int W, int H, const uint8_t* d_land, const float* d_rel, const float* d_filled,
                     const int32_t* d_recv, float pond_depth, int32_t* d_label, BasinArrays* out, int* h_count) {
    size_t N = (size_t)W * H;
    cudaStream_t sm = ctx->stream;
    int grid = ctx->num_sms * 8;
    CG_BUF(uint8_t, d_ponded, ctx, S_FLATS, N);
    CG_BUF(int, d_root, ctx, S_LABEL, N);
    CG_LAUNCH(ctx) k_ponded<<<grid, 256, 0, sm>>>(d_land, d_filled, d_rel, pond_depth, N, d_ponded);
    CG_CHECK_LAUNCH(ctx);
    int count = 0;
    cg_status st = component_labels(ctx, W, H, d_ponded, d_root, d_label, &count);
    if (st != CG_OK) return st;
    *h_count = count;
    *out = BasinArrays{};
    if (count == 0) return CG_OK;
    // One block: spill keys (8 bytes each) first for alignment, then seven 4-byte arrays.
    CG_BUF(unsigned long long, d_b, ctx, S_BASIN, (size_t)count * 5 + 8);
    BasinDev b;
    b.spill_key = d_b;
    b.cells = (int*)(d_b + count);
    b.floor_key = (unsigned*)(b.cells + count);
    out->cells = b.cells;
    out->entry = (int*)(b.floor_key + count);
    out->spill = out->entry + count;
    out->level = (float*)(out->spill + count);
    out->floor_ = out->level + count;
    out->depth = out->floor_ + count;
    CG_LAUNCH(ctx) k_basin_init<<<(count + 255) / 256, 256, 0, sm>>>(b, count);
    CG_LAUNCH(ctx) k_basin_gather<<<grid, 256, 0, sm>>>(d_label, d_ponded, d_land, d_rel, d_filled, d_recv, N, b);
    CG_LAUNCH(ctx) k_basin_finish<<<(count + 255) / 256, 256, 0, sm>>>(b, count, d_land, d_rel, d_filled, d_recv, (long long)N,
                                                        out->entry, out->spill, out->level, out->floor_, out->depth);
    CG_CHECK_LAUNCH(ctx);
    return CG_OK;
}

cg_status spillways_dev(cg_ctx* ctx, int W, int H, const uint8_t* d_land, const float* d_rel, const float* d_filled,
                        const int32_t* d_recv, float pond_depth, int32_t* d_label, cg_basins* hb) {
    cudaStream_t sm = ctx->stream;
    int count = 0;
    BasinArrays d;
    cg_status st = basins_dev(ctx, W, H, d_land, d_rel, d_filled, d_recv, pond_depth, d_label, &d, &count);
    if (st != CG_OK) return st;
    if (hb) {
        hb->count = count;
        hb->largest = -1;
        hb->largest_cells = 0;
        hb->largest_depth = 0.0f;
        hb->deepest = 0.0f;
    }
    if (count == 0 || !hb) return sync(ctx);
    std::vector<int> cells(count), entry(count), spill(count);
    std::vector<float> level(count), flo(count), depth(count);
    CG_CUDA(ctx, cudaMemcpyAsync(cells.data(), d.cells, count * sizeof(int), cudaMemcpyDeviceToHost, sm));
    CG_CUDA(ctx, cudaMemcpyAsync(entry.data(), d.entry, count * sizeof(int), cudaMemcpyDeviceToHost, sm));
    CG_CUDA(ctx, cudaMemcpyAsync(spill.data(), d.spill, count * sizeof(int), cudaMemcpyDeviceToHost, sm));
    CG_CUDA(ctx, cudaMemcpyAsync(level.data(), d.level, count * sizeof(float), cudaMemcpyDeviceToHost, sm));
    CG_CUDA(ctx, cudaMemcpyAsync(flo.data(), d.floor_, count * sizeof(float), cudaMemcpyDeviceToHost, sm));
    CG_CUDA(ctx, cudaMemcpyAsync(depth.data(), d.depth, count * sizeof(float), cudaMemcpyDeviceToHost, sm));
    CG_CUDA(ctx, cudaStreamSynchronize(sm));
    // The running largest / deepest of FlowRouting.kt:664-670, in basin order.
    int largest = -1, largest_cells = 0;
    float largest_depth = 0.0f, deepest = 0.0f;
    for (int i = 0; i < count; ++i) {
        if (cells[i] > largest_cells) {
            largest = i;
            largest_cells = cells[i];
            largest_depth = depth[i];
        }
        if (depth[i] > deepest) deepest = depth[i];
    }
    hb->largest = largest;
    hb->largest_cells = largest_cells;
    hb->largest_depth = largest_depth;
    hb->deepest = deepest;
    int n = count < hb->capacity ? count : hb->capacity;
    for (int i = 0; i < n; ++i) {
        if (hb->spill) hb->spill[i] = spill[i];
        if (hb->entry) hb->entry[i] = entry[i];
        if (hb->level) hb->level[i] = level[i];
        if (hb->floor) hb->floor[i] = flo[i];
        if (hb->cells) hb->cells[i] = cells[i];
    }
    return CG_OK;
}

}  // namespace cg
