// SeaLevelStage.percentileCut on the device (SeaLevelStage.kt:146-200, 579-651), bit-exact.
//
// The reference finds the height with the asked share of the planet's area below it: a 4096-bin
// histogram of cos(latitude) row weights brackets the answer, then the bracketing bin's cells are
// sorted by (height bits, index) and walked until the area below reaches the target. Both sums are
// sequential double sums in the reference, and the answer can flip on their last bit, so both are
// reproduced exactly:
//  - the histogram: per (row, bin) cell counts are exact integers, and each bin's sequential sum
//    over the rows in order is rebuilt by one warp, 32 rows at a time: inside one binade of the
//    running sum every addition adds a whole number of ulps, so a chunk is an integer prefix sum
//    (cg::warp_seq_sum, on the integer pipes); a row whose additions cross a binade or meet a tie is
//    taken alone by cg::seq_repeat_add, which takes `count` equal additions in closed form
//    (csrc/cg_fpemu.h);
//  - the bracket: its cells are sorted on the device and walked in the reference's order by one
//    warp with the same chunking.
// min, max, the bin of a cell and the land/relative split are elementwise or exact reductions.
#include <climits>
#include <cmath>
#include <vector>

#include "cg_common.cuh"
#include "cg_fpemu.h"
#include "cg_internal.h"

namespace cg {

namespace {

constexpr int BINS = 4096;   // SeaLevelStage.HISTOGRAM_BINS

struct CutState {
    unsigned lo_key, hi_key;   // ordered float keys for atomicMin / atomicMax
    float lowest, highest, per;
    int degenerate;            // 1: the answer is `lowest` (flat field or nothing below)
    int bracket_bin;
    int count;                 // cells in the bracket bin
    double below_bracket;
    float todays;              // the percentile's height, before the lowstand
    int land_cells;
};

__device__ __forceinline__ unsigned ordered_key(float f) {
    unsigned b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float from_ordered_key(unsigned u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}

// SeaLevelStage.sortableBits (SeaLevelStage.kt:648-651).
__device__ __forceinline__ int sortable_bits(float v) {
    int bits = __float_as_int(v);
    return bits < 0 ? (bits ^ 0x7FFFFFFF) : bits;
}

__device__ __forceinline__ int bin_of(float v, float lowest, float per) {
    float x = __fmul_rn(__fsub_rn(v, lowest), per);
    int b = (int)x;   // Float.toInt(): truncation
    return b < 0 ? 0 : (b > BINS - 1 ? BINS - 1 : b);
}

__global__ void k_cut_init(CutState* s) {
    s->lo_key = 0xFFFFFFFFu;
    s->hi_key = 0u;
    s->count = 0;
    s->land_cells = 0;
    s->degenerate = 0;
}

__global__ void k_minmax(const float* __restrict__ h, size_t N, CutState* s) {
    unsigned lo = 0xFFFFFFFFu, hi = 0u;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x) {
        unsigned k = ordered_key(h[i]);
        lo = min(lo, k);
        hi = max(hi, k);
    }
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xFFFFFFFFu, lo, o));
        hi = max(hi, __shfl_xor_sync(0xFFFFFFFFu, hi, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(&s->lo_key, lo);
        atomicMax(&s->hi_key, hi);
    }
}

__global__ void k_cut_prepare(CutState* s, double target) {
    float lo = from_ordered_key(s->lo_key), hi = from_ordered_key(s->hi_key);
    s->lowest = lo;
    s->highest = hi;
    if (__fsub_rn(hi, lo) <= 0.0f || target <= 0.0) {
        s->degenerate = 1;
        s->todays = lo;
        s->per = 0.0f;
    } else {
        s->per = __fdiv_rn((float)(BINS - 1), __fsub_rn(hi, lo));
    }
}

// One CTA per row: exact cell counts of every bin in that row.
__global__ void __launch_bounds__(512) k_row_counts(const float* __restrict__ h, int W, const CutState* s,
                                                    unsigned* __restrict__ counts) {
    __shared__ unsigned sh[BINS];
    if (s->degenerate) return;
    const float lo = s->lowest, per = s->per;
    for (int b = threadIdx.x; b < BINS; b += blockDim.x) sh[b] = 0u;
    __syncthreads();
    const float* rowp = h + (size_t)blockIdx.x * W;
    for (int c = threadIdx.x; c < W; c += blockDim.x) atomicAdd(&sh[bin_of(rowp[c], lo, per)], 1u);
    __syncthreads();
    unsigned* out = counts + (size_t)blockIdx.x * BINS;
    for (int b = threadIdx.x; b < BINS; b += blockDim.x) out[b] = sh[b];
}

// One warp per bin: the reference's sequential sum `histogram[bin] += rowWeights[row]`, in cell
// order, replayed exactly, 32 rows at a time (cg::warp_seq_sum).
__global__ void k_bin_sums(const unsigned* __restrict__ counts, const double* __restrict__ w, int H,
                           const CutState* s, double* __restrict__ hist) {
    const int b = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (b >= BINS || s->degenerate) return;
    double acc = 0.0;
    for (int base = 0; base < H; base += 32) {
        int r = base + lane;
        unsigned c = r < H ? counts[(size_t)r * BINS + b] : 0u;
        double wr = r < H ? w[r] : 0.0;
        if (!__any_sync(0xFFFFFFFFu, c != 0u)) continue;
        double before;
        acc = warp_seq_sum(acc, wr, (int64_t)c, &before);
    }
    if (lane == 0) hist[b] = acc;
}

// SeaLevelStage.kt:614-622: the first bin that brings the weight below up to the target. The
// histogram is staged in shared memory by the CTA; one thread then takes the reference's sums.
__global__ void __launch_bounds__(256) k_bracket_bin(const double* __restrict__ hist, double target, CutState* s) {
    __shared__ double sh[BINS];
    if (s->degenerate) return;
    for (int b = threadIdx.x; b < BINS; b += blockDim.x) sh[b] = hist[b];
    __syncthreads();
    if (threadIdx.x != 0) return;
    double below = 0.0;
    int bracket = BINS - 1;
    for (int b = 0; b < BINS; ++b) {
        if (below + sh[b] >= target) {
            bracket = b;
            break;
        }
        below += sh[b];
    }
    s->bracket_bin = bracket;
    s->below_bracket = below;
}

__global__ void k_bracket_collect(const float* __restrict__ h, size_t N, CutState* s, long long* __restrict__ keys) {
    if (s->degenerate) return;
    const unsigned FULL = 0xFFFFFFFFu;
    const float lo = s->lowest, per = s->per;
    const int bracket = s->bracket_bin;
    const int lane = threadIdx.x & 31;
    // Whole warps step together, so the bracket's cells of a warp take one atomic (the list's order
    // does not matter: it is sorted next).
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t base = (size_t)blockIdx.x * blockDim.x; base < N; base += stride) {
        const size_t i = base + threadIdx.x;
        const float v = i < N ? h[i] : 0.0f;
        const bool in = i < N && bin_of(v, lo, per) == bracket;
        const unsigned m = __ballot_sync(FULL, in);
        if (!m) continue;
        int slot = 0;
        if (lane == __ffs(m) - 1) slot = atomicAdd(&s->count, __popc(m));
        slot = __shfl_sync(FULL, slot, __ffs(m) - 1) + __popc(m & ((1u << lane) - 1u));
        if (in) keys[slot] = (long long)(((unsigned long long)(long long)sortable_bits(v) << 32) | (unsigned long long)i);
    }
}

// Bitonic sort of up to 16384 keys in one CTA's shared memory (padding with the largest key).
constexpr int SMALL_SORT = 16384;
__global__ void __launch_bounds__(1024) k_sort_small(long long* keys, const CutState* s) {
    extern __shared__ long long sk[];
    int n = s->count;
    if (s->degenerate || n <= 1 || n > SMALL_SORT) return;
    int P2 = 1;
    while (P2 < n) P2 <<= 1;
    for (int i = threadIdx.x; i < P2; i += blockDim.x) sk[i] = i < n ? keys[i] : LLONG_MAX;
    __syncthreads();
    for (int k = 2; k <= P2; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < P2; i += blockDim.x) {
                int l = i ^ j;
                if (l > i) {
                    bool up = (i & k) == 0;
                    long long a = sk[i], b = sk[l];
                    if ((a > b) == up) {
                        sk[i] = b;
                        sk[l] = a;
                    }
                }
            }
            __syncthreads();
        }
    for (int i = threadIdx.x; i < n; i += blockDim.x) keys[i] = sk[i];
}

// One compare-exchange stage of a global bitonic sort over P2 slots, padded with the largest key.
__global__ void k_sort_stage(long long* keys, int P2, int k, int j) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P2; i += gridDim.x * blockDim.x) {
        int l = i ^ j;
        if (l <= i) continue;
        long long a = keys[i], b = keys[l];
        bool up = (i & k) == 0;
        if ((a > b) == up) {
            keys[i] = b;
            keys[l] = a;
        }
    }
}

// The bitonic network over P2 keys with its short strides in shared memory: a CTA holds a chunk of
// SORT_CH keys and takes every compare-exchange whose stride is below SORT_CH (directions from the
// keys' global positions, as in k_sort_stage); only the longer strides go through global memory,
// one launch each.
constexpr int SORT_CH = 4096;

__device__ __forceinline__ void chunk_steps(long long* sk, int base, int k, int jmax) {
    for (int j = jmax; j > 0; j >>= 1) {
        for (int p = threadIdx.x; p < SORT_CH / 2; p += blockDim.x) {
            const int i = (p & (j - 1)) | ((p & ~(j - 1)) << 1);
            const int l = i | j;
            const bool up = ((base + i) & k) == 0;
            const long long a = sk[i], b = sk[l];
            if ((a > b) == up) {
                sk[i] = b;
                sk[l] = a;
            }
        }
        __syncthreads();
    }
}

// Every stage k <= SORT_CH, whole, per chunk (merge = 0); or the strides below SORT_CH of stage k.
__global__ void __launch_bounds__(1024) k_sort_chunk(long long* keys, int merge) {
    __shared__ long long sk[SORT_CH];
    const int base = blockIdx.x * SORT_CH;
    for (int i = threadIdx.x; i < SORT_CH; i += blockDim.x) sk[i] = keys[base + i];
    __syncthreads();
    if (merge == 0) {
        for (int k = 2; k <= SORT_CH; k <<= 1) chunk_steps(sk, base, k, k >> 1);
    } else {
        chunk_steps(sk, base, merge, SORT_CH / 2);
    }
    for (int i = threadIdx.x; i < SORT_CH; i += blockDim.x) keys[base + i] = sk[i];
}

__global__ void k_pad(long long* keys, int n, int P2) {
    for (int i = n + blockIdx.x * blockDim.x + threadIdx.x; i < P2; i += gridDim.x * blockDim.x) keys[i] = LLONG_MAX;
}

// SeaLevelStage.kt:636-644: walk the sorted bracket until the area below reaches the target.
//
// The walk's sum is sequential, but it rarely leaves its binade: then every entry adds a whole
// number of units in the last place, d_i = rne(w_i / U), and the sums before the entries are an
// integer prefix scan. One CTA takes the bracket CHUNK entries at a time: per entry d_i and whether
// it is clean (no tie at half a unit, the step stays in the binade); a block scan of the d_i; the
// answer is the first entry whose sum before it reaches the target, provided every earlier entry of
// the chunk is clean. From the first entry that is not, warp 0 replays the rest of the chunk exactly
// (32 entries at a time with cg::warp_seq_sum).
constexpr int WALK_THREADS = 1024;
constexpr int WALK_PER = 8;
constexpr int WALK_CHUNK = WALK_THREADS * WALK_PER;

// Warp 0's exact replay of entries [from, to) starting from `below`. Returns true with *cell the
// answer's cell when the sum before an entry reaches the target; otherwise *below is the sum after
// entry to - 1.
__device__ bool walk_replay(const long long* __restrict__ keys, const double* __restrict__ w, int W, double target,
                            int from, int to, double* below_io, int* cell_out) {
    const unsigned FULL = 0xFFFFFFFFu;
    const int lane = threadIdx.x & 31;
    double below = *below_io;
    for (int base = from; base < to; base += 32) {
        const int i = base + lane;
        const int cell = i < to ? (int)(keys[i] & 0xFFFFFFFFLL) : -1;
        const double wi = i < to ? w[pdiv(cell, W)] : 0.0;
        double before;
        const double after = warp_seq_sum(below, wi, i < to ? 1 : 0, &before);
        const unsigned hit = __ballot_sync(FULL, i < to && before >= target);
        if (hit) {
            *cell_out = __shfl_sync(FULL, cell, __ffs(hit) - 1);
            return true;
        }
        below = after;
    }
    *below_io = below;
    return false;
}

__global__ void __launch_bounds__(WALK_THREADS) k_bracket_walk(const float* __restrict__ h,
                                                               const long long* __restrict__ keys,
                                                               const double* __restrict__ w, int W, double target,
                                                               CutState* s) {
    const int64_t TOP = (int64_t)1 << 53;
    __shared__ long long s_warp[WALK_THREADS / 32];
    __shared__ int s_hit, s_unclean, s_done;
    __shared__ double s_below;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (s->degenerate) return;
    const int n = s->count;
    if (n == 0) {
        if (tid == 0) s->todays = s->highest;
        return;
    }
    double below = s->below_bracket;
    for (int base = 0; base < n; base += WALK_CHUNK) {
        const int end = min(n, base + WALK_CHUNK);
        if (tid == 0) {
            s_hit = INT_MAX;
            s_unclean = below > 0.0 ? INT_MAX : base;   // a zero sum has no binade: replay from the start
        }
        int e = 0;
        double U = 1.0;
        int64_t m = 0;
        if (below > 0.0) {
            e = ilogb(below);
            U = ldexp(1.0, e - 52);
            m = (int64_t)(below / U);
        }
        int64_t d[WALK_PER], q[WALK_PER];
        bool clean[WALK_PER];
        int64_t mine = 0;
        const int first = base + tid * WALK_PER;
#pragma unroll
        for (int k = 0; k < WALK_PER; ++k) {
            const int i = first + k;
            d[k] = 0;
            q[k] = 0;
            clean[k] = true;
            if (i < end) {
                const int cell = (int)(keys[i] & 0xFFFFFFFFLL);
                const double x = ldexp(w[pdiv(cell, W)], 52 - e);   // w / U, exact
                if (!(x < 9.0e15)) {
                    clean[k] = false;
                } else {
                    q[k] = (int64_t)x;
                    const double f = x - (double)q[k];
                    clean[k] = f != 0.5;
                    d[k] = q[k] + (f > 0.5 ? 1 : 0);
                }
            }
            mine += d[k];
        }
        // Exclusive block scan of the per-thread totals.
        int64_t incl = mine;
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= o) incl += t;
        }
        if (lane == 31) s_warp[warp] = incl;
        __syncthreads();
        if (warp == 0) {
            int64_t v = s_warp[lane], vi = v;
            for (int o = 1; o < 32; o <<= 1) {
                const int64_t t = __shfl_up_sync(0xFFFFFFFFu, vi, o);
                if (lane >= o) vi += t;
            }
            s_warp[lane] = vi - v;   // exclusive over warps
        }
        __syncthreads();
        int64_t run = m + s_warp[warp] + (incl - mine);   // the sum before this thread's first entry, in U
        int hit = INT_MAX, unclean = INT_MAX;
#pragma unroll
        for (int k = 0; k < WALK_PER; ++k) {
            const int i = first + k;
            if (i >= end) break;
            if (hit == INT_MAX && (double)run * U >= target) hit = i;
            if (unclean == INT_MAX && (!clean[k] || run + q[k] > TOP - 1)) unclean = i;
            run += d[k];
        }
        if (hit != INT_MAX) atomicMin(&s_hit, hit);
        if (unclean != INT_MAX) atomicMin(&s_unclean, unclean);
        __syncthreads();
        const int h_at = s_hit, u_at = s_unclean;
        if (h_at != INT_MAX && h_at <= u_at) {   // every entry before the answer added whole units inside the binade
            if (tid == 0) s->todays = h[(int)(keys[h_at] & 0xFFFFFFFFLL)];
            return;
        }
        // The sum before entry u_at (exact), from the thread that owns it; for a chunk that was clean
        // throughout, the sum after its last entry.
        if (tid == 0) s_done = 0;
        __syncthreads();
        {
            int64_t r2 = m + s_warp[warp] + (incl - mine);
#pragma unroll
            for (int k = 0; k < WALK_PER; ++k) {
                const int i = first + k;
                if (i == u_at) s_below = (double)r2 * U;
                if (i >= end) break;
                r2 += d[k];
                if (u_at == INT_MAX && i == end - 1) s_below = (double)r2 * U;
            }
        }
        __syncthreads();
        below = s_below;
        if (u_at != INT_MAX) {
            if (warp == 0) {
                double b = below;
                int cell;
                if (walk_replay(keys, w, W, target, u_at, end, &b, &cell)) {
                    if (lane == 0) {
                        s->todays = h[cell];
                        s_done = 1;
                    }
                } else if (lane == 0) {
                    s_below = b;
                }
            }
            __syncthreads();
            if (s_done) return;
            below = s_below;
        }
        __syncthreads();
    }
    if (tid == 0) s->todays = h[(int)(keys[n - 1] & 0xFFFFFFFFLL)];
}

// SeaLevelStage.landAndWaterAt (SeaLevelStage.kt:175-200).
__global__ void k_land_and_water(const float* __restrict__ h, size_t N, CutState* s, float lowstand,
                                 float land_half, float sea_half, uint8_t* __restrict__ land,
                                 float* __restrict__ rel) {
    const float shore = __fsub_rn(s->todays, lowstand);
    int count = 0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x) {
        float g = h[i];
        float d = __fsub_rn(g, shore);
        if (g >= shore) {
            land[i] = 1;
            rel[i] = __fdiv_rn(d, land_half);
            ++count;
        } else {
            land[i] = 0;
            rel[i] = __fdiv_rn(d, sea_half);
        }
    }
    for (int o = 16; o > 0; o >>= 1) count += __shfl_xor_sync(0xFFFFFFFFu, count, o);
    if ((threadIdx.x & 31) == 0 && count) atomicAdd(&s->land_cells, count);
}

}  // namespace

cg_status row_weights_dev(cg_ctx* ctx, int W, int H, const double** d_weights, double* total) {
    CG_BUF(double, d_w, ctx, S_ROWW, H);
    if (ctx->rw_w != W || ctx->rw_h != H) {
        // shorelineForFraction (SeaLevelStage.kt:580-584): a per-grid constant table, built once.
        std::vector<double> w(H);
        const double PI = 3.141592653589793;
        for (int row = 0; row < H; ++row) w[row] = std::cos(PI / 2 - (row + 0.5) / H * PI);
        double t = 0.0;
        for (int row = 0; row < H; ++row) t += w[row] * W;
        CG_CUDA(ctx, cudaMemcpyAsync(d_w, w.data(), sizeof(double) * H, cudaMemcpyHostToDevice, ctx->stream));
        CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        ctx->rw_w = W;
        ctx->rw_h = H;
        ctx->rw_total = t;
    }
    *d_weights = d_w;
    *total = ctx->rw_total;
    return CG_OK;
}

cg_status percentile_cut_dev(cg_ctx* ctx, int W, int H, const float* d_h, float sea_level, float land_half,
                             float sea_half, float lowstand_share, uint8_t* d_land, float* d_rel, float* h_shoreline,
                             int* h_land_cells) {
    size_t N = (size_t)W * H;
    const double* d_w;
    double total;
    cg_status st = row_weights_dev(ctx, W, H, &d_w, &total);
    if (st != CG_OK) return st;
    float submerged = sea_level < 0.0f ? 0.0f : (sea_level > 1.0f ? 1.0f : sea_level);
    double target = (double)submerged * total;
    CG_BUF(CutState, d_s, ctx, S_SMALL, 1);
    CG_BUF(unsigned, d_counts, ctx, S_HIST, (size_t)H * BINS);
    CG_BUF(double, d_hist, ctx, S_SCRATCH4, BINS);
    CG_BUF(long long, d_keys, ctx, S_BRACKET, N);
    cudaStream_t sm = ctx->stream;
    int grid = ctx->num_sms * 8;
    CG_LAUNCH(ctx) k_cut_init<<<1, 1, 0, sm>>>(d_s);
    CG_LAUNCH(ctx) k_minmax<<<grid, 256, 0, sm>>>(d_h, N, d_s);
    CG_LAUNCH(ctx) k_cut_prepare<<<1, 1, 0, sm>>>(d_s, target);
    CG_LAUNCH(ctx) k_row_counts<<<H, 512, 0, sm>>>(d_h, W, d_s, d_counts);
    CG_LAUNCH(ctx) k_bin_sums<<<BINS * 32 / 256, 256, 0, sm>>>(d_counts, d_w, H, d_s, d_hist);
    CG_LAUNCH(ctx) k_bracket_bin<<<1, 256, 0, sm>>>(d_hist, target, d_s);
    CG_LAUNCH(ctx) k_bracket_collect<<<grid, 256, 0, sm>>>(d_h, N, d_s, d_keys);
    CG_CHECK_LAUNCH(ctx);
    CutState hs;
    CG_CUDA(ctx, cudaMemcpyAsync(&hs, d_s, sizeof(hs), cudaMemcpyDeviceToHost, sm));
    CG_CUDA(ctx, cudaStreamSynchronize(sm));
    if (!hs.degenerate && hs.count > 1) {
        if (hs.count <= SMALL_SORT) {
            // Set on every call (it is cheap): a flag kept across calls would be shared by every
            // context and device of the process.
            CG_CUDA(ctx, cudaFuncSetAttribute(k_sort_small, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)(SMALL_SORT * sizeof(long long))));
            int P2 = 1;
            while (P2 < hs.count) P2 <<= 1;
            CG_LAUNCH(ctx) k_sort_small<<<1, 1024, P2 * sizeof(long long), sm>>>(d_keys, d_s);
        } else {
            int P2 = 1;
            while (P2 < hs.count) P2 <<= 1;
            int blocks = (P2 / 2 + 255) / 256;
            if (blocks > grid) blocks = grid;
            CG_LAUNCH(ctx) k_pad<<<blocks, 256, 0, sm>>>(d_keys, hs.count, P2);
            // P2 > SMALL_SORT >= SORT_CH: whole chunks of SORT_CH keys.
            CG_LAUNCH(ctx) k_sort_chunk<<<P2 / SORT_CH, 1024, 0, sm>>>(d_keys, 0);
            for (int k = 2 * SORT_CH; k <= P2; k <<= 1) {
                for (int j = k >> 1; j >= SORT_CH; j >>= 1)
                    CG_LAUNCH(ctx) k_sort_stage<<<blocks, 256, 0, sm>>>(d_keys, P2, k, j);
                CG_LAUNCH(ctx) k_sort_chunk<<<P2 / SORT_CH, 1024, 0, sm>>>(d_keys, k);
            }
        }
        CG_CHECK_LAUNCH(ctx);
    }
    CG_LAUNCH(ctx) k_bracket_walk<<<1, WALK_THREADS, 0, sm>>>(d_h, d_keys, d_w, W, target, d_s);
    CG_LAUNCH(ctx) k_land_and_water<<<grid, 256, 0, sm>>>(d_h, N, d_s, lowstand_share, land_half, sea_half, d_land, d_rel);
    CG_CHECK_LAUNCH(ctx);
    CG_CUDA(ctx, cudaMemcpyAsync(&hs, d_s, sizeof(hs), cudaMemcpyDeviceToHost, sm));
    CG_CUDA(ctx, cudaStreamSynchronize(sm));
    *h_shoreline = hs.todays - lowstand_share;
    *h_land_cells = hs.land_cells;
    return CG_OK;
}

}  // namespace cg
