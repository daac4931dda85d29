// The reference's sequential double sums of float fields (`var s = 0.0; for (c in cells) s += f[c]`:
// the rain and cover means of normaliseOverLand / shieldingOverLand, HydraulicErosion.kt:476-486,
// 557-567, and the flexure's load mean, Isostasy.kt:337-339), bit for bit, without a serial chain of
// double additions.
//
// Each addition rounds, so the sum depends on the order. But while the running sum s stays inside one
// binade [2^e, 2^(e+1)) (one sign), s is m u with m an integer in [2^52, 2^53) and u = 2^(e-52), and
// fl(s + x) = (m + r) u where r is x / u rounded to an integer, to nearest, ties to even: the tie's
// choice depends on the parity of m and nothing else, and a tie always leaves m even. So a run of
// additions inside a binade is an integer walk whose only state is m's parity: a block of values
// reduces, for each entering parity, to its total step, its lowest and highest partial steps (which
// say whether the walk stays inside the binade) and its leaving parity. Blocks are reduced in parallel
// under the binade an estimate of the running sum gives them; one CTA then walks the blocks, applying
// each block's reduction where the running sum is in the binade it was reduced for and its walk stays
// inside, and otherwise taking the block in pieces of 1024 values reduced on the spot for the binade
// the sum is actually in, with the serial double additions only for a piece inside which the sum
// crosses a binade (or is zero, as at the start).
#include <cstdint>

#include "cg_common.cuh"
#include "cg_internal.h"

namespace cg {
namespace {

constexpr int kSSThreads = 1024;
constexpr int kSSPer = 8;                        // values per thread in the parallel reduction
constexpr int kSSBlock = kSSThreads * kSSPer;    // values per block
constexpr long long kM0 = 1LL << 52, kM1 = 1LL << 53;
constexpr long long kBig = 1LL << 58;            // a partial step this large leaves any binade: give up

// The values summed: float fields (widened exactly), or double terms already in summation order.
template <typename T>
struct SumIn {
    const T* x;
    const uint8_t* mask;   // may be null: every value (float fields only)
    int mode;              // 0: x, 1: 1 - 0.5 x (the cover's shielding factor; float fields only)
    size_t n;
};

// A run of additions inside one binade, for each parity of m entering it.
struct Walk {
    long long step[2], lo[2], hi[2];   // total step; lowest and highest partial step (lo > hi: no values)
    int out[2];                        // parity of m leaving
    int fail;                          // a value the integer walk cannot hold (it leaves the binade)
};

__device__ __forceinline__ Walk walk_identity() {
    Walk w;
    for (int q = 0; q < 2; ++q) {
        w.step[q] = 0;
        w.lo[q] = kBig;
        w.hi[q] = -kBig;
        w.out[q] = q;
    }
    w.fail = 0;
    return w;
}

// a then b.
__device__ __forceinline__ Walk walk_then(const Walk& a, const Walk& b) {
    Walk w;
    for (int q = 0; q < 2; ++q) {
        const int mid = a.out[q];
        w.step[q] = a.step[q] + b.step[mid];
        const long long blo = a.step[q] + b.lo[mid], bhi = a.step[q] + b.hi[mid];
        w.lo[q] = b.lo[mid] > b.hi[mid] ? a.lo[q] : (a.lo[q] < blo ? a.lo[q] : blo);
        w.hi[q] = b.lo[mid] > b.hi[mid] ? a.hi[q] : (a.hi[q] > bhi ? a.hi[q] : bhi);
        w.out[q] = b.out[mid];
    }
    w.fail = a.fail | b.fail;
    if (w.step[0] > kBig || w.step[0] < -kBig || w.step[1] > kBig || w.step[1] < -kBig) w.fail = 1;
    return w;
}

__device__ __forceinline__ bool value_at(const SumIn<float>& in, size_t i, float* v) {
    if (i >= in.n) return false;
    if (in.mask && !in.mask[i]) return false;
    const float x = in.x[i];
    *v = in.mode == 1 ? __fsub_rn(1.0f, __fmul_rn(0.5f, x)) : x;
    return true;
}

__device__ __forceinline__ bool value_at(const SumIn<double>& in, size_t i, double* v) {
    if (i >= in.n) return false;
    *v = in.x[i];
    return true;
}

// One value's step in the binade with exponent field ef (u = 2^(ef - 1075)), for a sum of sign `neg`:
// the step r when it is not a tie, else the tie's floor f (r = f + ((parity + f) & 1)). An absent value
// (a masked cell) adds nothing, as the reference skips it; +0 and -0 add nothing to a nonzero sum.
struct Step {
    long long r;
    int tie, fail;
};

__device__ __forceinline__ Step step_of(float v, int ef, int neg) {
    Step s{0, 0, 0};
    const uint32_t b = __float_as_uint(v);
    const int fe = (int)((b >> 23) & 0xFF);
    if (fe == 0xFF) {
        s.fail = 1;
        return s;
    }
    long long M = (long long)(b & 0x7FFFFF);
    if (fe != 0) M |= 1LL << 23;
    if (M == 0) return s;
    const bool negative = ((b >> 31) != 0) != (neg != 0);   // y's sign: x's, flipped for a negative sum
    // y = M 2^k with k = (max(fe, 1) - 150) - (ef - 1075)
    const int k = (fe == 0 ? 1 : fe) - 150 - ef + 1075;
    if (k >= 0) {
        if (k > 29) {
            s.fail = 1;
            return s;
        }
        s.r = negative ? -(M << k) : (M << k);
        return s;
    }
    const int sh = -k;
    if (sh >= 40) return s;   // |y| < 2^-16: rounds to 0
    const long long a = M >> sh, frac = M & ((1LL << sh) - 1), half = 1LL << (sh - 1);
    if (frac == half) {
        s.tie = 1;
        s.r = negative ? -(a + 1) : a;   // floor(y)
    } else {
        const long long r = a + (frac > half ? 1 : 0);
        s.r = negative ? -r : r;
    }
    return s;
}

// The same for a double value: y = M 2^k with M < 2^53 and k = max(fe, 1) - ef. A value of 2^58 u or
// more, or NaN or infinity, is left to the serial additions; below u / 4 it adds nothing.
__device__ __forceinline__ Step step_of(double v, int ef, int neg) {
    Step s{0, 0, 0};
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const int fe = (int)((b >> 52) & 0x7FF);
    if (fe == 0x7FF) {
        s.fail = 1;
        return s;
    }
    long long M = (long long)(b & ((1ULL << 52) - 1));
    if (fe != 0) M |= 1LL << 52;
    if (M == 0) return s;
    const bool negative = ((b >> 63) != 0) != (neg != 0);
    const int k = (fe == 0 ? 1 : fe) - ef;
    if (k >= 0) {
        if (k > 5) {
            s.fail = 1;
            return s;
        }
        s.r = negative ? -(M << k) : (M << k);
        return s;
    }
    const int sh = -k;
    if (sh >= 55) return s;   // |y| < 2^-2: rounds to 0
    const long long a = M >> sh, frac = M & ((1LL << sh) - 1), half = 1LL << (sh - 1);
    if (frac == half) {
        s.tie = 1;
        s.r = negative ? -(a + 1) : a;
    } else {
        const long long r = a + (frac > half ? 1 : 0);
        s.r = negative ? -r : r;
    }
    return s;
}

// The walk of a run of values in order, for both entering parities.
struct LocalWalk {
    Walk w;
    __device__ void init() { w = walk_identity(); }
    __device__ void add(const Step& st) {
        if (st.fail) w.fail = 1;
        for (int q = 0; q < 2; ++q) {
            const int p = w.out[q];
            const long long r = st.tie ? st.r + ((p + (int)(st.r & 1)) & 1) : st.r;
            w.step[q] += r;
            if (w.step[q] < w.lo[q]) w.lo[q] = w.step[q];
            if (w.step[q] > w.hi[q]) w.hi[q] = w.step[q];
            w.out[q] = st.tie ? 0 : (p ^ (int)(r & 1));
            if (w.step[q] > kBig || w.step[q] < -kBig) w.fail = 1;
        }
    }
};

__device__ __forceinline__ Walk shfl_walk(const Walk& w, int from) {
    Walk o;
    for (int q = 0; q < 2; ++q) {
        o.step[q] = __shfl_sync(0xFFFFFFFFu, w.step[q], from);
        o.lo[q] = __shfl_sync(0xFFFFFFFFu, w.lo[q], from);
        o.hi[q] = __shfl_sync(0xFFFFFFFFu, w.hi[q], from);
        o.out[q] = __shfl_sync(0xFFFFFFFFu, w.out[q], from);
    }
    o.fail = __shfl_sync(0xFFFFFFFFu, w.fail, from);
    return o;
}

// The CTA's threads' walks composed in thread order; every thread calls it, thread 0 gets the result.
__device__ Walk cta_walk(const Walk& mine, Walk* sh_warps) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    Walk w = mine;
    // Within a warp: lane i takes lanes i .. i + 2 off - 1 (in order), a tree over the lanes.
    for (int off = 1; off < 32; off <<= 1) {
        const Walk o = shfl_walk(w, (lane + off) & 31);
        if ((lane & (2 * off - 1)) == 0 && lane + off < 32) w = walk_then(w, o);
    }
    if (lane == 0) sh_warps[warp] = w;
    __syncthreads();
    Walk total = walk_identity();
    if (threadIdx.x == 0)
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) total = walk_then(total, sh_warps[i]);
    __syncthreads();
    return total;
}

// A cheap estimate of each block's sum (any order): it only picks the binade each block is reduced for.
template <typename T>
__global__ void __launch_bounds__(kSSThreads) k_ss_estimate(SumIn<T> in, double* __restrict__ est) {
    __shared__ double part[kSSThreads / 32];
    const size_t base = (size_t)blockIdx.x * kSSBlock;
    double s = 0.0;
    for (int t = 0; t < kSSPer; ++t) {
        T v;
        if (value_at(in, base + (size_t)t * kSSThreads + threadIdx.x, &v)) s += (double)v;
    }
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xFFFFFFFFu, s, off);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int i = 0; i < kSSThreads / 32; ++i) t += part[i];
        est[blockIdx.x] = t;
    }
}

// The binade and sign each block is expected to begin in: exponent field | sign << 11, or -1 (zero).
__global__ void __launch_bounds__(1024) k_ss_spec(const double* __restrict__ est, int blocks, int* __restrict__ spec) {
    __shared__ double sh[1024];
    double carry = 0.0;
    for (int base = 0; base < blocks; base += 1024) {
        const int i = base + (int)threadIdx.x;
        const double v = i < blocks ? est[i] : 0.0;
        sh[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < 1024; o <<= 1) {
            const double t = threadIdx.x >= (unsigned)o ? sh[threadIdx.x - o] : 0.0;
            __syncthreads();
            sh[threadIdx.x] += t;
            __syncthreads();
        }
        if (i < blocks) {
            const double start = carry + sh[threadIdx.x] - v;
            const unsigned long long bits = (unsigned long long)__double_as_longlong(start);
            const int ef = (int)((bits >> 52) & 0x7FF);
            spec[i] = (start == 0.0 || ef == 0 || ef == 0x7FF) ? -1 : (ef | (int)((bits >> 63) << 11));
        }
        const double chunk = sh[1023];
        __syncthreads();
        carry += chunk;
    }
}

// Each block's walk under the binade it is expected to begin in. A thread's values are consecutive.
template <typename T>
__global__ void __launch_bounds__(kSSThreads) k_ss_walks(SumIn<T> in, const int* __restrict__ spec,
                                                        Walk* __restrict__ walks) {
    __shared__ Walk sh_warps[kSSThreads / 32];
    const int sp = spec[blockIdx.x];
    LocalWalk lw;
    lw.init();
    if (sp >= 0) {
        const size_t base = (size_t)blockIdx.x * kSSBlock + (size_t)threadIdx.x * kSSPer;
        for (int t = 0; t < kSSPer; ++t) {
            T v;
            if (value_at(in, base + t, &v)) lw.add(step_of(v, sp & 0x7FF, sp >> 11));
        }
    }
    Walk total = cta_walk(lw.w, sh_warps);
    if (threadIdx.x == 0) {
        if (sp < 0) total.fail = 1;
        walks[blockIdx.x] = total;
    }
}

// Applies a walk to s when s is in the binade it was made for and the walk stays inside. Every partial
// sum must round to m strictly inside (2^52, 2^53): then the exact sum it rounds lies in [2^52, 2^53) u
// and was rounded to the binade's ulp (a sum rounding to 2^52 itself may have come from below, where
// the ulp is u / 2).
__device__ __forceinline__ bool apply_walk(double* s, const Walk& w, int ef, int neg) {
    if (w.fail) return false;
    const unsigned long long bits = (unsigned long long)__double_as_longlong(*s);
    const int sef = (int)((bits >> 52) & 0x7FF);
    if (*s == 0.0 || sef != ef || (int)(bits >> 63) != neg) return false;
    const long long m = (long long)(bits & ((1ULL << 52) - 1)) | kM0;
    const int p = (int)(m & 1);
    if (w.lo[p] <= w.hi[p] && (m + w.lo[p] <= kM0 || m + w.hi[p] >= kM1)) return false;
    const long long m2 = m + w.step[p];
    if (m2 < kM0 || m2 >= kM1) return false;
    *s = __longlong_as_double((long long)(((unsigned long long)neg << 63) | ((unsigned long long)ef << 52) |
                                          (unsigned long long)(m2 - kM0)));
    return true;
}

// The walk over the blocks, one CTA. Thread 0 keeps the sum; the CTA reduces a piece on the spot, or
// stages it for thread 0's serial additions.
template <typename T>
__global__ void __launch_bounds__(kSSThreads) k_ss_chain(SumIn<T> in, const int* __restrict__ spec,
                                                        const Walk* __restrict__ walks, int blocks,
                                                        double* __restrict__ out, double divisor,
                                                        long long* __restrict__ counts) {
    constexpr int kBatch = 256;   // blocks whose walks are staged in shared memory at a time
    __shared__ Walk sh_warps[kSSThreads / 32];
    __shared__ Walk sh_walks[kBatch];
    __shared__ int sh_spec[kBatch];
    __shared__ T vals[kSSThreads];
    __shared__ uint8_t present[kSSThreads];
    __shared__ double s_sh;
    double s = 0.0;   // thread 0's
    long long whole = 0, reduced = 0, serial = 0;   // thread 0's: blocks, pieces, pieces
    for (int j = 0; j < blocks; ++j) {
        if (j % kBatch == 0) {
            __syncthreads();
            for (int i = threadIdx.x; i < kBatch && j + i < blocks; i += blockDim.x) {
                sh_walks[i] = walks[j + i];
                sh_spec[i] = spec[j + i];
            }
            __syncthreads();
        }
        int decided = 0;
        if (threadIdx.x == 0) {
            const int sp = sh_spec[j % kBatch];
            decided = sp >= 0 && apply_walk(&s, sh_walks[j % kBatch], sp & 0x7FF, sp >> 11);
            whole += decided;
            s_sh = s;
        }
        // The barrier hands thread 0's decision to every thread (no shared flag a later write could race).
        if (__syncthreads_or(decided)) continue;
        // The block in pieces of 1024, each reduced for the binade the sum is in when it begins.
        for (int piece = 0; piece < kSSPer; ++piece) {
            const size_t i = (size_t)j * kSSBlock + (size_t)piece * kSSThreads + threadIdx.x;
            T v = 0;
            const bool has = value_at(in, i, &v);
            vals[threadIdx.x] = v;
            present[threadIdx.x] = has ? 1 : 0;
            const double cur = s_sh;
            const unsigned long long bits = (unsigned long long)__double_as_longlong(cur);
            const int ef = (int)((bits >> 52) & 0x7FF), neg = (int)(bits >> 63);
            const bool reducible = cur != 0.0 && ef != 0 && ef != 0x7FF;
            LocalWalk lw;
            lw.init();
            if (reducible && has) lw.add(step_of(v, ef, neg));
            const Walk w = cta_walk(lw.w, sh_warps);   // includes the barrier that publishes vals
            if (threadIdx.x == 0) {
                if (reducible && apply_walk(&s, w, ef, neg)) {
                    ++reduced;
                } else {
                    ++serial;
                    for (int k = 0; k < kSSThreads; ++k)
                        if (present[k]) s = __dadd_rn(s, (double)vals[k]);
                }
                s_sh = s;
            }
            __syncthreads();
        }
    }
    if (threadIdx.x == 0) {
        *out = divisor != 0.0 ? __ddiv_rn(s, divisor) : s;
        if (counts) {
            counts[0] = whole;
            counts[1] = reduced;
            counts[2] = serial;
        }
    }
}

template <typename T>
cg_status seq_sum_run(cg_ctx* ctx, const SumIn<T>& in, double divisor, double* d_out, long long* d_counts) {
    const size_t n = in.n;
    const int blocks = (int)((n + kSSBlock - 1) / kSSBlock);
    cudaStream_t sm = ctx->stream;
    if (blocks == 0) {
        CG_CUDA(ctx, cudaMemsetAsync(d_out, 0, sizeof(double), sm));
        if (d_counts) CG_CUDA(ctx, cudaMemsetAsync(d_counts, 0, 3 * sizeof(long long), sm));
        return CG_OK;
    }
    CG_BUF(double, d_est, ctx, S_SS_EST, (size_t)blocks);
    CG_BUF(int, d_spec, ctx, S_SS_SPEC, (size_t)blocks);
    CG_BUF(Walk, d_walks, ctx, S_SS_WALK, (size_t)blocks);
    CG_LAUNCH(ctx) k_ss_estimate<T><<<blocks, kSSThreads, 0, sm>>>(in, d_est);
    CG_LAUNCH(ctx) k_ss_spec<<<1, 1024, 0, sm>>>(d_est, blocks, d_spec);
    CG_LAUNCH(ctx) k_ss_walks<T><<<blocks, kSSThreads, 0, sm>>>(in, d_spec, d_walks);
    CG_LAUNCH(ctx) k_ss_chain<T><<<1, kSSThreads, 0, sm>>>(in, d_spec, d_walks, blocks, d_out, divisor, d_counts);
    CG_CHECK_LAUNCH(ctx);
    return CG_OK;
}

}  // namespace

// The reference's sequential double sum of (mode 0) x or (mode 1) 1 - 0.5 x over the cells of `mask`
// (every cell when null), in cell order, into *d_out on the device; divided by `divisor` when it is
// not 0 (the mean's one division, in double).
cg_status seq_sum_dev(cg_ctx* ctx, const float* d_x, const uint8_t* d_mask, int mode, size_t n, double divisor,
                      double* d_out, long long* d_counts) {
    return seq_sum_run(ctx, SumIn<float>{d_x, d_mask, mode, n}, divisor, d_out, d_counts);
}

// `s = 0.0; for (v in x) s += v` over n double terms, into *d_out on the device.
cg_status seq_sum_f64_dev(cg_ctx* ctx, const double* d_x, size_t n, double* d_out) {
    return seq_sum_run(ctx, SumIn<double>{d_x, nullptr, 0, n}, 0.0, d_out, nullptr);
}

}  // namespace cg

using namespace cg;

extern "C" cg_status cg_sequential_sum(cg_ctx* ctx, const float* x, const uint8_t* mask, int32_t mode, int64_t n,
                                       double* sum, int64_t* counts) {
    if (!ctx || !sum || n < 0 || (n > 0 && !x) || (mode != 0 && mode != 1)) return CG_BAD_ARG;
    CG_CUDA(ctx, cudaSetDevice(ctx->device));
    ctx->run.active = false;
    const size_t N = (size_t)n;
    CG_BUF(float, d_x, ctx, S_SS_X, N);
    CG_BUF(uint8_t, d_m, ctx, S_SS_MASK, mask ? N : 1);
    CG_BUF(double, d_out, ctx, S_SS_OUT, 4);   // the sum, then the three counts
    if (N) CG_CUDA(ctx, cudaMemcpyAsync(d_x, x, N * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
    if (N && mask) CG_CUDA(ctx, cudaMemcpyAsync(d_m, mask, N, cudaMemcpyHostToDevice, ctx->stream));
    long long* d_counts = (long long*)(d_out + 1);
    CG_TRY_ST(seq_sum_dev(ctx, d_x, mask ? d_m : nullptr, mode, N, 0.0, d_out, d_counts));
    CG_CUDA(ctx, cudaMemcpyAsync(sum, d_out, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    if (counts) CG_CUDA(ctx, cudaMemcpyAsync(counts, d_counts, 3 * sizeof(long long), cudaMemcpyDeviceToHost, ctx->stream));
    CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return CG_OK;
}
