// Musgrave thermal sweeps (ErosionStage.thermalSweep, ErosionStage.kt:235-403), fused for GB300.
//
// One sweep is two passes in the reference: every cell's give rate from its 8 neighbours, then
// every cell's new height from its neighbours' give rates. Here one CTA owns a 64 x 32 tile and
// loads it with a halo of 2K cells into shared memory; it runs K sweeps there (K = 2, or 1 for an
// odd remainder), each sweep's region shrinking by two cells a side (one for the give pass, one for
// the move pass), and writes the tile back once. The passes are compute-bound, and the halo's
// redundant work grows with K while the memory traffic it saves is small next to the compute, so
// K stays at 2: global traffic is one read and one write per two sweeps.
//
// The arithmetic per cell is the reference's, in the same neighbour order, in float, with no
// fused multiply-add, so the result is bit-identical to ErosionStage.thermalSweep. Tiles away from
// the poles take a path without the per-neighbour row checks; both paths compute the same values.
#include "cg_common.cuh"
#include "cg_internal.h"

namespace cg {

namespace {

constexpr int TX = 64;
constexpr int TY = 32;
constexpr int THREADS = 256;   // 32 x 8
constexpr int KMAX = 2;

struct ThermalArgs {
    float limit[8];
    float settled;
    float rate;
};

// Settled-tile skip (the reference's own skip, ErosionStage.kt:269-342, restated for fused launches).
// A launch of K sweeps carries any change at most 2K cells, less than a tile's side, so a tile can
// change only if a cell of it or of one of its 8 neighbouring tiles changed in the previous launch.
// `prev` holds those per-tile "changed" bits (null: compute every tile); each launch writes its own
// into `cur`. A skipped tile is not even copied: the launches ping-pong between two buffers, and a
// tile that did not change in the previous launch holds the same bits in both.
struct TileFlags {
    const uint8_t* prev;
    uint8_t* cur;
};

// The give pass over the region's rows [m, RH - m) and columns [m, RW - m).
template <int RW, int RH, bool EDGE>
__device__ __forceinline__ void give_pass(const float* __restrict__ hs, float* __restrict__ gv, int m, int y0, int H,
                                          const ThermalArgs& a) {
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    for (int ry = m + ty; ry < RH - m; ry += 8) {
        const int gy = y0 + ry;
        if (EDGE && (gy < 0 || gy >= H)) continue;
        for (int rx = m + tx; rx < RW - m; rx += 32) {
            const int c = ry * RW + rx;
            const float here = hs[c];
            float excess = 0.0f, steepest = 0.0f;
#pragma unroll
            for (int n = 0; n < 8; ++n) {
                const int rs = thermal_row_step(n), cs = thermal_col_step(n);
                if (EDGE && (gy + rs < 0 || gy + rs >= H)) continue;
                const float drop = __fsub_rn(here, hs[c + rs * RW + cs]);
                if (drop <= 0.0f) continue;
                if (drop > steepest) steepest = drop;
                const float limit = a.limit[n];
                if (drop > limit) excess = __fadd_rn(excess, __fsub_rn(drop, limit));
            }
            float g = 0.0f;
            if (excess > a.settled) {
                const float p = __fmul_rn(a.rate, excess), q = __fmul_rn(steepest, 0.5f);
                g = __fdiv_rn(p <= q ? p : q, excess);
            }
            gv[c] = g;
        }
    }
}

// The move pass: h' = h - given + received, over rows [m, RH - m) and columns [m, RW - m).
template <int RW, int RH, bool EDGE>
__device__ __forceinline__ void move_pass(const float* __restrict__ hs, const float* __restrict__ gv,
                                          float* __restrict__ hn, int m, int y0, int H, const ThermalArgs& a) {
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    for (int ry = m + ty; ry < RH - m; ry += 8) {
        const int gy = y0 + ry;
        if (EDGE && (gy < 0 || gy >= H)) continue;
        for (int rx = m + tx; rx < RW - m; rx += 32) {
            const int c = ry * RW + rx;
            const float here = hs[c];
            const float gc = gv[c];
            float received = 0.0f, given = 0.0f;
#pragma unroll
            for (int n = 0; n < 8; ++n) {
                const int rs = thermal_row_step(n), cs = thermal_col_step(n);
                if (EDGE && (gy + rs < 0 || gy + rs >= H)) continue;
                const float limit = a.limit[n];
                const int nc = c + rs * RW + cs;
                const float incoming = __fsub_rn(hs[nc], here);
                if (incoming > limit) {
                    received = __fadd_rn(received, __fmul_rn(gv[nc], __fsub_rn(incoming, limit)));
                } else if (-incoming > limit) {
                    given = __fadd_rn(given, __fmul_rn(gc, __fsub_rn(-incoming, limit)));
                }
            }
            hn[c] = __fadd_rn(__fsub_rn(here, given), received);
        }
    }
}

template <int K>
__global__ void __launch_bounds__(THREADS) thermal_sweeps_kernel(const float* __restrict__ in, float* __restrict__ out,
                                                                 int W, int H, ThermalArgs a, TileFlags fl) {
    constexpr int HALO = 2 * K;
    constexpr int RW = TX + 2 * HALO;   // region width
    constexpr int RH = TY + 2 * HALO;   // region height
    __shared__ float sm_a[RW * RH], sm_b[RW * RH], sm_g[RW * RH];
    float* hs = sm_a;   // heights, current sweep
    float* hn = sm_b;   // heights, next sweep

    const int tile = blockIdx.y * gridDim.x + blockIdx.x;
    if (fl.prev) {
        bool near_change = false;
        for (int dy = -1; dy <= 1; ++dy) {
            int ty = (int)blockIdx.y + dy;
            if (ty < 0 || ty >= (int)gridDim.y) continue;
            for (int dx = -1; dx <= 1; ++dx) {
                int tx = ((int)blockIdx.x + dx + (int)gridDim.x) % (int)gridDim.x;
                if (fl.prev[ty * gridDim.x + tx]) near_change = true;
            }
        }
        if (!near_change) {
            if (threadIdx.x == 0) fl.cur[tile] = 0;
            return;
        }
    }

    const int x0 = blockIdx.x * TX - HALO;
    const int y0 = blockIdx.y * TY - HALO;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    for (int ry = ty; ry < RH; ry += 8) {
        const int gy = y0 + ry;
        const bool valid = gy >= 0 && gy < H;
        const float* rowp = in + (size_t)(valid ? gy : 0) * W;
        for (int rx = tx; rx < RW; rx += 32) hs[ry * RW + rx] = valid ? rowp[wrap_col(x0 + rx, W)] : 0.0f;
    }
    __syncthreads();

    // Every row of the region on the grid: no pole checks needed.
    const bool edge = y0 < 0 || y0 + RH > H;
#pragma unroll 1
    for (int s = 0; s < K; ++s) {
        if (edge) give_pass<RW, RH, true>(hs, sm_g, 2 * s + 1, y0, H, a);
        else give_pass<RW, RH, false>(hs, sm_g, 2 * s + 1, y0, H, a);
        __syncthreads();
        if (edge) move_pass<RW, RH, true>(hs, sm_g, hn, 2 * s + 2, y0, H, a);
        else move_pass<RW, RH, false>(hs, sm_g, hn, 2 * s + 2, y0, H, a);
        __syncthreads();
        float* t = hs;
        hs = hn;
        hn = t;
    }

    int changed = 0;
    for (int yy = ty; yy < TY; yy += 8) {
        const int gy = blockIdx.y * TY + yy;
        if (gy >= H) continue;
        for (int xx = tx; xx < TX; xx += 32) {
            const int gx = blockIdx.x * TX + xx;
            if (gx >= W) continue;
            const size_t idx = (size_t)gy * W + gx;
            const float v = hs[(yy + HALO) * RW + xx + HALO];
            if (__float_as_uint(v) != __float_as_uint(in[idx])) changed = 1;
            out[idx] = v;
        }
    }
    if (fl.cur) {
        changed = __syncthreads_or(changed);
        if (threadIdx.x == 0) fl.cur[tile] = changed ? 1 : 0;
    }
}

template <int K>
cudaError_t launch(const float* in, float* out, int W, int H, const ThermalArgs& a, cudaStream_t st,
                   TileFlags fl = TileFlags{nullptr, nullptr}) {
    dim3 grid((W + TX - 1) / TX, (H + TY - 1) / TY);
    thermal_sweeps_kernel<K><<<grid, THREADS, 0, st>>>(in, out, W, H, a, fl);
    return cudaGetLastError();
}

ThermalArgs args_of(const ThermalLaunch& t) {
    ThermalArgs a;
    for (int n = 0; n < 8; ++n) a.limit[n] = t.limit[n];
    a.settled = t.settled;
    a.rate = t.rate;
    return a;
}

}  // namespace

ThermalLaunch thermal_launch_args(cg_thermal_limits lim, float rate) {
    ThermalLaunch t;
    for (int n = 0; n < 8; ++n)
        t.limit[n] = n >= 4 ? lim.diagonal : (thermal_row_step(n) != 0 ? lim.north_south : lim.east_west);
    t.settled = lim.east_west * 1e-3f;   // SETTLED_SHARE_OF_CRITICAL_SLOPE (ErosionStage.kt:92)
    t.rate = rate;
    return t;
}

int thermal_step(int passes_left) { return passes_left >= KMAX ? KMAX : 1; }

int thermal_launches(int passes) {
    int n = 0;
    while (passes > 0) passes -= thermal_step(passes), ++n;
    return n;
}

// One fused launch of k sweeps (k = thermal_step(...)) from src into dst on `stream`.
cudaError_t thermal_launch(const float* src, float* dst, int W, int H, const ThermalLaunch& t, int k,
                           cudaStream_t stream) {
    ThermalArgs a = args_of(t);
    return k == 2 ? launch<2>(src, dst, W, H, a, stream) : launch<1>(src, dst, W, H, a, stream);
}

// `passes` sweeps from d_a; the result lands in *result (d_a or d_b). Deterministic ping-pong.
cg_status thermal_sweeps_dev(cg_ctx* ctx, int W, int H, float* d_a, float* d_b, cg_thermal_limits lim, int passes,
                             float rate, float** result) {
    const ThermalArgs a = args_of(thermal_launch_args(lim, rate));
    // Per-tile change bits of the previous and the current launch. The first launch computes every
    // tile (the destination holds nothing yet); after it, both buffers hold a tile's bits whenever
    // that tile did not change, so the skip needs no copy.
    const int tiles = ((W + TX - 1) / TX) * ((H + TY - 1) / TY);
    CG_BUF(uint8_t, d_flags, ctx, S_THERMFLAG, 2 * (size_t)tiles);
    uint8_t* prev = d_flags;
    uint8_t* cur = d_flags + tiles;
    float* src = d_a;
    float* dst = d_b;
    bool first = true;
    while (passes > 0) {
        const int k = thermal_step(passes);
        TileFlags fl{first ? nullptr : prev, cur};
        cudaError_t e = k == 2 ? launch<2>(src, dst, W, H, a, ctx->stream, fl) : launch<1>(src, dst, W, H, a, ctx->stream, fl);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "thermal_sweeps_kernel", __FILE__, __LINE__);
        passes -= k;
        ctx->launches++;
        first = false;
        float* t = src;
        src = dst;
        dst = t;
        uint8_t* tf = prev;
        prev = cur;
        cur = tf;
    }
    *result = src;
    return CG_OK;
}

}  // namespace cg
