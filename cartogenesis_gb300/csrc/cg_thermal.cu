// Musgrave thermal sweeps (ErosionStage.thermalSweep, ErosionStage.kt:235-403), fused and
// temporally blocked for GB300.
//
// One sweep is two passes in the reference: every cell's give rate from its 8 neighbours, then
// every cell's new height from its neighbours' give rates. Here one CTA owns a TX x TY tile and
// loads it with a halo of 2K cells into shared memory; it then runs K whole sweeps there, each
// sweep's region shrinking by two cells a side (one for the give pass, one for the move pass), and
// writes the tile back once. Global traffic is one read (plus halo) and one write per K sweeps
// instead of per sweep.
//
// The arithmetic per cell is the reference's, in the same neighbour order, in float, with no
// fused multiply-add, so the result is bit-identical to ErosionStage.thermalSweep. The reference's
// settled-tile skip is exact (T/ErosionSkipTest.kt), so sweeping every tile gives the same bits.
#include "cg_common.cuh"
#include "cg_internal.h"

namespace cg {

namespace {

constexpr int TX = 64;
constexpr int TY = 32;
constexpr int THREADS = 256;

struct ThermalArgs {
    float limit[8];
    float settled;
    float rate;
};

// Settled-tile skip (the reference's own skip, ErosionStage.kt:269-342, restated for fused launches).
// A launch of K sweeps carries any change at most 2K <= 16 cells, less than a tile's side, so a tile
// can change only if a cell of it or of one of its 8 neighbouring tiles changed in the previous
// launch. `prev` holds those per-tile "changed" bits (null: compute every tile); each launch writes
// its own into `cur`. A skipped tile is not even copied: the launches ping-pong between two buffers,
// and a tile that did not change in the previous launch holds the same bits in both.
struct TileFlags {
    const uint8_t* prev;
    uint8_t* cur;
};

template <int K>
__global__ void __launch_bounds__(THREADS) thermal_sweeps_kernel(const float* __restrict__ in, float* __restrict__ out,
                                                                 int W, int H, ThermalArgs a, TileFlags fl) {
    constexpr int HALO = 2 * K;
    constexpr int RW = TX + 2 * HALO;   // region width
    constexpr int RH = TY + 2 * HALO;   // region height
    extern __shared__ float smem[];
    float* hs = smem;                  // heights, current sweep
    float* hn = smem + RW * RH;        // heights, next sweep
    float* gv = smem + 2 * RW * RH;    // give rates

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

    for (int i = threadIdx.x; i < RW * RH; i += THREADS) {
        int ry = i / RW, rx = i - ry * RW;
        int gy = y0 + ry;
        float v = 0.0f;
        if (gy >= 0 && gy < H) v = in[(size_t)gy * W + wrap_col(x0 + rx, W)];
        hs[i] = v;
        hn[i] = v;
    }
    __syncthreads();

#pragma unroll 1
    for (int s = 0; s < K; ++s) {
        // Give pass over the region shrunk by 2s+1.
        {
            const int m = 2 * s + 1;
            const int w = RW - 2 * m, h = RH - 2 * m;
            for (int i = threadIdx.x; i < w * h; i += THREADS) {
                int ry = m + i / w, rx = m + i % w;
                int gy = y0 + ry;
                if (gy < 0 || gy >= H) continue;
                int c = ry * RW + rx;
                float here = hs[c];
                float excess = 0.0f, steepest = 0.0f;
#pragma unroll
                for (int n = 0; n < 8; ++n) {
                    int rs = thermal_row_step(n), cs = thermal_col_step(n);
                    int ny = gy + rs;
                    if (ny < 0 || ny >= H) continue;
                    float drop = here - hs[c + rs * RW + cs];
                    if (drop <= 0.0f) continue;
                    if (drop > steepest) steepest = drop;
                    float limit = a.limit[n];
                    if (drop > limit) excess = __fadd_rn(excess, __fsub_rn(drop, limit));
                }
                float g;
                if (excess <= a.settled) {
                    g = 0.0f;
                } else {
                    float p = __fmul_rn(a.rate, excess), q = __fmul_rn(steepest, 0.5f);
                    g = __fdiv_rn(p <= q ? p : q, excess);
                }
                gv[c] = g;
            }
        }
        __syncthreads();
        // Move pass over the region shrunk by 2s+2.
        {
            const int m = 2 * s + 2;
            const int w = RW - 2 * m, h = RH - 2 * m;
            for (int i = threadIdx.x; i < w * h; i += THREADS) {
                int ry = m + i / w, rx = m + i % w;
                int gy = y0 + ry;
                if (gy < 0 || gy >= H) continue;
                int c = ry * RW + rx;
                float here = hs[c];
                float gc = gv[c];
                float received = 0.0f, given = 0.0f;
#pragma unroll
                for (int n = 0; n < 8; ++n) {
                    int rs = thermal_row_step(n), cs = thermal_col_step(n);
                    int ny = gy + rs;
                    if (ny < 0 || ny >= H) continue;
                    float limit = a.limit[n];
                    int nc = c + rs * RW + cs;
                    float incoming = __fsub_rn(hs[nc], here);
                    if (incoming > limit) {
                        received = __fadd_rn(received, __fmul_rn(gv[nc], __fsub_rn(incoming, limit)));
                    } else if (-incoming > limit) {
                        given = __fadd_rn(given, __fmul_rn(gc, __fsub_rn(-incoming, limit)));
                    }
                }
                hn[c] = __fadd_rn(__fsub_rn(here, given), received);
            }
        }
        __syncthreads();
        float* t = hs;
        hs = hn;
        hn = t;
    }

    int changed = 0;
    for (int i = threadIdx.x; i < TX * TY; i += THREADS) {
        int ty = i / TX, tx = i - ty * TX;
        int gy = blockIdx.y * TY + ty, gx = blockIdx.x * TX + tx;
        if (gy >= H || gx >= W) continue;
        size_t idx = (size_t)gy * W + gx;
        float v = hs[(ty + HALO) * RW + tx + HALO];
        if (__float_as_uint(v) != __float_as_uint(in[idx])) changed = 1;
        out[idx] = v;
    }
    if (fl.cur) {
        changed = __syncthreads_or(changed);
        if (threadIdx.x == 0) fl.cur[tile] = changed ? 1 : 0;
    }
}

template <int K>
size_t smem_bytes() {
    return sizeof(float) * 3 * (TX + 4 * K) * (TY + 4 * K);
}

template <int K>
cudaError_t launch(const float* in, float* out, int W, int H, const ThermalArgs& a, cudaStream_t st,
                   TileFlags fl = TileFlags{nullptr, nullptr}) {
    static bool configured = false;
    size_t bytes = smem_bytes<K>();
    if (!configured) {
        cudaError_t e = cudaFuncSetAttribute(thermal_sweeps_kernel<K>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)bytes);
        if (e != cudaSuccess) return e;
        configured = true;
    }
    dim3 grid((W + TX - 1) / TX, (H + TY - 1) / TY);
    thermal_sweeps_kernel<K><<<grid, THREADS, bytes, st>>>(in, out, W, H, a, fl);
    return cudaGetLastError();
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

// One fused launch of k sweeps (k in {1, 2, 4, 8}) from src into dst on `stream`.
cudaError_t thermal_launch(const float* src, float* dst, int W, int H, const ThermalLaunch& t, int k,
                           cudaStream_t stream) {
    ThermalArgs a;
    for (int n = 0; n < 8; ++n) a.limit[n] = t.limit[n];
    a.settled = t.settled;
    a.rate = t.rate;
    switch (k) {
        case 8: return launch<8>(src, dst, W, H, a, stream);
        case 4: return launch<4>(src, dst, W, H, a, stream);
        case 2: return launch<2>(src, dst, W, H, a, stream);
        default: return launch<1>(src, dst, W, H, a, stream);
    }
}

int thermal_launches(int passes) {
    int n = 0;
    while (passes >= 8) passes -= 8, ++n;
    if (passes >= 4) passes -= 4, ++n;
    if (passes >= 2) passes -= 2, ++n;
    if (passes >= 1) ++n;
    return n;
}

// `passes` sweeps from d_a; the result lands in *result (d_a or d_b). Deterministic ping-pong.
cg_status thermal_sweeps_dev(cg_ctx* ctx, int W, int H, float* d_a, float* d_b, cg_thermal_limits lim, int passes,
                             float rate, float** result) {
    ThermalArgs a;
    for (int n = 0; n < 8; ++n)
        a.limit[n] = n >= 4 ? lim.diagonal : (thermal_row_step(n) != 0 ? lim.north_south : lim.east_west);
    a.settled = lim.east_west * 1e-3f;   // SETTLED_SHARE_OF_CRITICAL_SLOPE (ErosionStage.kt:92)
    a.rate = rate;
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
        cudaError_t e;
        TileFlags fl{first ? nullptr : prev, cur};
        if (passes >= 8) e = launch<8>(src, dst, W, H, a, ctx->stream, fl), passes -= 8;
        else if (passes >= 4) e = launch<4>(src, dst, W, H, a, ctx->stream, fl), passes -= 4;
        else if (passes >= 2) e = launch<2>(src, dst, W, H, a, ctx->stream, fl), passes -= 2;
        else e = launch<1>(src, dst, W, H, a, ctx->stream, fl), passes -= 1;
        if (e != cudaSuccess) return cuda_fail(ctx, e, "thermal_sweeps_kernel", __FILE__, __LINE__);
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
