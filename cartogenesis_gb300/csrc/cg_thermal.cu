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
#include <cuda.h>

#include <cmath>

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
    float lim0[8];   // max(limit, 0)
    float settled;
    float rate;
    float min_lim0;  // the least of lim0
    int plain;       // every limit >= 0 and settled >= 0: the shortcuts below are exact
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

// The region load by the tensor memory accelerator: one cp.async.bulk.tensor.2d per CTA of the
// whole (TX + 2 HALO) x (TY + 2 HALO) region, rows off the grid filled with zeros by the copy
// itself. Used for K = 2 (the region's first column, x0 = 64 bx - 4, is 16-byte aligned as TMA
// requires) on tiles whose region does not wrap east-west; the two wrapping tile columns and the
// odd single-sweep launch load by threads. `err` (device) is set when a copy's wait runs out, after
// which the CTA waits once more for its copy and leaves without computing; the host reports it.
struct RegionLoad {
    CUtensorMap map;   // the source field, box = the region
    int on;            // a map was made for this launch
    int* err;
};

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Waits on the mbarrier's phase 0 for at most `tries` polls; true when the phase completed.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, int tries) {
    for (int i = 0; i < tries; ++i) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(bar), "r"(0)
            : "memory");
        if (done) return true;
    }
    return false;
}

// Per-cell rules, written without branches: the conditions become predicated adds in the
// reference's neighbour order, so the sums round exactly as the reference's loop does.
// Neighbours by name: E/W the same row, S/N the rows below/above, and the diagonals SE (+1,+1),
// NE (+1,-1), SW (-1,+1), NW (-1,-1) as (column step, row step).
struct Window {
    float nw, n, ne, w, c, e, sw, s, se;   // the 3 x 3 block around a cell
};

// The give rate of a cell away from the poles with plain limits (every limit and the settled share
// >= 0), the same bits as give_rate with fewer instructions:
//  - a cell no drop of which exceeds the least max(limit, 0) gives nothing. Float subtraction is
//    monotone, so c - min(neighbours) bounds every drop from above, and then the excess stays +0,
//    which is not above the settled share (>= 0): the rate is +0, as the full rule returns;
//  - the steepest drop as a running max: the reference keeps the larger of the two, and the heights
//    are finite; the max may return -0 where the rule keeps +0, which changes neither the rate's
//    products nor any sum (every sum starts at +0 and adds terms >= 0).
__device__ __forceinline__ float give_rate_plain(const Window& v, const ThermalArgs& a) {
    const float lowest = fminf(fminf(fminf(v.e, v.w), fminf(v.s, v.n)), fminf(fminf(v.se, v.ne), fminf(v.sw, v.nw)));
    if (__fsub_rn(v.c, lowest) <= a.min_lim0) return 0.0f;
    const float nb[8] = {v.e, v.w, v.s, v.n, v.se, v.ne, v.sw, v.nw};
    float excess = 0.0f, steepest = 0.0f;
#pragma unroll
    for (int n = 0; n < 8; ++n) {
        const float drop = __fsub_rn(v.c, nb[n]);
        steepest = fmaxf(steepest, drop);
        const float over = __fsub_rn(drop, a.limit[n]);
        if (drop > a.lim0[n]) excess = __fadd_rn(excess, over);
    }
    float g = 0.0f;
    if (excess > a.settled) {
        const float p = __fmul_rn(a.rate, excess), q = __fmul_rn(steepest, 0.5f);
        g = __fdiv_rn(p <= q ? p : q, excess);
    }
    return g;
}

// The new height of a cell away from the poles with plain limits, the same bits as `moved`: with a
// limit >= 0 a drop that moves material either way has magnitude |incoming|, so one absolute value
// replaces the select of the sign; a term is added as +0 where the rule skips it (sums start at +0
// and gain only terms >= 0, so adding +0 changes no bit).
__device__ __forceinline__ float moved_plain(const Window& v, const Window& g, const ThermalArgs& a) {
    const float nb[8] = {v.e, v.w, v.s, v.n, v.se, v.ne, v.sw, v.nw};
    const float gn[8] = {g.e, g.w, g.s, g.n, g.se, g.ne, g.sw, g.nw};
    float received = 0.0f, given = 0.0f;
#pragma unroll
    for (int n = 0; n < 8; ++n) {
        const float limit = a.limit[n];
        const float incoming = __fsub_rn(nb[n], v.c);
        const bool in = incoming > limit;
        const bool out = incoming < -limit;
        const float p = __fmul_rn(in ? gn[n] : g.c, __fsub_rn(fabsf(incoming), limit));
        received = __fadd_rn(received, in ? p : 0.0f);
        given = __fadd_rn(given, out ? p : 0.0f);
    }
    return __fadd_rn(__fsub_rn(v.c, given), received);
}

// The give rate of a cell (ErosionStage.kt:283-311). `lim0[n]` is max(limit, 0): a drop counts
// towards the excess when it is positive and above the limit. `has_s` / `has_n`: the rows below /
// above exist (false only at the poles).
__device__ __forceinline__ float give_rate(const Window& v, bool has_s, bool has_n, const ThermalArgs& a) {
    const float nb[8] = {v.e, v.w, v.s, v.n, v.se, v.ne, v.sw, v.nw};
    const bool ok[8] = {true, true, has_s, has_n, has_s, has_n, has_s, has_n};
    float excess = 0.0f, steepest = 0.0f;
#pragma unroll
    for (int n = 0; n < 8; ++n) {
        const float drop = __fsub_rn(v.c, nb[n]);
        if (ok[n] && drop > steepest) steepest = drop;
        const float over = __fsub_rn(drop, a.limit[n]);
        if (ok[n] && drop > a.lim0[n]) excess = __fadd_rn(excess, over);
    }
    float g = 0.0f;
    if (excess > a.settled) {
        const float p = __fmul_rn(a.rate, excess), q = __fmul_rn(steepest, 0.5f);
        g = __fdiv_rn(p <= q ? p : q, excess);
    }
    return g;
}

// The new height of a cell from its neighbours' give rates (ErosionStage.kt:313-340).
__device__ __forceinline__ float moved(const Window& v, const Window& g, bool has_s, bool has_n,
                                       const ThermalArgs& a) {
    const float nb[8] = {v.e, v.w, v.s, v.n, v.se, v.ne, v.sw, v.nw};
    const float gn[8] = {g.e, g.w, g.s, g.n, g.se, g.ne, g.sw, g.nw};
    const bool ok[8] = {true, true, has_s, has_n, has_s, has_n, has_s, has_n};
    float received = 0.0f, given = 0.0f;
#pragma unroll
    for (int n = 0; n < 8; ++n) {
        const float limit = a.limit[n];
        const float incoming = __fsub_rn(nb[n], v.c);
        const bool in = incoming > limit;
        const bool out = !in && -incoming > limit;
        // One product serves both branches: (incoming - limit) * g_n coming in, (-incoming - limit) * g_c
        // going out; the sums take it only under their own condition, in the reference's order.
        const float p = __fmul_rn(in ? gn[n] : g.c, __fsub_rn(in ? incoming : -incoming, limit));
        if (ok[n] && in) received = __fadd_rn(received, p);
        if (ok[n] && out) given = __fadd_rn(given, p);
    }
    return __fadd_rn(__fsub_rn(v.c, given), received);
}

// One pass over the region's rows [M, RH - M) and columns [M, RW - M). A thread takes a column
// segment of up to SEG rows and slides a 3 x 3 window down it, so each cell costs three
// shared-memory loads per field instead of nine. Work items are (segment, column), columns
// fastest, so a warp's loads are consecutive words. MOVE: the move pass (reads gv, writes dst),
// else the give pass (writes gv).
template <int RW, int RH, int M, bool MOVE, bool EDGE>
__device__ __forceinline__ void pass(const float* __restrict__ hs, float* __restrict__ gv, float* __restrict__ dst,
                                     int y0, int H, const ThermalArgs& a, int halo, bool& changed) {
    constexpr int SEG = 4;
    constexpr int COLS = RW - 2 * M, ROWS = RH - 2 * M;
    constexpr int SEGS = (ROWS + SEG - 1) / SEG;
    constexpr int ITEMS = COLS * SEGS;
    for (int item = threadIdx.x; item < ITEMS; item += THREADS) {
        const int col = M + item % COLS;
        const int r0 = M + (item / COLS) * SEG;
        const int r1 = r0 + SEG < RH - M ? r0 + SEG : RH - M;
        const float* p = hs + (r0 - 1) * RW + col;
        Window v;
        v.nw = p[-1], v.n = p[0], v.ne = p[1];
        v.w = p[RW - 1], v.c = p[RW], v.e = p[RW + 1];
        Window g{};
        unsigned or_top = 0, or_mid = 0;   // bitwise OR of the give rates' bits, per window row
        if (MOVE) {
            const float* q = gv + (r0 - 1) * RW + col;
            g.nw = q[-1], g.n = q[0], g.ne = q[1];
            g.w = q[RW - 1], g.c = q[RW], g.e = q[RW + 1];
            or_top = __float_as_uint(g.nw) | __float_as_uint(g.n) | __float_as_uint(g.ne);
            or_mid = __float_as_uint(g.w) | __float_as_uint(g.c) | __float_as_uint(g.e);
        }
#pragma unroll
        for (int k = 0; k < SEG; ++k) {
            const int ry = r0 + k;
            if (ry >= r1) break;
            const float* below = hs + (ry + 1) * RW + col;
            v.sw = below[-1], v.s = below[0], v.se = below[1];
            unsigned or_bot = 0;
            if (MOVE) {
                const float* gb = gv + (ry + 1) * RW + col;
                g.sw = gb[-1], g.s = gb[0], g.se = gb[1];
                or_bot = __float_as_uint(g.sw) | __float_as_uint(g.s) | __float_as_uint(g.se);
            }
            const int gy = y0 + ry;
            const bool on = !EDGE || (gy >= 0 && gy < H);
            const bool has_s = !EDGE || gy + 1 < H;
            const bool has_n = !EDGE || gy - 1 >= 0;
            if (on) {
                if (MOVE) {
                    // Every give rate around the cell +0: each product the rule could add is +0, so the
                    // sums stay +0 and the cell moves to (h - 0) + 0. Rows off the grid (EDGE) are
                    // left to the full rule.
                    const bool still = !EDGE && (or_top | or_mid | or_bot) == 0u;
                    const float nv = still ? __fadd_rn(__fsub_rn(v.c, 0.0f), 0.0f)
                                           : (!EDGE && a.plain) ? moved_plain(v, g, a) : moved(v, g, has_s, has_n, a);
                    dst[ry * RW + col] = nv;
                    // A cell of the tile itself that moved (in any sweep) marks the tile as changed.
                    if (__float_as_uint(nv) != __float_as_uint(v.c) && ry >= halo && ry < RH - halo &&
                        col >= halo && col < RW - halo)
                        changed = true;
                } else {
                    gv[ry * RW + col] = (!EDGE && a.plain) ? give_rate_plain(v, a) : give_rate(v, has_s, has_n, a);
                }
            }
            v.nw = v.w, v.n = v.c, v.ne = v.e;
            v.w = v.sw, v.c = v.s, v.e = v.se;
            if (MOVE) {
                g.nw = g.w, g.n = g.c, g.ne = g.e;
                g.w = g.sw, g.c = g.s, g.e = g.se;
                or_top = or_mid;
                or_mid = or_bot;
            }
        }
    }
}

// K sweeps on the region in shared memory: hs holds the heights and ends with the result
// (swapping with hn each sweep); the region's valid part shrinks by two cells a side per sweep.
template <int RW, int RH, int K, bool EDGE>
__device__ __forceinline__ float* sweeps(float* hs, float* hn, float* gv, int y0, int H, const ThermalArgs& a,
                                         bool& changed) {
    constexpr int HALO = 2 * K;
    pass<RW, RH, 1, false, EDGE>(hs, gv, nullptr, y0, H, a, HALO, changed);
    __syncthreads();
    pass<RW, RH, 2, true, EDGE>(hs, gv, hn, y0, H, a, HALO, changed);
    __syncthreads();
    if constexpr (K == 2) {
        pass<RW, RH, 3, false, EDGE>(hn, gv, nullptr, y0, H, a, HALO, changed);
        __syncthreads();
        pass<RW, RH, 4, true, EDGE>(hn, gv, hs, y0, H, a, HALO, changed);
        __syncthreads();
        return hs;
    } else {
        return hn;
    }
}

template <int K>
__global__ void __launch_bounds__(THREADS, 6) thermal_sweeps_kernel(const float* __restrict__ in, float* __restrict__ out,
                                                                 int W, int H, ThermalArgs a, TileFlags fl,
                                                                 const __grid_constant__ RegionLoad rl) {
    constexpr int HALO = 2 * K;
    constexpr int RW = TX + 2 * HALO;   // region width
    constexpr int RH = TY + 2 * HALO;   // region height
    __shared__ __align__(128) float sm_a[RW * RH];
    __shared__ __align__(16) float sm_b[RW * RH], sm_g[RW * RH];
    __shared__ __align__(8) unsigned long long bar;

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
    if (K == 2 && rl.on && x0 >= 0 && x0 + RW <= W) {
        const uint32_t b = smem_addr(&bar);
        if (threadIdx.x == 0) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b) : "memory");
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(RW * RH * 4) : "memory");
            asm volatile(
                "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
                ::"r"(smem_addr(sm_a)), "l"(&rl.map), "r"(x0), "r"(y0), "r"(b)
                : "memory");
        }
        __syncthreads();
        if (!mbar_wait(b, 1 << 22)) {
            // The copy did not land: record it, give it one more bounded wait, and leave.
            if (threadIdx.x == 0) {
                atomicOr(rl.err, 1);
                mbar_wait(b, 1 << 22);
            }
            __syncthreads();
            return;
        }
    } else {
        for (int ry = ty; ry < RH; ry += 8) {
            const int gy = y0 + ry;
            const bool valid = gy >= 0 && gy < H;
            const float* rowp = in + (size_t)(valid ? gy : 0) * W;
            for (int rx = tx; rx < RW; rx += 32) sm_a[ry * RW + rx] = valid ? rowp[wrap_col(x0 + rx, W)] : 0.0f;
        }
    }
    __syncthreads();

    // Tiles whose region lies inside the grid's rows take the path without pole checks.
    const bool edge = y0 < 0 || y0 + RH > H;
    bool moved_any = false;
    const float* res = edge ? sweeps<RW, RH, K, true>(sm_a, sm_b, sm_g, y0, H, a, moved_any)
                            : sweeps<RW, RH, K, false>(sm_a, sm_b, sm_g, y0, H, a, moved_any);

    for (int yy = ty; yy < TY; yy += 8) {
        const int gy = blockIdx.y * TY + yy;
        if (gy >= H) continue;
        for (int xx = tx; xx < TX; xx += 32) {
            const int gx = blockIdx.x * TX + xx;
            if (gx >= W) continue;
            out[(size_t)gy * W + gx] = res[(yy + HALO) * RW + xx + HALO];
        }
    }
    if (fl.cur) {
        const int changed = __syncthreads_or(moved_any);
        if (threadIdx.x == 0) fl.cur[tile] = changed ? 1 : 0;
    }
}

template <int K>
cudaError_t launch(const float* in, float* out, int W, int H, const ThermalArgs& a, cudaStream_t st,
                   TileFlags fl = TileFlags{nullptr, nullptr}, const RegionLoad* rl = nullptr) {
    dim3 grid((W + TX - 1) / TX, (H + TY - 1) / TY);
    static const RegionLoad none{};
    thermal_sweeps_kernel<K><<<grid, THREADS, 0, st>>>(in, out, W, H, a, fl, rl ? *rl : none);
    return cudaGetLastError();
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// The driver's cuTensorMapEncodeTiled, fetched through the runtime (the library links no libcuda).
EncodeTiledFn encode_tiled() {
    static EncodeTiledFn fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)p;
    }
    return fn;
}

// The region-load map of a field for K = 2 launches: the whole W x H field, a box of the region.
// Off (threads load every tile) where the driver has no encoder or the grid is too narrow.
RegionLoad region_load_of(const float* field, int W, int H, int* err) {
    RegionLoad rl{};
    rl.err = err;
    constexpr int RW = TX + 8, RH = TY + 8;
    EncodeTiledFn enc = encode_tiled();
    if (!enc || !err || W < 2 * RW || (((uintptr_t)field) & 15) != 0) return rl;
    const cuuint64_t dims[2] = {(cuuint64_t)W, (cuuint64_t)H};
    const cuuint64_t strides[1] = {(cuuint64_t)W * sizeof(float)};
    const cuuint32_t box[2] = {RW, RH};
    const cuuint32_t estride[2] = {1, 1};
    if (enc(&rl.map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void*)field, dims, strides, box, estride,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS)
        rl.on = 1;
    return rl;
}

ThermalArgs args_of(const ThermalLaunch& t) {
    ThermalArgs a;
    a.plain = t.settled >= 0.0f;
    a.min_lim0 = 3.402823466e+38f;
    for (int n = 0; n < 8; ++n) {
        a.limit[n] = t.limit[n];
        a.lim0[n] = t.limit[n] > 0.0f ? t.limit[n] : 0.0f;
        a.min_lim0 = std::fmin(a.min_lim0, a.lim0[n]);
        if (!(t.limit[n] >= 0.0f)) a.plain = 0;
    }
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
    CG_BUF(int, d_err, ctx, S_THERMERR, 1);
    uint8_t* prev = d_flags;
    uint8_t* cur = d_flags + tiles;
    float* src = d_a;
    float* dst = d_b;
    const RegionLoad maps[2] = {region_load_of(d_a, W, H, d_err), region_load_of(d_b, W, H, d_err)};
    bool first = true;
    while (passes > 0) {
        const int k = thermal_step(passes);
        TileFlags fl{first ? nullptr : prev, cur};
        const RegionLoad* rl = &maps[src == d_a ? 0 : 1];
        cudaError_t e = k == 2 ? launch<2>(src, dst, W, H, a, ctx->stream, fl, rl)
                               : launch<1>(src, dst, W, H, a, ctx->stream, fl);
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

cg_status thermal_error_reset_dev(cg_ctx* ctx) {
    CG_BUF(int, d_err, ctx, S_THERMERR, 1);
    CG_CUDA(ctx, cudaMemsetAsync(d_err, 0, sizeof(int), ctx->stream));
    return CG_OK;
}

cg_status thermal_error_check(cg_ctx* ctx) {
    CG_BUF(int, d_err, ctx, S_THERMERR, 1);
    int err = 0;
    CG_CUDA(ctx, cudaMemcpyAsync(&err, d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (err) return fail(ctx, CG_TIMEOUT, "thermal sweeps: a region copy did not arrive in its bounded wait");
    return CG_OK;
}

}  // namespace cg
