// FlowRouting.fillDepressions on the device (FlowRouting.kt:52-111), reproducing the sequential
// priority flood's result exactly.
//
// The reference pops cells off a heap keyed (Q, index), Q = bits(fl(f + 4)), and gives each cell
// the level of the first neighbour popped next to it: f(n) = g(n) if g(n) > f(parent), else
// fl(f(parent) + 1e-6). The popped Q never decreases, so a cell's parent is the neighbour of least
// Q; when that is unique, f(n) = phi(min over neighbours of f, g(n)), a monotone fixed point. The
// device computes that fixed point in parallel and then checks, cell by cell, whether the
// quantised key ever left the parent open:
//  (1) pointer jumping along strictly Q-descending neighbour chains finds every cell with such a
//      chain to an outlet; those keep their own height (their first popped neighbour is lower);
//  (2) the rest relax to the fixed point of f(n) = min_m phi(f(m), g(n)) from +inf, tile by tile
//      in shared memory, each tile iterating to local convergence before its borders are
//      republished (the monotone Bellman-Ford of a Dijkstra with non-decreasing edge functions);
//  (3) a check pass finds cells whose least-Q neighbours share a key but would give different
//      levels. The reference takes the one popped first: among neighbours that entered that key's
//      level from below, the lowest index. Such a cell is pinned to that neighbour. A tie whose
//      candidates were themselves reached inside the level (flat ground within one key quantum)
//      needs the level's own pop order: the lowest such level is replayed exactly, one thread
//      running the reference's heap over that level's cells (those that entered from below seed it;
//      lower levels are final by then), and every cell it reaches is pinned to its exact parent.
//      The levels from the lowest changed one upward are recomputed, and the check repeats; each
//      replay settles its level for good, so the lowest open level only rises. The replay's list
//      and heap are sized for the whole grid, so a level of any size is replayed. If the repairs'
//      guard (256 passes) is ever reached with ties still open, the fill returns CG_INEXACT: its
//      result is then not the reference's, and the stage does not carry on with it.
#include <algorithm>
#include <cfloat>
#include <cooperative_groups.h>
#include <climits>
#include <vector>

#include "cg_common.cuh"
#include "cg_internal.h"

namespace cg {

namespace cgr = cooperative_groups;

namespace {

constexpr float kStep = 1e-6f;   // FlowRouting.FLAT_GRADIENT_STEP
constexpr int T = 32;            // tile side
constexpr int TH = 8;            // tile rows per thread pass (block is 32 x 8)
constexpr int kReplaySpan = 1 << 12;   // key levels (consecutive float values) one replay orders

// Cell classes. PINNED: parent fixed by the index rule on a key tie; EXACT: parent fixed by
// replaying its key level's pops (both follow that parent instead of the minimum).
enum : uint8_t { C_WATER = 0, C_SEED = 1, C_DRAINED = 2, C_OPEN = 3, C_PINNED = 4, C_EXACT = 5 };

__device__ __forceinline__ bool follows_parent(uint8_t c) { return c == C_PINNED || c == C_EXACT; }

__device__ __forceinline__ int qkey(float f) { return __float_as_int(__fadd_rn(f, 4.0f)); }   // FlowRouting.encode
__device__ __forceinline__ float phi(float fp, float g) { return g > fp ? g : __fadd_rn(fp, kStep); }

struct FillCounters {
    unsigned long long ties, unresolved, repaired;
    int active;
    int changed;
    int min_level;      // the lowest key level holding a tie only its own pops can order
    int overflow;       // that level was too large to replay
    int repair_level;   // the lowest key level at which a pin changed a cell's level
};

// (0) classes and initial levels.
__global__ void k_fill_init(const uint8_t* __restrict__ land, const float* __restrict__ g, int W, int H,
                            uint8_t* __restrict__ cls, float* __restrict__ f, int* __restrict__ ptr) {
    size_t N = (size_t)W * H;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x) {
        const int row = pdiv((int)i, W);
        if (!land[i]) {
            cls[i] = C_WATER;
            f[i] = g[i];
            ptr[i] = (int)i;
            continue;
        }
        if (row == 0 || row == H - 1) {
            cls[i] = C_SEED;
            f[i] = g[i];
            ptr[i] = (int)i;
            continue;
        }
        // Steepest strictly Q-descending neighbour on the unfilled ground (water counts as is).
        const int col = pmod((int)i, W);
        int q = qkey(g[i]);
        int best = (int)i, bq = q;
        for (int rs = -1; rs <= 1; ++rs) {
            int nr = row + rs;
            for (int cs = -1; cs <= 1; ++cs) {
                if (rs == 0 && cs == 0) continue;
                int n = nr * W + wrap_col(col + cs, W);
                int qn = qkey(g[n]);
                if (qn < bq || (qn == bq && qn < q && n < best)) {
                    bq = qn;
                    best = n;
                }
            }
        }
        cls[i] = C_OPEN;
        f[i] = INFINITY;
        ptr[i] = best;
    }
}

// (1) pointer jumping to the chain's root, in place: p[i] <- p[p[i]]. Whatever a concurrent update
// lets a thread read is an ancestor of i on its chain, so the pass only jumps further, and a pass
// that changes no pointer leaves every cell on its root. `changed` is set when some pointer moved.
__global__ void k_jump(int* __restrict__ p, size_t N, int* __restrict__ changed) {
    bool moved = false;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x) {
        const int o = p[i];
        const int n = p[o];
        if (n != o) {
            p[i] = n;
            moved = true;
        }
    }
    if (__any_sync(0xFFFFFFFFu, moved) && (threadIdx.x & 31) == 0) atomicOr(changed, 1);
}

__global__ void k_mark_drained(const int* __restrict__ root, const float* __restrict__ g, size_t N,
                               uint8_t* __restrict__ cls, float* __restrict__ f) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x) {
        if (cls[i] != C_OPEN) continue;
        uint8_t rc = cls[root[i]];
        if (rc == C_WATER || rc == C_SEED) {
            cls[i] = C_DRAINED;
            f[i] = g[i];
        }
    }
}

// (2) tile relaxation. A CTA takes a 32x32 tile, loads f and g with a one-cell halo, relaxes its
// OPEN cells to local convergence, and writes back what fell. PINNED cells take their designated
// parent instead of the minimum. Returns (in every thread) whether a border cell fell or the tile
// is still moving: then it and its neighbours go on the next pass's list.
struct TileSmem {
    float sf[T + 2][T + 3];
    float sg[T][T + 1];
    uint8_t sc[T][T];
    int any_border;
};

__device__ __forceinline__ bool relax_tile(TileSmem& sm, int tile, float* __restrict__ f, const float* __restrict__ g,
                           const uint8_t* __restrict__ cls, const int* __restrict__ pin_parent, int W, int H,
                           int tiles_x, int max_sweeps) {
    const int ty0 = (tile / tiles_x) * T, tx0 = (tile % tiles_x) * T;
    auto& sf = sm.sf;
    auto& sg = sm.sg;
    auto& sc = sm.sc;
    const int lx = threadIdx.x & 31, ly = threadIdx.x >> 5;   // 32 x 8
    for (int i = threadIdx.x; i < (T + 2) * (T + 2); i += 256) {
        int yy = i / (T + 2), xx = i % (T + 2);
        int gy = ty0 + yy - 1;
        float v = INFINITY;
        // L1-bypassing loads: neighbouring tiles on other SMs wrote these in earlier passes of the
        // same launch, and a stale L1 line could make the tile look settled.
        if (gy >= 0 && gy < H) v = __ldcg(f + (size_t)gy * W + wrap_col(tx0 + xx - 1, W));
        sf[yy][xx] = v;
    }
    for (int i = threadIdx.x; i < T * T; i += 256) {
        int yy = i / T, xx = i % T;
        int gy = ty0 + yy, gx = tx0 + xx;
        bool in = gy < H && gx < W;
        sg[yy][xx] = in ? g[(size_t)gy * W + gx] : 0.0f;
        sc[yy][xx] = in ? cls[(size_t)gy * W + gx] : (uint8_t)C_WATER;
    }
    __syncthreads();
    bool border_changed = false;
    int unsettled = 1;
    for (int sweep = 0; sweep < max_sweeps && unsettled; ++sweep) {
        bool changed = false;
        for (int yy = ly; yy < T; yy += TH) {
            uint8_t c = sc[yy][lx];
            if (c != C_OPEN && !follows_parent(c)) continue;
            int gy = ty0 + yy;
            float gn = sg[yy][lx];
            float best = sf[yy + 1][lx + 1];
            if (c == C_OPEN) {
                for (int rs = -1; rs <= 1; ++rs) {
                    int ny = gy + rs;
                    if (ny < 0 || ny >= H) continue;
                    for (int cs = -1; cs <= 1; ++cs) {
                        if (rs == 0 && cs == 0) continue;
                        float fm = sf[yy + 1 + rs][lx + 1 + cs];
                        float v = phi(fm, gn);
                        if (v < best) best = v;
                    }
                }
            } else {
                int p = pin_parent[(size_t)gy * W + tx0 + lx];
                int pr = pdiv(p, W), pc = pmod(p, W);
                int dy = pr - gy;
                int dx = pc - (tx0 + lx);
                if (dx > 1) dx -= W;
                if (dx < -1) dx += W;
                float v = phi(sf[yy + 1 + dy][lx + 1 + dx], gn);
                if (v != best) best = v;   // a pinned cell follows its parent up as well as down
            }
            if (best != sf[yy + 1][lx + 1]) {
                sf[yy + 1][lx + 1] = best;
                changed = true;
                // A border cell, or the last column when the grid is narrower than a tile (its
                // east neighbour wraps to a column this tile only sees through its halo).
                if (yy == 0 || yy == T - 1 || lx == 0 || lx == T - 1 || tx0 + lx == W - 1) border_changed = true;
            }
        }
        unsettled = __syncthreads_or(changed);
    }
    // Still moving after the sweep budget: run this tile again next pass.
    const bool again = __syncthreads_or(border_changed) || unsettled;
    for (int yy = ly; yy < T; yy += TH) {
        int gy = ty0 + yy, gx = tx0 + lx;
        if (gy >= H || gx >= W) continue;
        uint8_t c = sc[yy][lx];
        if (c != C_OPEN && !follows_parent(c)) continue;
        float v = sf[yy + 1][lx + 1];
        size_t idx = (size_t)gy * W + gx;
        if (__ldcg(f + idx) != v) f[idx] = v;
    }
    __syncthreads();   // the shared tile is free for the next one
    return again;
}

// The relaxation passes in one cooperative launch. Pass p takes the tiles of list[p & 1] (each marked
// in mark[p & 1]); a tile that must run again puts itself and its 8 neighbours on the other list,
// once each (the mark), and clears its own mark for the list after next. A grid barrier separates
// the passes; the loop ends when a pass leaves the next list empty, or at max_passes (timed_out).
struct RelaxArgs {
    float* f;
    const float* g;
    const uint8_t* cls;
    const int* pin;
    int W, H, tiles_x, tiles_y;
    int* list[2];
    int* mark[2];
    int* count;   // [2]
    int* timed_out;
    int max_passes;
};

__global__ void __launch_bounds__(256) k_relax_passes(RelaxArgs a) {
    cgr::grid_group grid = cgr::this_grid();
    __shared__ TileSmem sm;
    int pass = 0;
    for (; pass < a.max_passes; ++pass) {
        const int cur = pass & 1, nxt = cur ^ 1;
        const int n = *(volatile int*)&a.count[cur];
        if (n == 0) break;
        for (int t = blockIdx.x; t < n; t += gridDim.x) {
            const int tile = __ldcg(a.list[cur] + t);
            if (threadIdx.x == 0) a.mark[cur][tile] = 0;
            if (relax_tile(sm, tile, a.f, a.g, a.cls, a.pin, a.W, a.H, a.tiles_x, 4 * T) && threadIdx.x < 9) {
                const int dy = (int)threadIdx.x / 3 - 1, dx = (int)threadIdx.x % 3 - 1;
                const int y = tile / a.tiles_x + dy;
                if (y >= 0 && y < a.tiles_y) {
                    const int nb = y * a.tiles_x + (tile % a.tiles_x + dx + a.tiles_x) % a.tiles_x;
                    if (atomicExch(&a.mark[nxt][nb], 1) == 0) a.list[nxt][atomicAdd(&a.count[nxt], 1)] = nb;
                }
            }
        }
        grid.sync();
        if (blockIdx.x == 0 && threadIdx.x == 0) a.count[cur] = 0;
        grid.sync();
    }
    if (pass == a.max_passes && blockIdx.x == 0 && threadIdx.x == 0 && *(volatile int*)&a.count[pass & 1] != 0)
        *a.timed_out = 1;
}

// A tile is on the first pass's list if it holds a cell still to settle (a level reset to +inf).
__global__ void k_tiles_with_open(const uint8_t* __restrict__ cls, const float* __restrict__ f, int W, int H,
                                  int tiles_x, int* __restrict__ mark, int* __restrict__ list,
                                  int* __restrict__ count) {
    int tile = blockIdx.x;
    const int ty0 = (tile / tiles_x) * T, tx0 = (tile % tiles_x) * T;
    int has = 0;
    for (int i = threadIdx.x; i < T * T; i += blockDim.x) {
        int gy = ty0 + i / T, gx = tx0 + i % T;
        if (gy < H && gx < W) {
            size_t c = (size_t)gy * W + gx;
            if (cls[c] >= C_OPEN && isinf(f[c])) has = 1;
        }
    }
    has = __syncthreads_or(has);
    if (threadIdx.x == 0) {
        mark[tile] = has ? 1 : 0;
        if (has) list[atomicAdd(count, 1)] = tile;
    }
}

// (3) the exact parent check. For each OPEN/PINNED cell: its least-Q neighbours; if they give
// different levels, the reference's parent is the lowest-index one among those that entered the
// level from below. Writes the parent into pin_parent (and marks the cell PINNED) when that parent
// disagrees with the current level.
__global__ void k_check_ties(const float* __restrict__ f, const float* __restrict__ g, uint8_t* __restrict__ cls,
                             int* __restrict__ pin_parent, int W, int H, FillCounters* cnt) {
    size_t N = (size_t)W * H;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x) {
        uint8_t c = cls[i];
        if (c != C_OPEN && c != C_PINNED) continue;   // EXACT cells were ordered by replaying their level
        const int row = pdiv((int)i, W), col = pmod((int)i, W);
        float gn = g[i];
        int qmin = INT_MAX;
        for (int rs = -1; rs <= 1; ++rs) {
            int nr = row + rs;
            if (nr < 0 || nr >= H) continue;
            for (int cs = -1; cs <= 1; ++cs) {
                if (rs == 0 && cs == 0) continue;
                int n = nr * W + wrap_col(col + cs, W);
                int q = qkey(f[n]);
                if (q < qmin) qmin = q;
            }
        }
        float v0 = 0.0f;
        bool first = true, differ = false, inside_level = false;
        int pick = INT_MAX;
        for (int rs = -1; rs <= 1; ++rs) {
            int nr = row + rs;
            if (nr < 0 || nr >= H) continue;
            for (int cs = -1; cs <= 1; ++cs) {
                if (rs == 0 && cs == 0) continue;
                int n = nr * W + wrap_col(col + cs, W);
                float fm = f[n];
                if (qkey(fm) != qmin) continue;
                float v = phi(fm, gn);
                if (first) v0 = v, first = false;
                else if (v != v0) differ = true;
                if (n < pick) pick = n;
                // Reached inside its own key level: an unraised land cell whose least-Q neighbour
                // shares its key. Water and the polar outlets are in the heap from the start.
                uint8_t cm = cls[n];
                if ((cm == C_OPEN || follows_parent(cm) || cm == C_DRAINED) && fm == g[n]) {
                    int mr = pdiv(n, W), mc = pmod(n, W), mq = INT_MAX;
                    for (int a = -1; a <= 1; ++a) {
                        int r2 = mr + a;
                        if (r2 < 0 || r2 >= H) continue;
                        for (int b = -1; b <= 1; ++b) {
                            if (a == 0 && b == 0) continue;
                            int q2 = qkey(f[r2 * W + wrap_col(mc + b, W)]);
                            if (q2 < mq) mq = q2;
                        }
                    }
                    if (mq == qmin) inside_level = true;
                }
            }
        }
        if (!differ) {
            // No tie (any more): the least neighbour decides; release a pin from an earlier pass.
            if (c == C_PINNED) {
                cls[i] = C_OPEN;
                if (f[i] != v0) {
                    atomicAdd(&cnt->repaired, 1ull);
                    atomicMin(&cnt->repair_level, qmin);
                }
            }
            continue;
        }
        atomicAdd(&cnt->ties, 1ull);
        if (inside_level) {
            // Only the level's own pops can order this tie: replay the lowest such level.
            atomicAdd(&cnt->unresolved, 1ull);
            atomicMin(&cnt->min_level, qmin);
            continue;
        }
        float want = phi(f[pick], gn);
        if (c != C_PINNED || pin_parent[i] != pick) {
            pin_parent[i] = pick;
            cls[i] = C_PINNED;
            if (want != f[i]) {
                atomicAdd(&cnt->repaired, 1ull);
                atomicMin(&cnt->repair_level, qmin);
            }
        }
    }
}

// Resets every unsettled cell at or above key level Q to +inf. A cell's level depends only on its
// parent chain, which runs through strictly lower levels, so cells below Q are already final.
__global__ void k_reset_from(const uint8_t* __restrict__ cls, float* __restrict__ f, size_t N, int Q) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x)
        if ((cls[i] == C_OPEN || follows_parent(cls[i])) && qkey(f[i]) >= Q) f[i] = INFINITY;
}

// The cells whose current level has a key in [Q, Qmax] (the candidates for the replay's heap), up
// to cap: land, and water touching land (open water elsewhere never enters the flood).
__global__ void k_gather_level(const float* __restrict__ f, const uint8_t* __restrict__ cls, int W, int H, int Q,
                               int Qmax, int* __restrict__ list, int* __restrict__ count, int cap) {
    size_t N = (size_t)W * H;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x) {
        const int q = qkey(f[i]);
        if (q < Q || q > Qmax) continue;
        if (cls[i] == C_WATER) {
            const int row = pdiv((int)i, W), col = pmod((int)i, W);
            bool touches = false;
            for (int rs = -1; rs <= 1 && !touches; ++rs) {
                int nr = row + rs;
                if (nr < 0 || nr >= H) continue;
                for (int cs = -1; cs <= 1; ++cs)
                    if ((rs || cs) && cls[nr * W + wrap_col(col + cs, W)] != C_WATER) touches = true;
            }
            if (!touches) continue;
        }
        int s = atomicAdd(count, 1);
        if (s < cap) list[s] = (int)i;
    }
}

// In the heap before key level Q opens: water and the polar outlets (pushed at the start) and every
// cell with a neighbour below Q (pushed when that neighbour was popped). Lower levels are exact here.
__device__ bool entered_below(const float* f, const uint8_t* cls, int W, int H, int cell, int Q) {
    uint8_t c = cls[cell];
    if (c == C_WATER || c == C_SEED) return true;
    int row = pdiv(cell, W), col = pmod(cell, W);
    for (int rs = -1; rs <= 1; ++rs) {
        int nr = row + rs;
        if (nr < 0 || nr >= H) continue;
        for (int cs = -1; cs <= 1; ++cs) {
            if (rs == 0 && cs == 0) continue;
            if (qkey(f[nr * W + wrap_col(col + cs, W)]) < Q) return true;
        }
    }
    return false;
}

// Whether each cell was in the heap before key level Q opened (entered_below), for the replay: a
// cell's answer depends only on levels below Q, which the replay never writes.
__global__ void k_entered_below(const float* __restrict__ f, const uint8_t* __restrict__ cls, int W, int H, int Q,
                                uint8_t* __restrict__ eb) {
    const size_t N = (size_t)W * H;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x)
        eb[i] = entered_below(f, cls, W, H, (int)i, Q) ? 1 : 0;
}

// Replays key levels Q..Qmax of the priority flood (FlowRouting.kt:93-109) with one thread: a
// min-heap on (key, index), seeded with the gathered cells that entered it from below Q (those
// were pushed, with their final levels, before level Q opened: lower levels are exact here). Each
// pop visits its neighbours in the reference's order, and each neighbour not yet visited takes its
// level from the popped cell and joins the heap, as the reference pushes it. Popping stops at the
// first key above Qmax. Every cell so reached gets its exact parent (class EXACT); a cell pushed
// with a key above Qmax has its final level too, its first popped neighbour being the one that
// reached it. Rewritten levels never fall below Q, so `entered_below` keeps its meaning throughout.
// Bounded by the heap's capacity (each cell is pushed at most once); an overflow is reported.
__global__ void k_replay_level(float* __restrict__ f, const float* __restrict__ g, uint8_t* __restrict__ cls,
                               int* __restrict__ pin, int* __restrict__ mark, int gen, const int* __restrict__ list,
                               const int* __restrict__ list_n, long long* __restrict__ heap, int cap, int W, int H,
                               int Q, int Qmax, const uint8_t* __restrict__ eb, FillCounters* cnt) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    int n = *list_n;
    if (n > cap) {
        cnt->overflow = 1;
        return;
    }
    int hs = 0;
    auto push = [&](long long v) -> bool {
        if (hs >= cap) return false;
        int s = hs++;
        heap[s] = v;
        while (s > 0) {
            int p = (s - 1) >> 1;
            if (heap[p] <= heap[s]) break;
            long long t = heap[p];
            heap[p] = heap[s];
            heap[s] = t;
            s = p;
        }
        return true;
    };
    auto pop = [&]() -> long long {
        long long top = heap[0];
        heap[0] = heap[--hs];
        int s = 0;
        while (true) {
            int l = 2 * s + 1;
            if (l >= hs) break;
            int r = l + 1;
            int m = (r < hs && heap[r] < heap[l]) ? r : l;
            if (heap[s] <= heap[m]) break;
            long long t = heap[m];
            heap[m] = heap[s];
            heap[s] = t;
            s = m;
        }
        return top;
    };
    auto key_of = [&](int cell) { return ((long long)qkey(f[cell]) << 32) | (unsigned)cell; };
    for (int k = 0; k < n; ++k)
        if (eb[list[k]] && !push(key_of(list[k]))) {
            cnt->overflow = 1;
            return;
        }
    while (hs > 0 && (int)(heap[0] >> 32) <= Qmax) {
        int x = (int)(pop() & 0xFFFFFFFFll);
        float fx = f[x];
        int row = pdiv(x, W), col = pmod(x, W);
        for (int rs = -1; rs <= 1; ++rs) {
            int nr = row + rs;
            if (nr < 0 || nr >= H) continue;
            for (int cs = -1; cs <= 1; ++cs) {
                if (rs == 0 && cs == 0) continue;
                int y = nr * W + wrap_col(col + cs, W);
                if (mark[y] == gen || eb[y]) continue;
                mark[y] = gen;
                float fy = phi(fx, g[y]);
                if (cls[y] != C_DRAINED) {
                    pin[y] = x;
                    cls[y] = C_EXACT;
                }
                f[y] = fy;
                if (!push(key_of(y))) {
                    cnt->overflow = 1;
                    return;
                }
            }
        }
    }
}

}  // namespace

cg_status fill_depressions_dev(cg_ctx* ctx, int W, int H, const uint8_t* d_land, const float* d_rel, float* d_filled,
                               int64_t* ties, int64_t* unresolved) {
    size_t N = (size_t)W * H;
    cudaStream_t sm = ctx->stream;
    CG_BUF(uint8_t, d_cls, ctx, S_FILLFLAG, N);
    CG_BUF(int, d_ptr, ctx, S_PTR, N);
    CG_BUF(int, d_moved, ctx, S_PTR2, 2);   // the jumping passes' change flags
    CG_BUF(int, d_pin, ctx, S_FILLQ, N);
    int tiles_x = (W + T - 1) / T, tiles_y = (H + T - 1) / T, tiles = tiles_x * tiles_y;
    // Two tile lists and their marks, two list counts, the timeout flag (zeroed before each relaxation).
    CG_BUF(int, d_marks, ctx, S_TILEFLAG, 2 * (size_t)tiles);
    CG_BUF(int, d_lists, ctx, S_FILLLIST, 2 * (size_t)tiles + 4);
    RelaxArgs ra;
    ra.f = d_filled;
    ra.g = d_rel;
    ra.cls = d_cls;
    ra.pin = d_pin;
    ra.W = W;
    ra.H = H;
    ra.tiles_x = tiles_x;
    ra.tiles_y = tiles_y;
    ra.list[0] = d_lists;
    ra.list[1] = d_lists + tiles;
    ra.count = d_lists + 2 * (size_t)tiles;
    ra.timed_out = ra.count + 2;
    ra.mark[0] = d_marks;
    ra.mark[1] = d_marks + tiles;
    ra.max_passes = 4 * (tiles_x + tiles_y) + 64;
    int per_sm = 0;
    CG_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_relax_passes, 256, 0));
    if (per_sm < 1) return fail(ctx, CG_CUDA, "k_relax_passes cannot be resident");
    const int relax_grid = ctx->num_sms * std::min(per_sm, 8);
    CG_BUF(FillCounters, d_cnt, ctx, S_FILLF, 1);
    int grid = ctx->num_sms * 8;
    CG_CUDA(ctx, cudaMemsetAsync(d_cnt, 0, sizeof(FillCounters), sm));
    CG_LAUNCH(ctx) k_fill_init<<<grid, 256, 0, sm>>>(d_land, d_rel, W, H, d_cls, d_filled, d_ptr);
    // Chains are at most N long: ceil(log2 N) jumps reach every root; most worlds need far fewer, so
    // the passes stop at the first that moves no pointer (checked every second pass).
    int jumps = 1;
    while (((size_t)1 << jumps) < N) ++jumps;
    for (int j = 0; j < jumps + 2; j += 2) {
        CG_CUDA(ctx, cudaMemsetAsync(d_moved, 0, 2 * sizeof(int), sm));
        CG_LAUNCH(ctx) k_jump<<<grid, 256, 0, sm>>>(d_ptr, N, d_moved);
        CG_LAUNCH(ctx) k_jump<<<grid, 256, 0, sm>>>(d_ptr, N, d_moved + 1);
        int moved[2] = {0, 0};
        CG_CUDA(ctx, cudaMemcpyAsync(moved, d_moved, sizeof(moved), cudaMemcpyDeviceToHost, sm));
        CG_CUDA(ctx, cudaStreamSynchronize(sm));
        if (!moved[1]) break;
    }
    CG_LAUNCH(ctx) k_mark_drained<<<grid, 256, 0, sm>>>(d_ptr, d_rel, N, d_cls, d_filled);
    CG_CHECK_LAUNCH(ctx);

    // Scratch of the level replays: a generation mark per cell, the level's cells and the heap, each
    // sized for every cell of the grid (a key level can hold any share of the grid).
    const int cap = (int)N;
    CG_BUF(int, d_mark, ctx, S_SCRATCH3, N);
    CG_BUF(uint8_t, d_eb, ctx, S_FILLEB, N);
    CG_BUF(int, d_replay, ctx, S_CG4, 3 * (size_t)cap + 4);
    int* d_list = d_replay;
    long long* d_heap = (long long*)(d_replay + cap + (cap & 1));   // 8-byte aligned
    int* d_list_n = d_replay + 3 * (size_t)cap + 2;
    CG_CUDA(ctx, cudaMemsetAsync(d_mark, 0, N * sizeof(int), sm));
    int gen = 0;

    FillCounters hc;
    int64_t tie_total = 0, unresolved_total = 0;
    int replays = 0;
    // Each pass either settles, pins tie parents by the index rule, or replays the lowest level
    // holding a tie the index rule cannot order; the cap is a guard, not the expected exit.
    const int max_repairs = 256;
    for (int repair = 0; repair <= max_repairs; ++repair) {
        CG_CUDA(ctx, cudaMemsetAsync(d_lists, 0, (2 * (size_t)tiles + 4) * sizeof(int), sm));
        CG_CUDA(ctx, cudaMemsetAsync(d_marks, 0, 2 * (size_t)tiles * sizeof(int), sm));
        CG_LAUNCH(ctx) k_tiles_with_open<<<tiles, 256, 0, sm>>>(d_cls, d_filled, W, H, tiles_x, ra.mark[0], ra.list[0],
                                                                ra.count);
        CG_CHECK_LAUNCH(ctx);
        // Relax until no tile changes, in one cooperative launch. Bounded: every pass lowers some level
        // or stops, and levels only take values from a finite set; the cap is a guard, not the exit.
        {
            void* kargs[] = {&ra};
            ctx->launches++;
            CG_CUDA(ctx, cudaLaunchCooperativeKernel((void*)k_relax_passes, relax_grid, 256, kargs, 0, sm));
        }
        int timed_out = 0;
        CG_CUDA(ctx, cudaMemcpyAsync(&timed_out, ra.timed_out, sizeof(int), cudaMemcpyDeviceToHost, sm));
        CG_CUDA(ctx, cudaStreamSynchronize(sm));
        if (timed_out) return fail(ctx, CG_TIMEOUT, "fill relaxation did not settle in %d passes", ra.max_passes);
        FillCounters zero{};
        zero.min_level = INT_MAX;
        zero.repair_level = INT_MAX;
        CG_CUDA(ctx, cudaMemcpyAsync(d_cnt, &zero, sizeof(zero), cudaMemcpyHostToDevice, sm));
        CG_LAUNCH(ctx) k_check_ties<<<grid, 256, 0, sm>>>(d_filled, d_rel, d_cls, d_pin, W, H, d_cnt);
        CG_CHECK_LAUNCH(ctx);
        CG_CUDA(ctx, cudaMemcpyAsync(&hc, d_cnt, sizeof(hc), cudaMemcpyDeviceToHost, sm));
        CG_CUDA(ctx, cudaStreamSynchronize(sm));
        if (repair == 0) tie_total = (int64_t)hc.ties;
        unresolved_total = (int64_t)hc.unresolved;
        if (hc.repaired == 0 && hc.unresolved == 0) break;
        if (repair == max_repairs) {
            unresolved_total += (int64_t)hc.repaired;
            break;
        }
        int from = hc.repaired ? hc.repair_level : INT_MAX;
        if (hc.unresolved) {
            // Replay from the lowest key level Q whose ties only its own pops can order, or from the
            // lowest level at which a pin changed in this pass if that is lower: below it every level
            // is final (a pin's parent sits at or above that level), so the replay's seeds (cells
            // entered from below Q) hold their final levels, and the replay orders the pinned cells it
            // reaches exactly too. The first replays of a call take that level alone; later ones run
            // on through a span of key levels that doubles up to kReplaySpan: a broad flat raises a
            // staircase of levels, each with such ties, and one replay then orders many of them.
            const int Q = hc.repaired ? std::min(hc.min_level, hc.repair_level) : hc.min_level;
            const int span = replays < 8 ? 0 : std::min(1 << std::min(replays - 8, 12), kReplaySpan);
            const int Qmax = Q + span;
            ++replays;
            ++gen;
            CG_CUDA(ctx, cudaMemsetAsync(d_list_n, 0, sizeof(int), sm));
            CG_LAUNCH(ctx) k_gather_level<<<grid, 256, 0, sm>>>(d_filled, d_cls, W, H, Q, Qmax, d_list, d_list_n, cap);
            CG_LAUNCH(ctx) k_entered_below<<<grid, 256, 0, sm>>>(d_filled, d_cls, W, H, Q, d_eb);
            CG_LAUNCH(ctx) k_replay_level<<<1, 32, 0, sm>>>(d_filled, d_rel, d_cls, d_pin, d_mark, gen, d_list, d_list_n,
                                                            d_heap, cap, W, H, Q, Qmax, d_eb, d_cnt);
            CG_CHECK_LAUNCH(ctx);
            int overflow = 0;
            CG_CUDA(ctx, cudaMemcpyAsync(&overflow, &d_cnt->overflow, sizeof(int), cudaMemcpyDeviceToHost, sm));
            CG_CUDA(ctx, cudaStreamSynchronize(sm));
            if (overflow) {   // cannot happen with cap = N; kept as a guard
                unresolved_total += 1;
                break;
            }
            if (Q < from) from = Q;
        }
        // Recompute the levels at and above the lowest one that changed.
        CG_LAUNCH(ctx) k_reset_from<<<grid, 256, 0, sm>>>(d_cls, d_filled, N, from);
    }
    if (ties) *ties = tie_total;
    if (unresolved) *unresolved = unresolved_total;
    if (unresolved_total > 0)
        return fail(ctx, CG_INEXACT, "fillDepressions left %lld quantised-key ties unordered", (long long)unresolved_total);
    return CG_OK;
}

}  // namespace cg
