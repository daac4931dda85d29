// Profile P2's deposition on the device: the walk of HydraulicErosion.apply (HydraulicErosion.kt:
// 1068-1349) with its sea lobes and lake fans (DeltaFan.kt growFan), settle (1351-1364) and the
// closing mouths pass (openMouths, 1804-1892), each bit for bit the reference's.
//
// The reference walks the round's drainage order one cell after another. That order is level-major
// (a cell's rank sorts by its Kahn level, then by its drainage key), so the walk runs level by level
// from the sources, in one cooperative launch per round with grid barriers between the steps of a
// level:
//  A. every cell of the level does its own walk at once (HydraulicErosion.kt:1068-1186): a cell reads
//     only its own state and its donors', which sit on lower levels. What arrives is the notch's
//     hand-off plus the donors' hand-offs added in rank order, the reference's double additions in
//     the reference's order. A cell whose mouth has something to lay (a sea lobe or a lake fan with a
//     budget and an open apex) is listed, in rank order per CTA segment.
//  B. the listed mouths lay in rank order wherever two of them could see each other. A lake fan's
//     admission (its best-first growth inside the rim) reads only fixed fields (the land, the lake's
//     depth), so every lake fan of the round is admitted before the walk, a thread each with its own
//     visited bits over the box its rim can reach, and its admitted cells sorted by distance (the
//     laying heap's pop order) into a pool. A chunk of mouths gets a laying schedule: the lake fans'
//     (fan, cell) pairs and the sea lobes' (lobe, box tile) pairs grouped by cell or tile, each mouth
//     counting the earlier mouths on its cells or tiles and learning the next ones. A mouth's warp
//     waits for its count to reach 0 (a bounded poll inside the cooperative launch), lays (a lake fan
//     as a scan of its sorted cells, 32 needs at a time; a sea lobe whole on lane 0, its admission
//     reading the sediment earlier lobes laid), and releases the next ones. Every deposit is logged,
//     and the level's log is assembled in rank order from the mouths' own logs.
//  C. a fan changes only sea cells and ponded land, which no own walk reads, except (a) a ponded cell
//     of the fan's own level ranked after it, whose settled height took its own subtraction before
//     the fan's addition instead of after: its settled height is replayed in rank order from its
//     group of log entries; and (b) a donor whose settled height a later (dry) cell of the level read
//     in its headroom. Such a cell's own walk is taken again with its donors as the reference's walk
//     shows them at its rank. Nothing else of the level reads that cell, so where its step hands
//     everything on the fix is local; where it has a mouth, its fan changes with it: every fan from
//     its rank on is undone (over the grid, from the log), the cell refitted, and those fans laid
//     again, and the search, an atomic minimum over the log, repeats past it. Both are rare; the
//     level schedule itself is shown on the host to give the reference walk's bits
//     (tests/native/deposit_host.cpp).
// Settle is elementwise, and the mouths pass reads only each cell's receiver, so it runs receivers
// first, level by level from the top, like the incision.
#include <algorithm>
#include <climits>
#include <cooperative_groups.h>
#include <vector>

#include "cg_common.cuh"
#include "cg_deposit.cuh"
#include "cg_internal.h"
#include "cg_params.h"
#include "cg_util.h"

namespace cg {

namespace cgr = cooperative_groups;
using namespace dep;

namespace {

constexpr int kThreads = 256;
constexpr int kTile = 16;   // a sea lobe's box is scheduled in tiles of kTile x kTile cells
constexpr int kNoTouch = 0x7F7F7F7F;   // `first`'s resting value (a byte-wise memset)
constexpr long long kSpinLimit = 1LL << 24;   // a lake fan's wait for its turn, in polls (seconds)

// Control words of a walk.
enum {
    W_EVENTS = 0, W_ERROR = 1, W_MOUTH_ID = 2, W_GEN = 3, W_ABORT = 4, W_REPLAYED = 5, W_WAVEBASE = 6, W_WAVES = 7,
    W_WAIT0 = 8, W_WAIT1 = 9, W_REFITTED = 10, W_ESTART = 11, W_DONE = 12, W_RELAID = 13, W_PAIRS = 14, W_DISTINCT = 15,
    W_CHECK_SITE = 16, W_CHECK_VALUE = 17, W_CHECK_BOUND = 18, W_NDONOR = 19,
    W_REFITGEN = 20, W_BEST = 21, W_TOUCHN = 22, W_NREPLAY = 23, W_NREFIT = 24, W_FGEN = 25, W_NLAKE = 26,
    W_NSEA = 27, W_SEAWAIT0 = 28, W_SEAWAIT1 = 29, W_CUT = 30, W_RC = 31, W_WORDS = 32
};

struct WalkDev {
    Params p;
    Fields f;
    const int* order;       // land cells in drainage order (rank order)
    const int* rank_of;     // per cell
    const long long* key;   // per cell: level << 32 | deepest source
    const int* level_start; // [levels + 1]
    int levels;
    const double* load;     // per cell: the notch's hand-off
    double* handoff;        // per cell: what a cell hands its receiver
    uint8_t* used;          // per cell: its own walk read its donors' settled heights
    float* s0;              // per rank: settled height before the own walk
    float* d0;              // per rank: sediment before the own walk
    double* ev_carried;     // per rank: what a listed mouth carries
    int8_t* ev_kind;        // per rank: SEA or LAKE
    int* seg_events;        // per rank: listed ranks, compacted within each CTA's segment
    int* seg_count;         // per CTA
    int* seg_off;           // per CTA + 1: its listed mouths' first place in `events`
    int* seg_part;          // per CTA + 1: a grid-wide scan's slice sums
    int* events;            // the level's listed ranks, dense, in rank order
    // The round's lake fans, admitted before the walk (k_admit_lakes): per candidate mouth cell its
    // admitted cells sorted by distance and each one's level less its terrain, in a pool.
    const int* cand_of;     // per cell: its candidate index, -1 if it is no lake mouth
    const int* cand_n;      // per candidate: admitted cells
    const long long* cand_off;   // per candidate: first pool entry
    const int* pool_cells;
    const double* pool_base;
    int ncand;
    long long pool_total;
    // The mouths of a chunk, `slots` of them at a time.
    int slots, cap, box_words;
    long long* slot_off;    // per slot: its fan's first pool entry
    int* slot_n;            // per slot: admitted cells (a lake fan) or box tiles (a sea lobe)
    int* slot_box;          // per slot, a sea lobe's box in tiles: first column (may be < 0), first row, columns, rows
    int* slot_state;        // per slot: 1 while a lake fan waits to lay, 2 while a sea lobe waits, else 0
    double* slot_laid;      // per slot: what its fan laid
    Touch* slot_touch;      // per slot: its fan's deposits, `cap` entries
    int* slot_touch_n;
    // A chunk's laying schedule: each (fan, admitted cell) pair, grouped by cell, knows the fan that
    // follows it on that cell in rank order; a fan lays once every fan before it on its cells has.
    int pair_cap;
    int* poff;              // per slot + 1: its first pair
    int* pair_fan;          // per pair: its slot
    int* pair_cell;
    int* pair_pos;          // per pair: its place in its cell's group (arrival order)
    int* pair_succ;         // per pair: the slot of the next fan on its cell, or -1
    int* group;             // pairs grouped by cell
    int* dcell;             // the chunk's distinct cells
    int* doff;              // per distinct cell + 1: its group's first entry
    int* cell_cnt;          // per cell: pairs on it (0 outside a chunk's scheduling)
    int* cell_d;            // per cell: its distinct index (valid for the chunk's cells)
    int* blockers;          // per slot: earlier fans still to lay on its cells
    // The sea lobes' boxes in tiles of kTile x kTile cells (a tile's schedule id is N + its index), and
    // each warp's heap (a sea lobe runs on its warp's lane 0): heap_warps heaps of `cap` entries.
    int tiles_x, tiles_y, box_x, box_y, heap_warps;
    uint32_t* warp_bits;    // per warp: a sea lobe's visited bits over its box (box_words)
    int* heap_cells;
    float* heap_keys;
    float* heap_pens;
    int* heap_admitted;
    int* stamp;             // per cell: the stage's fan stamps
    // The level's fan deposits, for the repairs.
    Touch* touches;
    int touch_cap;
    int* ev_touch;          // per listed mouth (dense index): its first touch; [n + 1]
    int* mark;              // per cell: the generation that listed it for a replay
    int* replay;            // cells to replay
    int* refit;             // cells to refit
    int* rlist;             // the log's entries on the cells to replay, grouped by cell (touch_cap)
    int* first;             // per cell: its earliest log entry being undone (kNoTouch at rest)
    int* touch_ev;          // per level-log entry: its event's index
    int* roff;              // per cell to replay + 1: its group's first entry
    float* acc;             // per cell: a replayed settled height
    uint8_t* own_done;      // per cell: the replay has taken the cell's own subtraction
    int* words;             // W_* control words
    unsigned long long* timers;   // T_*: nanoseconds of the walk's parts, kept by CTA 0's thread 0
};

// The walk's parts that CTA 0's thread 0 times (it runs every serial part and meets every grid barrier):
// own walks and listing, schedules, the laying of lake fans and sea lobes, the logs, the repairs.
enum { T_WALKS = 0, T_SCHEDULE = 1, T_LAKES = 2, T_SEAS = 3, T_REPAIRS = 4, T_COUNT = 5 };

__device__ __forceinline__ unsigned long long now_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ int level_of_cell(const WalkDev& w, int c) { return (int)(w.key[c] >> 32); }

// What arrives at `c`: the notch's hand-off, then each donor's hand-off in rank order.
__device__ double arriving(const WalkDev& w, int c) {
    const int W = w.p.W, H = w.p.H;
    const int col = c % W, row = c / W;
    int donors[8], ranks[8], n = 0;
    for (int rs = -1; rs <= 1; ++rs) {
        const int nr = row + rs;
        if (nr < 0 || nr >= H) continue;
        for (int cs = -1; cs <= 1; ++cs) {
            if (rs == 0 && cs == 0) continue;
            const int d = nr * W + ((col + cs) & (W - 1));
            if (w.f.dirs[d] != c || !w.f.land[d]) continue;
            const int rk = w.rank_of[d];
            int j = n++;
            while (j > 0 && ranks[j - 1] > rk) {
                ranks[j] = ranks[j - 1];
                donors[j] = donors[j - 1];
                --j;
            }
            ranks[j] = rk;
            donors[j] = d;
        }
    }
    double carried = w.load[c];
    for (int k = 0; k < n; ++k) carried = __dadd_rn(carried, w.handoff[donors[k]]);
    return carried;
}

// Whether a cell's mouth has anything to lay: a budget and an apex the fan accepts.
__device__ bool mouth_live(const WalkDev& w, int c, double carried, int kind) {
    const double budget = mouth_budget(w.p, w.f, c, carried, kind);
    return budget > 0.0 && mouth_accepts(w.p, w.f, kind == SEA, w.f.dirs[c]);
}

__device__ Heap warp_heap(const WalkDev& w, int gwarp) {
    const size_t o = (size_t)gwarp * w.cap;
    return Heap{w.heap_cells + o, w.heap_keys + o, w.heap_pens + o, w.heap_admitted + o, w.cap, 0, 0};
}

// The round's lake mouths and their fans' admissions, ahead of the walk. A lake fan's admission (its
// best-first growth inside the rim, DeltaFan.growFan) reads only fixed fields: the land, the lake's
// depth (ground less relative height) and the rim, which depends on the mouth and its receiver. So
// every cell whose step ends in a lake (kind LAKE: dry, its land receiver ponded) has its fan admitted
// once per round, all at once, whether or not the walk later gives it anything to lay.
struct AdmitDev {
    Params p;
    Fields f;
    int cap, box_words;
    const int* cand;        // candidate mouth cells
    int ncand;
    int* cand_n;            // pass 1 writes the admitted counts
    const long long* cand_off;   // pass 2 reads the pool offsets
    int* pool_cells;
    double* pool_base;
    int* h_cells;           // per thread: a heap of `cap` entries and the visited bits of a box
    float* h_keys;
    float* h_pens;
    int* h_admitted;
    uint32_t* h_bits;
    int fill;               // 0: count, 1: fill the pool
    int* err;
};

__global__ void k_lake_candidates(Params p, Fields f, int N, int* __restrict__ cand, int* __restrict__ ncand,
                                  int* __restrict__ cand_of) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < N; c += gridDim.x * blockDim.x) {
        int idx = -1;
        const int r = f.dirs[c];
        if (f.land[c] && r >= 0 && f.land[r] && !ponded(p, f, c) && ponded(p, f, r)) {
            idx = atomicAdd(ncand, 1);
            cand[idx] = c;
        }
        cand_of[c] = idx;
    }
}

// A candidate's admission; pass 1 counts its admitted cells, pass 2 writes them to the pool sorted by
// distance from the apex with the cell as the tie break (the laying heap's pop order), each with its
// level less its terrain (lay_admitted's need before the sediment).
__global__ void __launch_bounds__(128) k_admit_lakes(AdmitDev a) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int threads = gridDim.x * blockDim.x;
    int* cells = a.h_cells + (size_t)t * a.cap;
    float* keys = a.h_keys + (size_t)t * a.cap;
    float* pens = a.h_pens + (size_t)t * a.cap;
    int* admitted = a.h_admitted + (size_t)t * a.cap;
    uint32_t* bits = a.h_bits + (size_t)t * a.box_words;
    for (int i = t; i < a.ncand; i += threads) {
        const int c = a.cand[i];
        for (int j = 0; j < a.box_words; ++j) bits[j] = 0u;
        Rim m;
        mouth_rim(a.p, a.f, c, LAKE, m);
        int outside = 0;
        BoxVisited visited{bits, a.p.W, m.apex_column, m.apex_row, box_bx(a.p), box_by(a.p), &outside};
        Heap h{cells, keys, pens, admitted, a.cap, 0, 0};
        const int n = admit(a.p, a.f, m, false, visited, h);
        if (outside) atomicOr(a.err, 2);   // the rim reached past its box: cannot happen
        if (!a.fill) {
            a.cand_n[i] = n;
            continue;
        }
        h.size = 0;
        for (int k = 0; k < n; ++k) {
            const int x = admitted[k];
            const float co = rim_column_offset(m, x), ro = rim_row_offset(m, x);
            heap_push(h, x, sqrt_rn(co * co + ro * ro), 0.0f);
        }
        int* sorted = a.pool_cells + a.cand_off[i];
        double* base = a.pool_base + a.cand_off[i];
        int got = 0, x;
        float pen;
        while (heap_pop(h, x, pen)) {
            const float co = rim_column_offset(m, x), ro = rim_row_offset(m, x);
            const float distance = sqrt_rn(co * co + ro * ro);
            float fraction = distance / m.reach_cells;
            if (fraction > 1.0f) fraction = 1.0f;
            const float depth =
                2.0f * a.p.pond_depth * (1.0f + kLakeFanSlope * fraction) * (0.9f + 0.35f * cell_wobble(x));
            const float level = a.p.shoreline + (a.f.ground[x] - depth) * a.p.land_range;
            sorted[got] = x;
            base[got] = (double)level - (double)a.f.surface[x];
            ++got;
        }
    }
}

// Exclusive prefix sum of n 64-bit counts by one CTA, chunk after chunk; out[n] receives the total.
__global__ void __launch_bounds__(1024) k_scan64_one_block(const long long* __restrict__ in, long long* __restrict__ out,
                                                          int n) {
    __shared__ long long sh[1024];
    long long carry = 0;
    for (int base = 0; base < n; base += 1024) {
        const int i = base + (int)threadIdx.x;
        const long long v = i < n ? in[i] : 0;
        sh[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < 1024; o <<= 1) {
            const long long t = threadIdx.x >= (unsigned)o ? sh[threadIdx.x - o] : 0;
            __syncthreads();
            sh[threadIdx.x] += t;
            __syncthreads();
        }
        if (i < n) out[i] = carry + sh[threadIdx.x] - v;
        const long long chunk = sh[1023];
        __syncthreads();
        carry += chunk;
    }
    if (threadIdx.x == 0) out[n] = carry;
}

__global__ void k_widen_counts(const int* __restrict__ n, int count, long long* __restrict__ out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) out[i] = n[i];
}

// An exclusive prefix sum by one CTA (every thread of it calls this), chunk after chunk; out[n]
// receives the total. get(i) gives element i. sh is the CTA's shared scratch: no __restrict__ on it,
// which would let the compiler keep a thread's own sh entry in a register across the barriers that
// publish it to the other threads.
template <class Get>
__device__ void cta_exclusive_scan(Get get, int n, int* out, int* sh) {
    int carry = 0;
    for (int base = 0; base < n; base += kThreads) {
        const int i = base + (int)threadIdx.x;
        const int v = i < n ? get(i) : 0;
        sh[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < kThreads; o <<= 1) {
            const int t = threadIdx.x >= (unsigned)o ? sh[threadIdx.x - o] : 0;
            __syncthreads();
            sh[threadIdx.x] += t;
            __syncthreads();
        }
        if (i < n) out[i] = carry + sh[threadIdx.x] - v;
        const int chunk = sh[kThreads - 1];
        __syncthreads();
        carry += chunk;
    }
    if (threadIdx.x == 0) out[n] = carry;
    __syncthreads();
}

// An exclusive prefix sum over the whole grid, called by every thread: each CTA sums a slice, one CTA
// scans the slices' sums, then each CTA scans its slice from its offset; out[n] receives the total.
// For long arrays, where one CTA stepping through them would hold the grid. `part` holds gridDim.x + 1
// ints.
template <class Get>
__device__ void grid_exclusive_scan(Get get, int n, int* out, int* part, int* sh) {
    cgr::grid_group grid = cgr::this_grid();
    const int per = (n + (int)gridDim.x - 1) / (int)gridDim.x;
    const int lo = min(n, (int)blockIdx.x * per), hi = min(n, lo + per);
    int sum = 0;
    for (int i = lo + (int)threadIdx.x; i < hi; i += kThreads) sum += get(i);
    sh[threadIdx.x] = sum;
    __syncthreads();
    for (int o = kThreads / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
    __syncthreads();
    grid.sync();
    if (blockIdx.x == 0) {
        const int* pp = part;
        cta_exclusive_scan([=](int i) { return __ldcg(&pp[i]); }, (int)gridDim.x, part, sh);
    }
    grid.sync();
    int carry = __ldcg(&part[blockIdx.x]);
    for (int base = lo; base < hi; base += kThreads) {
        const int i = base + (int)threadIdx.x;
        const int v = i < hi ? get(i) : 0;
        sh[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < kThreads; o <<= 1) {
            const int t = threadIdx.x >= (unsigned)o ? sh[threadIdx.x - o] : 0;
            __syncthreads();
            sh[threadIdx.x] += t;
            __syncthreads();
        }
        if (i < hi) out[i] = carry + sh[threadIdx.x] - v;
        const int chunk = sh[kThreads - 1];
        __syncthreads();
        carry += chunk;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) out[n] = __ldcg(&part[gridDim.x]);
}

// An index check of the laying schedule: v must lie in [0, hi). A failure records its site, value and
// bound (the first one only), raises error bit 32, and the caller skips the access.
__device__ __noinline__ void check_failed(const WalkDev& w, long long v, long long hi, int site) {
    if (atomicCAS(&w.words[W_CHECK_SITE], 0, site) == 0) {
        w.words[W_CHECK_VALUE] = (int)v;
        w.words[W_CHECK_BOUND] = (int)hi;
    }
    atomicOr(&w.words[W_ERROR], 32);
}
__device__ __forceinline__ bool index_ok(const WalkDev& w, long long v, long long hi, int site) {
    if (v >= 0 && v < hi) return true;
    check_failed(w, v, hi, site);
    return false;
}

// A lake fan's laying by one warp (lay_admitted's loop over the distance-sorted admitted cells). A
// fan's cells are distinct, so laying into one changes no other's need: the warp reads 32 needs at
// once and lays into the ones above zero one after another, in order, while the budget lasts. The
// deposits go to the slot's own log.
__device__ void lay_lake_warp(const WalkDev& w, int s, double budget, int lane) {
    const unsigned FULL = 0xFFFFFFFFu;
    const int n = w.slot_n[s];
    const int* sorted = w.pool_cells + w.slot_off[s];
    const double* base = w.pool_base + w.slot_off[s];
    Touch* log = w.slot_touch + (size_t)s * w.cap;
    double remaining = budget, laid = 0.0;
    int logged = 0;
    for (int i0 = 0; i0 < n && remaining > 0.0; i0 += 32) {
        const int i = i0 + lane;
        int x = -1;
        double need = 0.0;
        if (i < n) {
            x = sorted[i];
            if (index_ok(w, x, (long long)w.p.W * w.p.H, 9)) need = __dsub_rn(base[i], (double)__ldcg(&w.f.sediment[x]));
        }
        unsigned live = __ballot_sync(FULL, i < n && need > 0.0);
        while (live && remaining > 0.0) {
            const int j = __ffs(live) - 1;
            live &= live - 1;
            double moved = 0.0;
            if (lane == j) {
                // HydraulicErosion.raise and the settled height's rise, through L2: an earlier fan on
                // this cell may have laid on another SM in this same wave.
                const float prior = __ldcg(&w.f.sediment[x]), settled = __ldcg(&w.f.settled[x]);
                const float now = (float)((double)prior + (need < remaining ? need : remaining));
                __stcg(&w.f.sediment[x], now);
                moved = (double)now - (double)prior;
                const float increment = (float)(moved * (double)w.p.to_relative);
                __stcg(&w.f.settled[x], settled + increment);
                log[logged] = Touch{x, settled, prior, increment};
            }
            moved = __shfl_sync(FULL, moved, j);
            ++logged;
            remaining -= moved;
            laid += moved;
        }
    }
    if (lane == 0) {
        w.slot_laid[s] = laid;
        w.slot_touch_n[s] = logged;
    }
}

// The kind of a cell's step (own_walk's answer), read from the fixed fields alone.
__device__ __forceinline__ int kind_of(const WalkDev& w, int c) {
    const int r = w.f.dirs[c];
    if (r < 0) return OFF_MAP;
    if (!w.f.land[r]) return SEA;
    if (!ponded(w.p, w.f, c) && ponded(w.p, w.f, r)) return LAKE;
    return ON;
}

// Cell d's settled height as the reference's walk shows it to the cell of rank `rc` of this level:
// its value before the level's fans, plus the increments of the level's fans ranked before rc, in
// order. False when no fan of the level touched d (its current value is then the answer). Reads d's
// group of log entries (in log order), which the last repairs build for the donors of the cells they
// refit.
__device__ bool settled_as_of(const WalkDev& w, int d, int rc, float* out) {
    const int i = w.cell_d[d];
    const int* g = w.rlist + w.roff[i];
    const int m = w.roff[i + 1] - w.roff[i];
    if (m == 0) return false;
    float v = w.touches[g[0]].settled_before;
    for (int a = 0; a < m; ++a)
        if (w.events[w.touch_ev[g[a]]] < rc) v += w.touches[g[a]].increment;
    *out = v;
    return true;
}

// A dry cell of the level whose headroom read a donor that an earlier fan of the level raised, when
// its step hands everything on to a land receiver (kind ON): its own walk is taken again from its
// state before it, with each donor's settled height as the reference's walk shows it at the cell's
// rank. Nothing else of the level reads such a cell (fans touch only ponded land and sea, and cells of
// one level never read one another), so the fix is local. Returns false (a whole redo is needed)
// where the cell has a mouth, whose fan would change with it.
__device__ bool refit_cell(const WalkDev& w, int c) {
    if (kind_of(w, c) != ON) return false;
    const int rc = w.rank_of[c];
    w.f.settled[c] = w.s0[rc];
    w.f.sediment[c] = w.d0[rc];
    const int W = w.p.W, H = w.p.H, col = c % W, row = c / W;
    int patched[8];
    float kept[8];
    int np = 0;
    for (int rs = -1; rs <= 1; ++rs) {
        const int nr = row + rs;
        if (nr < 0 || nr >= H) continue;
        for (int cs = -1; cs <= 1; ++cs) {
            if (rs == 0 && cs == 0) continue;
            const int d = nr * W + ((col + cs) & (W - 1));
            if (w.f.dirs[d] != c) continue;
            float v;
            if (settled_as_of(w, d, rc, &v)) {
                patched[np] = d;
                kept[np++] = w.f.settled[d];
                w.f.settled[d] = v;
            }
        }
    }
    double carried = arriving(w, c);
    bool used;
    double incised = 0.0, deposited = 0.0;
    own_walk(w.p, w.f, c, carried, &used, &incised, &deposited);
    w.handoff[c] = carried;
    for (int i = 0; i < np; ++i) w.f.settled[patched[i]] = kept[i];
    return true;
}

// The walk made the reference's again from rank rc (the earliest mouth conflict), once every fan
// ranked at or after rc is undone (undo_from_grid) and the level's log cut back to before them: the
// conflicted cell's own walk taken again on the state the reference's walk shows it (its own state
// before the walk, and its donors as every fan ranked before it left them, which is now the current
// state); its mouth listed or unlisted as its new load decides. ec is the index of the first event
// ranked at or after rc, the first to lay again; *n is updated.
__device__ void refit_mouth_cell(const WalkDev& w, int rc, int ec, int refit_gen, int* n) {
    const int c = w.order[rc];
    w.f.settled[c] = w.s0[rc];
    w.f.sediment[c] = w.d0[rc];
    double carried = arriving(w, c);
    bool used;
    double incised = 0.0, deposited = 0.0;
    const int kind = own_walk(w.p, w.f, c, carried, &used, &incised, &deposited);
    w.used[c] = used ? 1 : 0;
    if (kind == LAKE) w.handoff[c] = carried;
    w.mark[c] = refit_gen;
    const bool listed = ec < *n && w.events[ec] == rc;
    const bool live = (kind == SEA || kind == LAKE) && mouth_live(w, c, carried, kind);
    if (live) {
        w.ev_carried[rc] = carried;
        w.ev_kind[rc] = (int8_t)kind;
        if (!listed) {
            for (int e = *n; e > ec; --e) w.events[e] = w.events[e - 1];
            w.events[ec] = rc;
            ++*n;
        }
    } else if (listed) {
        for (int e = ec; e + 1 < *n; ++e) w.events[e] = w.events[e + 1];
        --*n;
    }
}

// The level log's entries [cut, T) undone over the grid, called by every thread: a cell takes back
// the state before its earliest entry in the range (what undoing the entries latest first leaves).
// `first` holds kNoTouch outside this call.
__device__ void undo_from_grid(const WalkDev& w, int cut, int T) {
    cgr::grid_group grid = cgr::this_grid();
    const int tid = (int)(blockIdx.x * blockDim.x + threadIdx.x), stride = (int)(gridDim.x * blockDim.x);
    for (int t = cut + tid; t < T; t += stride) atomicMin(&w.first[w.touches[t].cell], t);
    grid.sync();
    for (int t = cut + tid; t < T; t += stride) {
        const Touch tt = w.touches[t];
        if (__ldcg(&w.first[tt.cell]) != t) continue;
        w.f.settled[tt.cell] = tt.settled_before;
        w.f.sediment[tt.cell] = tt.sediment_before;
        w.first[tt.cell] = kNoTouch;
    }
}

// The level-log entry t's event (recorded as the log is assembled).
__device__ __forceinline__ int event_of(const WalkDev& w, int t, int) { return w.touch_ev[t]; }

// The earliest cell of level L, ranked after a fan of the level that raised one of its donors, whose
// headroom read that donor and which has a mouth of its own (its step ends at the sea or in a lake):
// its own walk, and so its fan, are not the reference's. Cells refitted already (mark = the level's
// refit generation) are final and skipped. Over the grid: each thread takes log entries and the
// lowest rank found wins (atomicMin into W_BEST, INT_MAX when there is none).
__device__ void mouth_conflicts_grid(const WalkDev& w, int L, int n) {
    const int T = *(volatile int*)&w.words[W_TOUCHN];
    const int refit_gen = *(volatile int*)&w.words[W_REFITGEN];
    int best = INT_MAX;
    for (int t = (int)(blockIdx.x * blockDim.x + threadIdx.x); t < T; t += (int)(gridDim.x * blockDim.x)) {
        const int x = w.touches[t].cell;
        if (!w.f.land[x]) continue;
        const int rr = w.f.dirs[x];
        if (rr < 0 || !w.f.land[rr] || level_of_cell(w, rr) != L) continue;
        const int r = w.rank_of[rr];
        if (r >= best || !w.used[rr] || w.mark[rr] == refit_gen || kind_of(w, rr) == ON) continue;
        if (r > w.events[event_of(w, t, n)]) best = r;
    }
    if (best != INT_MAX) atomicMin(&w.words[W_BEST], best);
}

// The last repairs of level L, with its final log of n events, called by every thread of the grid:
// (b) a dry cell whose step hands everything on (kind ON) and whose headroom read a donor an earlier
// fan of the level raised is refitted with its donors as the reference's walk showed them; (a) a
// ponded cell of the level ranked after a fan that laid into it has its settled height replayed, its
// own subtraction and the fans' increments in rank order. Steps: (1) the cells to replay and to refit
// listed from the log (each once: atomicExch on its mark); (2) the refits, a thread each (a donor has
// one receiver and cells of a level never read one another, so they share nothing), and the log's
// entries counted per cell to replay; (3) offsets; (4) the entries scattered into per-cell groups;
// (5) each group put back in log order and replayed by one thread: the additions of a walk over the
// whole log, in its order.
__device__ void final_repairs_grid(const WalkDev& w, int L, int n, int touch_n, int* sh_scan) {
    cgr::grid_group grid = cgr::this_grid();
    const int tid = (int)(blockIdx.x * blockDim.x + threadIdx.x), stride = (int)(gridDim.x * blockDim.x);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        w.ev_touch[n] = touch_n;
        w.words[W_TOUCHN] = touch_n;
        w.words[W_FGEN] = ++w.words[W_GEN];
        w.words[W_NREPLAY] = 0;
        w.words[W_NREFIT] = 0;
        w.words[W_NDONOR] = 0;
    }
    grid.sync();
    const int T = *(volatile int*)&w.words[W_TOUCHN];
    const int gen = *(volatile int*)&w.words[W_FGEN];
    for (int t = tid; t < T; t += stride) {
        const int x = w.touches[t].cell;
        if (!w.f.land[x]) continue;
        const int rank = w.events[event_of(w, t, n)];
        if (level_of_cell(w, x) == L && w.rank_of[x] > rank && atomicExch(&w.mark[x], gen) != gen) {
            const int i = atomicAdd(&w.words[W_NREPLAY], 1);
            w.replay[i] = x;
            w.cell_d[x] = i;
        }
        const int rr = w.f.dirs[x];
        if (rr >= 0 && w.f.land[rr] && level_of_cell(w, rr) == L && w.rank_of[rr] > rank && w.used[rr] &&
            kind_of(w, rr) == ON && atomicExch(&w.mark[rr], -gen) != -gen) {   // a dry cell: never a replay's
            const int j = atomicAdd(&w.words[W_NREFIT], 1);
            w.refit[j] = rr;
        }
    }
    grid.sync();
    const int R = *(volatile int*)&w.words[W_NREPLAY], F = *(volatile int*)&w.words[W_NREFIT];
    if (R == 0 && F == 0) return;   // every thread reads the same counts: the grid leaves together
    // The refitted cells' donors join the groups, after the cells to replay (a donor sits on a lower
    // level, so it is never one of those, and it has one receiver, so it joins once).
    const int W = w.p.W, H = w.p.H;
    for (int j = tid; j < F; j += stride) {
        const int c = w.refit[j], col = c % W, row = c / W;
        for (int rs = -1; rs <= 1; ++rs) {
            const int nr = row + rs;
            if (nr < 0 || nr >= H) continue;
            for (int cs = -1; cs <= 1; ++cs) {
                if (rs == 0 && cs == 0) continue;
                const int d = nr * W + ((col + cs) & (W - 1));
                if (w.f.dirs[d] != c || atomicExch(&w.mark[d], gen) == gen) continue;
                const int k = R + atomicAdd(&w.words[W_NDONOR], 1);
                w.replay[k] = d;
                w.cell_d[d] = k;
            }
        }
    }
    grid.sync();
    const int G = R + *(volatile int*)&w.words[W_NDONOR];
    for (int t = tid; t < T; t += stride) {
        const int x = w.touches[t].cell;
        if (w.f.land[x] && __ldcg(&w.mark[x]) == gen) atomicAdd(&w.cell_cnt[x], 1);
    }
    grid.sync();
    if (blockIdx.x == 0) {
        const int* cnt = w.cell_cnt;
        const int* rp = w.replay;
        cta_exclusive_scan([=](int i) { return __ldcg(&cnt[rp[i]]); }, G, w.roff, sh_scan);
    }
    grid.sync();
    for (int t = tid; t < T; t += stride) {
        const int x = w.touches[t].cell;
        if (!w.f.land[x] || __ldcg(&w.mark[x]) != gen) continue;
        const int p = atomicSub(&w.cell_cnt[x], 1) - 1;   // the counts return to 0
        w.rlist[w.roff[w.cell_d[x]] + p] = t;
    }
    grid.sync();
    for (int i = tid; i < G; i += stride) {   // each group back in log order (groups are short)
        int* g = w.rlist + w.roff[i];
        const int m = w.roff[i + 1] - w.roff[i];
        for (int a = 1; a < m; ++a) {
            const int v = g[a];
            int b = a - 1;
            while (b >= 0 && g[b] > v) {
                g[b + 1] = g[b];
                --b;
            }
            g[b + 1] = v;
        }
    }
    grid.sync();
    for (int j = tid; j < F; j += stride) {
        refit_cell(w, w.refit[j]);
        atomicAdd(&w.words[W_REFITTED], 1);
    }
    for (int i = tid; i < R; i += stride) {
        const int x = w.replay[i];
        const int* g = w.rlist + w.roff[i];
        const int m = w.roff[i + 1] - w.roff[i];
        const int rx = w.rank_of[x];
        float acc = w.s0[rx];
        bool own = false;
        for (int a = 0; a < m; ++a) {
            const int t = g[a];
            if (!own && w.events[event_of(w, t, n)] > rx) {
                const double moved = w.f.incised_at[x];
                if (moved > 0.0) acc -= (float)(moved * (double)w.p.to_relative);
                own = true;
            }
            acc += w.touches[t].increment;
        }
        if (!own) {
            const double moved = w.f.incised_at[x];
            if (moved > 0.0) acc -= (float)(moved * (double)w.p.to_relative);
        }
        w.f.settled[x] = acc;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) w.words[W_REPLAYED] += R;
}

// The round's walk, level by level (steps A, B, C above), in one cooperative launch.
__global__ void __launch_bounds__(kThreads) k_deposit_levels(WalkDev w) {
    cgr::grid_group grid = cgr::this_grid();
    __shared__ int warp_counts[kThreads / 32];
    __shared__ int sh_scan[kThreads];
    __shared__ int block_base;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const bool timer = blockIdx.x == 0 && threadIdx.x == 0;
    unsigned long long tm[T_COUNT] = {0, 0, 0, 0, 0};
    unsigned long long t0 = 0;
    for (int L = 0; L < w.levels; ++L) {
        if (timer) t0 = now_ns();
        const int lo = w.level_start[L], hi = w.level_start[L + 1];
        // A: own walks over this CTA's segment of the level, listing live mouths in rank order.
        const int seg = (hi - lo + (int)gridDim.x - 1) / (int)gridDim.x;
        const int s_lo = lo + (int)blockIdx.x * seg;
        const int s_hi = min(hi, s_lo + seg);
        if (threadIdx.x == 0) block_base = 0;
        __syncthreads();
        for (int base = s_lo; base < s_hi; base += kThreads) {
            const int k = base + (int)threadIdx.x;
            bool listed = false;
            if (k < s_hi) {
                const int c = w.order[k];
                w.s0[k] = w.f.settled[c];
                w.d0[k] = w.f.sediment[c];
                double carried = arriving(w, c);
                bool used;
                double incised = 0.0, deposited = 0.0;
                const int kind = own_walk(w.p, w.f, c, carried, &used, &incised, &deposited);
                w.used[c] = used ? 1 : 0;
                if (kind == ON || kind == LAKE) w.handoff[c] = carried;
                if ((kind == SEA || kind == LAKE) && mouth_live(w, c, carried, kind)) {
                    listed = true;
                    w.ev_carried[k] = carried;
                    w.ev_kind[k] = (int8_t)kind;
                }
            }
            const unsigned ballot = __ballot_sync(0xFFFFFFFFu, listed);
            if (lane == 0) warp_counts[warp] = __popc(ballot);
            __syncthreads();
            int before = block_base;
            for (int i = 0; i < warp; ++i) before += warp_counts[i];
            if (listed) w.seg_events[s_lo + before + __popc(ballot & ((1u << lane) - 1u))] = k;
            __syncthreads();
            if (threadIdx.x == 0) {
                int total = 0;
                for (int i = 0; i < kThreads / 32; ++i) total += warp_counts[i];
                block_base += total;
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) w.seg_count[blockIdx.x] = block_base;
        grid.sync();
        // The listed mouths, dense and in rank order: each CTA's segment at the offset of the ones before.
        if (blockIdx.x == 0) {
            const int* sc = w.seg_count;
            cta_exclusive_scan([=](int i) { return sc[i]; }, (int)gridDim.x, w.seg_off, sh_scan);
            if (threadIdx.x == 0) w.words[W_EVENTS] = w.seg_off[gridDim.x];
        }
        grid.sync();
        for (int i = threadIdx.x; i < block_base; i += blockDim.x) w.events[w.seg_off[blockIdx.x] + i] = w.seg_events[s_lo + i];
        grid.sync();
        if (timer) tm[T_WALKS] += now_ns() - t0;
        const int n = *(volatile int*)&w.words[W_EVENTS];
        const int lane = threadIdx.x & 31;
        const int gwarp = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
        const int nwarps = (int)((gridDim.x * blockDim.x) >> 5);
        int touch_n = 0;   // the level's log length (kept by the one thread that writes the log)
        int n_now = n, e_start = 0;
        int refit_gen = 0;   // thread 0's mark for the level's refitted mouth cells (a fresh generation)
        // B, and C's mouth conflicts: lay the events from e_start in rank order (chunks of `slots`); then
        // if a cell with a mouth read a donor an earlier fan raised, make the walk the reference's again
        // from that cell (refit_mouth_cell) and lay what follows it again. Each pass moves past at least
        // one such cell, so there are at most as many passes as the level has cells, and one more.
        const int passes = hi - lo + 1;
        for (int pass = 0; pass <= passes; ++pass) {
            for (int e0 = e_start; e0 < n_now; e0 += w.slots) {
                if (timer) t0 = now_ns();
                const int e1 = min(n_now, e0 + w.slots);
                // The chunk's lake fans, their admissions taken from the round's pool.
                for (int e = e0 + (int)(blockIdx.x * blockDim.x + threadIdx.x); e < e1;
                     e += (int)(gridDim.x * blockDim.x)) {
                    const int k = w.events[e];
                    const bool lake = w.ev_kind[k] == LAKE;
                    bool ok = lake;
                    if (lake) {
                        const int ci = w.cand_of[w.order[k]];
                        ok = index_ok(w, ci, w.ncand, 1);
                        if (ok) ok = index_ok(w, w.cand_n[ci], (long long)w.cap + 1, 3);
                        if (ok) ok = index_ok(w, w.cand_off[ci] + w.cand_n[ci], w.pool_total + 1, 2);
                        if (ok) {
                            w.slot_off[e - e0] = w.cand_off[ci];
                            w.slot_n[e - e0] = w.cand_n[ci];
                        }
                    }
                    int state = ok ? 1 : 0;
                    if (w.ev_kind[k] == SEA) {   // the tiles of the box its lobe can read or write
                        const int apex = w.f.dirs[w.order[k]];
                        const int acol = apex % w.p.W, arow = apex / w.p.W;
                        const int c0 = acol - w.box_x, c1 = acol + w.box_x;
                        const int r0 = max(0, arow - w.box_y), r1 = min(w.p.H - 1, arow + w.box_y);
                        const int tx0 = c0 >= 0 ? c0 / kTile : -((-c0 + kTile - 1) / kTile);
                        const int tx1 = c1 >= 0 ? c1 / kTile : -((-c1 + kTile - 1) / kTile);
                        const int ntx = min(tx1 - tx0 + 1, w.tiles_x), nty = r1 / kTile - r0 / kTile + 1;
                        int* box = w.slot_box + 4 * (e - e0);
                        box[0] = tx0;
                        box[1] = r0 / kTile;
                        box[2] = ntx;
                        box[3] = nty;
                        w.slot_n[e - e0] = ntx * nty;
                        state = 2;
                    }
                    w.slot_state[e - e0] = state;
                    w.slot_touch_n[e - e0] = 0;
                    w.blockers[e - e0] = 0;
                }
                grid.sync();
                // The lake fans lay in waves, a warp each, in rank order wherever they share a cell: the
                // chunk's (fan, cell) pairs are grouped by cell, each pair learning whether an earlier
                // fan is on its cell (the fan's blocker count) and which fan follows it there. A fan lays
                // once its count is 0 and then releases its followers; disjoint fans lay at once (their
                // layings touch different cells). Bounded: the lowest waiting rank is never blocked, so
                // every wave lays at least one fan.
                const int S = e1 - e0;
                if (blockIdx.x == 0) {
                    const int* st = w.slot_state;
                    const int* sn = w.slot_n;
                    cta_exclusive_scan([=](int i) { return st[i] ? sn[i] : 0; }, S, w.poff, sh_scan);
                    int lakes = 0, seas = 0;
                    for (int base = 0; base < S; base += kThreads) {
                        const int i = base + (int)threadIdx.x;
                        lakes += __syncthreads_count(i < S && st[i] == 1);
                        seas += __syncthreads_count(i < S && st[i] == 2);
                    }
                    if (threadIdx.x == 0) {
                        w.words[W_PAIRS] = w.poff[S];
                        w.words[W_DISTINCT] = 0;
                        w.words[W_NLAKE] = lakes;
                        w.words[W_NSEA] = seas;
                        if (w.poff[S] > w.pair_cap) w.words[W_ERROR] |= 16;
                    }
                }
                grid.sync();
                const int P = min(*(volatile int*)&w.words[W_PAIRS], w.pair_cap);
                for (int q = (int)(blockIdx.x * blockDim.x + threadIdx.x); q < P; q += (int)(gridDim.x * blockDim.x)) {
                    int a = 0, b = S;   // the slot whose pairs hold q: poff[a] <= q < poff[a + 1]
                    while (b - a > 1) {
                        const int m = (a + b) >> 1;
                        if (w.poff[m] <= q) a = m;
                        else b = m;
                    }
                    int x = 0;
                    const int k = q - w.poff[a];
                    if (index_ok(w, k, w.slot_n[a], 12)) {
                        if (w.slot_state[a] == 2) {   // a sea lobe's tile
                            const int* box = w.slot_box + 4 * a;
                            const int ntx = box[2];
                            int tx = (box[0] + k % ntx) % w.tiles_x;
                            if (tx < 0) tx += w.tiles_x;
                            x = w.p.W * w.p.H + (box[1] + k / ntx) * w.tiles_x + tx;
                        } else {
                            x = w.pool_cells[w.slot_off[a] + k];
                        }
                    }
                    if (!index_ok(w, x, (long long)w.p.W * w.p.H + (long long)w.tiles_x * w.tiles_y, 4)) x = 0;
                    w.pair_fan[q] = a;
                    w.pair_cell[q] = x;
                    const int pos = atomicAdd(&w.cell_cnt[x], 1);
                    w.pair_pos[q] = pos;
                    if (pos == 0) {
                        const int d = atomicAdd(&w.words[W_DISTINCT], 1);
                        w.dcell[d] = x;
                        w.cell_d[x] = d;
                    }
                }
                grid.sync();
                const int D = *(volatile int*)&w.words[W_DISTINCT];
                {
                    const int* cnt = w.cell_cnt;
                    const int* dc = w.dcell;
                    if (D > 4 * kThreads) {   // long: over the grid
                        grid_exclusive_scan([=](int i) { return __ldcg(&cnt[dc[i]]); }, D, w.doff, w.seg_part, sh_scan);
                    } else if (blockIdx.x == 0) {
                        cta_exclusive_scan([=](int i) { return __ldcg(&cnt[dc[i]]); }, D, w.doff, sh_scan);
                    }
                }
                grid.sync();
                // Every pair is counted on exactly one distinct cell.
                if (blockIdx.x == 0 && threadIdx.x == 0 && __ldcg(&w.doff[D]) != P) check_failed(w, w.doff[D], P, 13);
                for (int q = (int)(blockIdx.x * blockDim.x + threadIdx.x); q < P; q += (int)(gridDim.x * blockDim.x)) {
                    const int d = w.cell_d[w.pair_cell[q]];
                    if (!index_ok(w, d, D, 5)) continue;
                    const int at = w.doff[d] + w.pair_pos[q];
                    if (index_ok(w, at, P, 6)) w.group[at] = q;
                }
                grid.sync();
                for (int q = (int)(blockIdx.x * blockDim.x + threadIdx.x); q < P; q += (int)(gridDim.x * blockDim.x)) {
                    const int x = w.pair_cell[q];
                    const int d = w.cell_d[x];
                    if (!index_ok(w, d, D, 5)) continue;
                    const int* g = w.group + w.doff[d];
                    const int m = __ldcg(&w.cell_cnt[x]);
                    if (!index_ok(w, w.doff[d] + m, (long long)P + 1, 7)) continue;
                    const int r = w.events[e0 + w.pair_fan[q]];
                    bool pred = false;
                    int succ = -1, rs = 0;
                    for (int j = 0; j < m; ++j) {
                        if (!index_ok(w, g[j], P, 8)) continue;
                        const int f = w.pair_fan[g[j]];
                        const int rf = w.events[e0 + f];
                        if (rf < r) pred = true;
                        else if (rf > r && (succ < 0 || rf < rs)) {
                            succ = f;
                            rs = rf;
                        }
                    }
                    w.pair_succ[q] = succ;
                    if (pred) atomicAdd(&w.blockers[w.pair_fan[q]], 1);
                }
                grid.sync();
                for (int q = (int)(blockIdx.x * blockDim.x + threadIdx.x); q < P; q += (int)(gridDim.x * blockDim.x))
                    w.cell_cnt[w.pair_cell[q]] = 0;   // every cell's count back to 0 for the next chunk
                int waves = 0;
                if (timer) {
                    const unsigned long long t = now_ns();
                    tm[T_SCHEDULE] += t - t0;
                    t0 = t;
                }
                const int n_lakes = *(volatile int*)&w.words[W_NLAKE], n_seas = *(volatile int*)&w.words[W_NSEA];
                // A fan's warp waits for its count to reach 0 (the fans before it on its cells laid), inside
                // the cooperative launch: every CTA is resident, each warp takes its slots in rank order and
                // a count only waits on lower ranks, so the lowest waiting fan always runs. The wait is
                // bounded; a warp that gives up raises the abort word, which every other waiter also
                // heeds, and the walk reports the error.
                // A lake fan touches only ponded land and a sea lobe only sea cells, so the two kinds wait
                // only on their own (their schedule ids are cells and tiles, apart) and lay in one pass. A
                // sea lobe runs whole on its warp's lane 0, reading and writing the fields through L2.
                if (n_lakes + n_seas > 0) {
                    for (int sl = gwarp; sl < S; sl += nwarps) {
                        const int kind_slot = w.slot_state[sl];
                        if (kind_slot != 1 && kind_slot != 2) continue;
                        int go = 1;
                        if (lane == 0) {
                            long long spins = 0;
                            while (*(volatile int*)&w.blockers[sl] != 0) {
                                if (*(volatile int*)&w.words[W_ABORT] || ++spins > kSpinLimit) {
                                    atomicOr(&w.words[W_ERROR], 4);
                                    atomicExch(&w.words[W_ABORT], 1);
                                    go = 0;
                                    break;
                                }
                                __nanosleep(64);
                            }
                        }
                        if (!__shfl_sync(0xFFFFFFFFu, go, 0)) continue;
                        __threadfence();
                        const int rank = w.events[e0 + sl];
                        const int c = w.order[rank];
                        const double carried = w.ev_carried[rank];
                        if (kind_slot == 1) {
                            lay_lake_warp(w, sl, mouth_budget(w.p, w.f, c, carried, LAKE), lane);
                        } else {
                            uint32_t* bits = w.warp_bits + (size_t)gwarp * w.box_words;
                            for (int j = lane; j < w.box_words; j += 32) bits[j] = 0u;
                            __syncwarp();
                            if (lane == 0) {
                                Heap h = warp_heap(w, gwarp);
                                TouchLog log{w.slot_touch + (size_t)sl * w.cap, w.cap, 0, 0};
                                int outside = 0;
                                const int bx = w.box_x, by = w.box_y, W = w.p.W;
                                mouth_with(w.p, w.f, c, carried, SEA,
                                           [=, &outside](const Rim& m) {
                                               return BoxVisited{bits, W, m.apex_column, m.apex_row, bx, by, &outside};
                                           },
                                           h, &log);
                                if (log.overflow) atomicOr(&w.words[W_ERROR], 1);
                                if (outside) atomicOr(&w.words[W_ERROR], 2);   // past the box its tiles cover
                                w.slot_touch_n[sl] = log.count;
                            }
                        }
                        __syncwarp();
                        __threadfence();
                        for (int q = w.poff[sl] + lane; q < min(w.poff[sl + 1], P); q += 32)   // P: past an overflow
                            if (w.pair_succ[q] >= 0 && index_ok(w, w.pair_succ[q], S, 11)) atomicSub(&w.blockers[w.pair_succ[q]], 1);
                        if (lane == 0) {
                            if (kind_slot == 1) w.handoff[c] = __dsub_rn(carried, w.slot_laid[sl]);
                            w.slot_state[sl] = 0;
                        }
                    }
                    grid.sync();
                    ++waves;
                }
                if (timer) {
                    const unsigned long long t = now_ns();
                    tm[T_LAKES] += t - t0;
                    t0 = t;
                }
                // The chunk's deposits into the level's log in rank order: each event's entries at the
                // offset of the events before it.
                if (blockIdx.x == 0) {
                    const int* tn = w.slot_touch_n;
                    cta_exclusive_scan([=](int i) { return tn[i]; }, S, w.poff, sh_scan);
                    if (threadIdx.x == 0) {
                        w.words[W_WAVES] += waves;
                        w.words[W_TOUCHN] = touch_n;
                    }
                }
                grid.sync();
                {
                    const int base = *(volatile int*)&w.words[W_TOUCHN];
                    const int total = w.poff[S];
                    const int room = w.touch_cap - base;
                    const int copied = total < room ? total : room;
                    if (total > room && blockIdx.x == 0 && threadIdx.x == 0) w.words[W_ERROR] |= 1;
                    const int tid = (int)(blockIdx.x * blockDim.x + threadIdx.x), stride = (int)(gridDim.x * blockDim.x);
                    for (int e = tid; e < S; e += stride) w.ev_touch[e0 + e] = base + min(w.poff[e], copied);
                    for (int q = tid; q < copied; q += stride) {
                        int a = 0, b = S;
                        while (b - a > 1) {
                            const int m = (a + b) >> 1;
                            if (w.poff[m] <= q) a = m;
                            else b = m;
                        }
                        w.touches[base + q] = w.slot_touch[(size_t)a * w.cap + (q - w.poff[a])];
                        w.touch_ev[base + q] = e0 + a;
                    }
                    if (blockIdx.x == 0 && threadIdx.x == 0) touch_n = base + copied;
                }
                if (timer) tm[T_SEAS] += now_ns() - t0;
                grid.sync();
            }
            if (timer) t0 = now_ns();
            if (blockIdx.x == 0 && threadIdx.x == 0) {
                w.ev_touch[n_now] = touch_n;
                if (pass == 0) refit_gen = ++w.words[W_GEN];
                w.words[W_REFITGEN] = refit_gen;
                w.words[W_BEST] = INT_MAX;
                w.words[W_TOUCHN] = touch_n;
            }
            grid.sync();
            mouth_conflicts_grid(w, L, n_now);
            grid.sync();
            if (blockIdx.x == 0 && threadIdx.x == 0) {
                const int best = *(volatile int*)&w.words[W_BEST];
                const int rc = best == INT_MAX ? -1 : best;
                if (rc < 0) {
                    w.words[W_DONE] = 1;
                } else {
                    if (pass == passes) w.words[W_ERROR] |= 8;
                    int a = 0, b = n_now;   // the first event ranked at or after rc (events are in rank order)
                    while (a < b) {
                        const int m = (a + b) >> 1;
                        if (w.events[m] < rc) a = m + 1;
                        else b = m;
                    }
                    w.words[W_ESTART] = a;
                    w.words[W_CUT] = a < n_now ? w.ev_touch[a] : touch_n;
                    w.words[W_RC] = rc;
                    w.words[W_DONE] = 0;
                }
            }
            grid.sync();
            if (!*(volatile int*)&w.words[W_DONE]) {
                // Every fan ranked at or after rc undone, the log cut back to before them, the cell refitted.
                const int cut = *(volatile int*)&w.words[W_CUT];
                undo_from_grid(w, cut, *(volatile int*)&w.words[W_TOUCHN]);
                grid.sync();
                if (blockIdx.x == 0 && threadIdx.x == 0) {
                    touch_n = cut;
                    int nn = n_now;
                    refit_mouth_cell(w, w.words[W_RC], w.words[W_ESTART], refit_gen, &nn);
                    w.words[W_EVENTS] = nn;
                    w.words[W_RELAID]++;
                }
            }
            grid.sync();
            if (timer) tm[T_REPAIRS] += now_ns() - t0;
            if (*(volatile int*)&w.words[W_DONE]) break;
            e_start = *(volatile int*)&w.words[W_ESTART];
            n_now = *(volatile int*)&w.words[W_EVENTS];
            grid.sync();
        }
        // C: the last repairs, with every deposit of the level in its log.
        if (timer) t0 = now_ns();
        if (n_now > 0) final_repairs_grid(w, L, n_now, touch_n, sh_scan);
        grid.sync();
        if (timer) tm[T_REPAIRS] += now_ns() - t0;
    }
    if (timer)
        for (int i = 0; i < T_COUNT; ++i) w.timers[i] = tm[i];
}

// settled = relative + sediment * toRelative, with no load and nothing incised yet
// (HydraulicErosion.kt:940-945).
__global__ void k_round_begin(const float* __restrict__ rel, const float* __restrict__ sediment, size_t N,
                              float to_relative, float* __restrict__ settled, double* __restrict__ load,
                              double* __restrict__ incised_at) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x) {
        settled[i] = __fadd_rn(rel[i], __fmul_rn(sediment[i], to_relative));
        load[i] = 0.0;
        incised_at[i] = 0.0;
    }
}

__global__ void k_rank_of(const int* __restrict__ order, int n, int* __restrict__ rank_of) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) rank_of[order[k]] = k;
}

// Each level's first rank in the drainage order (level-major): level_start[levels] = n.
__global__ void k_level_bounds(const int* __restrict__ order, const long long* __restrict__ key, int n, int levels,
                               int* __restrict__ level_start) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const int L = (int)(key[order[k]] >> 32);
        const int prev = k > 0 ? (int)(key[order[k - 1]] >> 32) : -1;
        for (int l = prev + 1; l <= L; ++l) level_start[l] = k;
        if (k == n - 1)
            for (int l = L + 1; l <= levels; ++l) level_start[l] = n;
    }
}

// settle(): the stage's deposition laid on the rock at once; the sediment stays as the spoil the
// mouths pass reads (HydraulicErosion.kt:1351-1364, 1451-1462).
__global__ void k_settle(float* __restrict__ h, const float* __restrict__ sediment, size_t N) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x)
        h[i] = __fadd_rn(h[i], sediment[i]);
}

struct MouthsDev {
    int W;
    float pond_depth, drawn_river_cells, shoreline, fall_per_cell_width, floor_, step_ns, step_diag;
    const uint8_t* land;
    const float* filled;
    const float* rel;
    const float* area;
    const int32_t* recv;
    const float* spoil;
    float* working;
    const int* start;
    const int* bucket;
    int levels;
};

// Math.min(float, float) on the JVM: NaN if either is, and -0 below +0.
__device__ __forceinline__ float jvm_minf(float a, float b) {
    if (a != a) return a;
    if (b != b) return b;
    if (a == 0.0f && b == 0.0f) return __float_as_int(a) < 0 ? a : b;
    return a < b ? a : b;
}

// One cell of openMouths' pass (HydraulicErosion.kt:1855-1890).
__device__ void mouth_cell(const MouthsDev& d, int cell) {
    if (d.area[cell] < d.drawn_river_cells) return;
    const float standing = __fsub_rn(d.filled[cell], d.rel[cell]);
    const bool on_flat = standing > 0.0f && (standing <= d.pond_depth || d.spoil[cell] > 0.0f);
    if (!on_flat) return;
    const int receiver = d.recv[cell];
    if (receiver < 0) return;
    const float below = d.land[receiver] ? d.working[receiver] : d.shoreline;
    const bool same_row = cell / d.W == receiver / d.W, same_col = cell % d.W == receiver % d.W;
    const float step = (!same_row && !same_col) ? d.step_diag : (!same_row ? d.step_ns : 1.0f);
    float fall = __fmul_rn(d.fall_per_cell_width, step);
    if (fall < 1e-7f) fall = 1e-7f;   // MIN_DISTRIBUTARY_FALL
    const float now = d.working[cell];
    float want = jvm_minf(now, __fadd_rn(below, fall));
    if (want < d.floor_) want = d.floor_;
    if (now > want) d.working[cell] = (float)__dadd_rn((double)now, (double)__fsub_rn(want, now));
}

// Receivers first: levels from the top down, a grid barrier between levels.
__global__ void __launch_bounds__(256) k_mouths_levels(MouthsDev d) {
    cgr::grid_group grid = cgr::this_grid();
    const int stride = gridDim.x * blockDim.x;
    for (int level = d.levels - 1; level >= 0; --level) {
        const int lo = d.start[level], hi = d.start[level + 1];
        for (int i = lo + blockIdx.x * blockDim.x + threadIdx.x; i < hi; i += stride) mouth_cell(d, d.bucket[i]);
        grid.sync();
    }
}

__global__ void k_zero_float(float* __restrict__ a, size_t N) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x) a[i] = 0.0f;
}

}  // namespace

// The laying schedule's ids: the cells, then the sea lobes' box tiles.
size_t schedule_ids(int W, int H) {
    return (size_t)W * H + (size_t)((W + kTile - 1) / kTile) * ((H + kTile - 1) / kTile);
}

cg_status deposit_stage_reset_dev(cg_ctx* ctx, int W, int H) {
    const size_t N = (size_t)W * H;
    const size_t ids = schedule_ids(W, H);
    CG_BUF(float, d_sediment, ctx, S_SEDIMENT, N);
    CG_BUF(int, d_stamp, ctx, S_STAMP, N);
    CG_BUF(int, d_mark, ctx, S_DEPMARK, N);
    CG_BUF(int, d_cellcnt, ctx, S_DEPCELLCNT, 2 * ids);
    CG_BUF(int, d_first, ctx, S_DEPFIRST, N);
    CG_BUF(int, d_words, ctx, S_DEPWORDS, W_WORDS);
    CG_LAUNCH(ctx) k_zero_float<<<ctx->num_sms * 8, 256, 0, ctx->stream>>>(d_sediment, N);
    CG_CHECK_LAUNCH(ctx);
    // Fan ids and replay generations restart at 0, so every stamp and mark must too; the laying
    // schedule's per-cell counts start at 0 (each chunk leaves them at 0).
    CG_CUDA(ctx, cudaMemsetAsync(d_stamp, 0, N * sizeof(int), ctx->stream));
    CG_CUDA(ctx, cudaMemsetAsync(d_mark, 0, N * sizeof(int), ctx->stream));
    CG_CUDA(ctx, cudaMemsetAsync(d_cellcnt, 0, ids * sizeof(int), ctx->stream));
    CG_CUDA(ctx, cudaMemsetAsync(d_first, 0x7F, N * sizeof(int), ctx->stream));   // kNoTouch
    CG_CUDA(ctx, cudaMemsetAsync(d_words, 0, W_WORDS * sizeof(int), ctx->stream));
    return CG_OK;
}

cg_status deposit_round_begin_dev(cg_ctx* ctx, int W, int H, const float* d_rel, float to_relative, float** d_settled,
                                  double** d_load, double** d_incised_at) {
    const size_t N = (size_t)W * H;
    CG_BUF(float, sediment, ctx, S_SEDIMENT, N);
    CG_BUF(float, settled, ctx, S_SETTLED, N);
    CG_BUF(double, load, ctx, S_LOAD, N);
    CG_BUF(double, incised_at, ctx, S_INCISED, N);
    CG_LAUNCH(ctx) k_round_begin<<<ctx->num_sms * 8, 256, 0, ctx->stream>>>(d_rel, sediment, N, to_relative, settled,
                                                                          load, incised_at);
    CG_CHECK_LAUNCH(ctx);
    *d_settled = settled;
    *d_load = load;
    *d_incised_at = incised_at;
    return CG_OK;
}

cg_status deposit_walk_dev(cg_ctx* ctx, const cg_erosion_params& cp, const DepositRound& r, DepositCounts* counts) {
    const int W = cp.width, H = cp.height;
    const size_t N = (size_t)W * H;
    cudaStream_t sm = ctx->stream;
    if (r.land_cells <= 0 || r.levels <= 0) return CG_OK;
    const int n = r.land_cells;
    WalkDev w;
    w.p = make_params(cp, (float)r.land_cells, r.land_range, r.to_relative, r.shoreline);
    CG_BUF(float, d_sediment, ctx, S_SEDIMENT, N);
    w.f = Fields{r.recv, r.land, r.ground, r.rel, r.area, r.surface, d_sediment, r.settled, r.incised_at};
    // The drainage order and each level's first rank.
    CG_BUF(int32_t, d_order, ctx, S_ORDER, N);
    CG_TRY_ST(order_from_keys_dev(ctx, W, H, r.land, r.key, n, d_order));
    CG_BUF(int, d_rank, ctx, S_DEPRANK, N);
    CG_BUF(int, d_lstart, ctx, S_DEPLEVEL, (size_t)r.levels + 1);
    const int grid = ctx->num_sms * 8;
    CG_LAUNCH(ctx) k_rank_of<<<grid, 256, 0, sm>>>(d_order, n, d_rank);
    CG_LAUNCH(ctx) k_level_bounds<<<grid, 256, 0, sm>>>(d_order, r.key, n, r.levels, d_lstart);
    CG_CHECK_LAUNCH(ctx);
    w.order = d_order;
    w.rank_of = d_rank;
    w.key = r.key;
    w.level_start = d_lstart;
    w.levels = r.levels;
    w.load = r.load;
    CG_BUF(double, d_handoff, ctx, S_HANDOFF, N);
    CG_BUF(uint8_t, d_used, ctx, S_DEPUSED, N);
    CG_BUF(float, d_s0, ctx, S_DEPS0, (size_t)n);
    CG_BUF(float, d_d0, ctx, S_DEPD0, (size_t)n);
    CG_BUF(double, d_evc, ctx, S_DEPEVC, (size_t)n);
    CG_BUF(int8_t, d_evk, ctx, S_DEPEVK, (size_t)n);
    CG_BUF(int, d_seg, ctx, S_DEPSEG, (size_t)n);
    CG_BUF(int, d_events, ctx, S_DEPEVENTS, (size_t)n + 1);
    CG_BUF(int, d_evtouch, ctx, S_DEPEVTOUCH, (size_t)n + 1);
    w.handoff = d_handoff;
    w.used = d_used;
    w.s0 = d_s0;
    w.d0 = d_d0;
    w.ev_carried = d_evc;
    w.ev_kind = d_evk;
    w.seg_events = d_seg;
    w.events = d_events;
    w.ev_touch = d_evtouch;
    // The heap's capacity (DeltaFan.Scratch), the round's lake fans admitted ahead of the walk, and the
    // chunks' mouth slots.
    w.cap = heap_capacity(w.p);
    w.box_words = box_words(w.p);
    w.slots = 2048;
    const size_t S = (size_t)w.slots, cap = (size_t)w.cap;
    CG_BUF(int, d_candof, ctx, S_DEPCANDOF, N);
    CG_BUF(int, d_cand, ctx, S_DEPCAND, (size_t)n + 2);
    int* d_ncand = d_cand + n;
    CG_BUF(int, d_words, ctx, S_DEPWORDS, W_WORDS);
    CG_CUDA(ctx, cudaMemsetAsync(d_ncand, 0, sizeof(int), sm));
    CG_LAUNCH(ctx) k_lake_candidates<<<grid, 256, 0, sm>>>(w.p, w.f, (int)N, d_cand, d_ncand, d_candof);
    CG_CHECK_LAUNCH(ctx);
    int ncand = 0;
    CG_CUDA(ctx, cudaMemcpyAsync(&ncand, d_ncand, sizeof(int), cudaMemcpyDeviceToHost, sm));
    CG_CUDA(ctx, cudaStreamSynchronize(sm));
    CG_BUF(int, d_candn, ctx, S_DEPCANDN, (size_t)ncand + 1);
    CG_BUF(long long, d_candoff, ctx, S_DEPCANDOFF, (size_t)ncand + 1);
    long long pool_total = 0;
    int* d_pool_cells = nullptr;
    double* d_pool_base = nullptr;
    if (ncand > 0) {
        AdmitDev a;
        a.p = w.p;
        a.f = w.f;
        a.cap = w.cap;
        a.box_words = w.box_words;
        a.cand = d_cand;
        a.ncand = ncand;
        a.cand_n = d_candn;
        a.cand_off = d_candoff;
        a.err = d_words + W_ERROR;
        const int threads = ctx->num_sms * 128;
        const size_t T = (size_t)threads;
        CG_BUF(int, d_hc, ctx, S_DEPSLOT0, T * cap);
        CG_BUF(float, d_hk, ctx, S_DEPSLOT1, T * cap);
        CG_BUF(float, d_hp, ctx, S_DEPSLOT2, T * cap);
        CG_BUF(int, d_ha, ctx, S_DEPSLOT3, T * cap);
        CG_BUF(uint32_t, d_hb, ctx, S_DEPSLOT6, T * (size_t)w.box_words);
        a.h_cells = d_hc;
        a.h_keys = d_hk;
        a.h_pens = d_hp;
        a.h_admitted = d_ha;
        a.h_bits = d_hb;
        a.pool_cells = nullptr;
        a.pool_base = nullptr;
        a.fill = 0;
        CG_LAUNCH(ctx) k_admit_lakes<<<ctx->num_sms, 128, 0, sm>>>(a);
        CG_CHECK_LAUNCH(ctx);
        // Offsets: an exclusive scan of the counts in 64 bits.
        CG_BUF(long long, d_wide, ctx, S_DEPCANDW, (size_t)ncand + 1);
        CG_LAUNCH(ctx) k_widen_counts<<<(ncand + 255) / 256, 256, 0, sm>>>(d_candn, ncand, d_wide);
        CG_CHECK_LAUNCH(ctx);
        CG_LAUNCH(ctx) k_scan64_one_block<<<1, 1024, 0, sm>>>(d_wide, d_candoff, ncand);
        CG_CHECK_LAUNCH(ctx);
        CG_CUDA(ctx, cudaMemcpyAsync(&pool_total, d_candoff + ncand, sizeof(long long), cudaMemcpyDeviceToHost, sm));
        CG_CUDA(ctx, cudaStreamSynchronize(sm));
        CG_BUF(int, d_pc, ctx, S_DEPSLOT4, (size_t)pool_total + 1);
        CG_BUF(double, d_pb, ctx, S_DEPSLOT5, (size_t)pool_total + 1);
        d_pool_cells = d_pc;
        d_pool_base = d_pb;
        a.pool_cells = d_pc;
        a.pool_base = d_pb;
        a.fill = 1;
        CG_LAUNCH(ctx) k_admit_lakes<<<ctx->num_sms, 128, 0, sm>>>(a);
        CG_CHECK_LAUNCH(ctx);
    }
    w.cand_of = d_candof;
    w.cand_n = d_candn;
    w.cand_off = d_candoff;
    w.ncand = ncand;
    w.pool_total = pool_total;
    w.pool_cells = d_pool_cells;
    w.pool_base = d_pool_base;
    CG_BUF(long long, d_soff, ctx, S_DEPSLOTOFF, S);
    CG_BUF(int, d_sn, ctx, S_DEPSLOT7, 6 * S);
    CG_BUF(double, d_slaid, ctx, S_DEPSLOT8, S);
    CG_BUF(Touch, d_stouch, ctx, S_DEPSLOT9, S * cap);
    CG_BUF(int, d_stn, ctx, S_DEPSLOT10, S);
    w.pair_cap = (int)std::min<size_t>(S * cap, (size_t)1 << 30);
    const size_t PC = (size_t)w.pair_cap;
    // poff (S + 1), blockers (S + 1), then seven arrays of PC: pair_fan, pair_cell, pair_pos,
    // pair_succ, group, dcell, and doff (its D + 1 <= PC + 1 entries run into the spare 2).
    CG_BUF(int, d_sched, ctx, S_DEPCLAIM, 7 * PC + 2 * S + 4);
    const size_t ids = schedule_ids(W, H);
    CG_BUF(int, d_cellcnt, ctx, S_DEPCELLCNT, 2 * ids);
    w.tiles_x = (W + kTile - 1) / kTile;
    w.tiles_y = (H + kTile - 1) / kTile;
    w.box_x = box_bx(w.p);
    w.box_y = box_by(w.p);
    w.poff = d_sched;
    w.blockers = d_sched + S + 1;
    w.pair_fan = w.blockers + S + 1;
    w.pair_cell = w.pair_fan + PC;
    w.pair_pos = w.pair_cell + PC;
    w.pair_succ = w.pair_pos + PC;
    w.group = w.pair_succ + PC;
    w.dcell = w.group + PC;
    w.doff = w.dcell + PC;
    w.cell_cnt = d_cellcnt;
    w.cell_d = d_cellcnt + ids;
    w.slot_off = d_soff;
    w.slot_n = d_sn;
    w.slot_state = d_sn + S;
    w.slot_box = d_sn + 2 * S;
    w.slot_laid = d_slaid;
    w.slot_touch = d_stouch;
    w.slot_touch_n = d_stn;
    CG_BUF(int, d_stamp, ctx, S_STAMP, N);
    w.stamp = d_stamp;
    w.touch_cap = (int)std::min<size_t>(N, (size_t)1 << 26);
    CG_BUF(Touch, d_touch, ctx, S_DEPTOUCH, (size_t)w.touch_cap);
    w.touches = d_touch;
    CG_BUF(int, d_mark, ctx, S_DEPMARK, N);
    CG_BUF(int, d_replay, ctx, S_DEPREPLAY, 2 * N);
    w.mark = d_mark;
    w.replay = d_replay;
    w.refit = d_replay + N;
    CG_BUF(int, d_rlist, ctx, S_DEPRLIST, (size_t)w.touch_cap + (size_t)N + 1);
    w.rlist = d_rlist;
    CG_BUF(int, d_first, ctx, S_DEPFIRST, N);
    w.first = d_first;
    CG_BUF(int, d_tev, ctx, S_DEPTOUCHEV, (size_t)w.touch_cap);
    w.touch_ev = d_tev;
    w.roff = d_rlist + w.touch_cap;
    CG_BUF(float, d_acc, ctx, S_DEPACC, N);
    CG_BUF(uint8_t, d_own, ctx, S_DEPOWN, N);
    w.acc = d_acc;
    w.own_done = d_own;
    w.words = d_words;
    CG_BUF(unsigned long long, d_timers, ctx, S_DEPTIMERS, T_COUNT);
    w.timers = d_timers;
    // The round's own counts (the fan ids, generations and wave numbers carry on through the stage).
    for (int word : {W_REPLAYED, W_WAVES, W_REFITTED, W_RELAID, W_ABORT})
        CG_CUDA(ctx, cudaMemsetAsync(d_words + word, 0, sizeof(int), sm));
    int per_sm = 0;
    CG_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_deposit_levels, kThreads, 0));
    if (per_sm < 1) return fail(ctx, CG_CUDA, "deposition kernel cannot be resident");
    const int cgrid = ctx->num_sms * (per_sm < 2 ? per_sm : 2);
    CG_BUF(int, d_segc, ctx, S_DEPSEGC, 3 * (size_t)cgrid + 2);
    w.seg_count = d_segc;
    w.seg_off = d_segc + cgrid;
    w.seg_part = d_segc + 2 * (size_t)cgrid + 1;
    // A heap per warp, for the sea lobes.
    w.heap_warps = cgrid * (kThreads / 32);
    const size_t HC = (size_t)w.heap_warps * cap;
    CG_BUF(int, d_hc, ctx, S_DEPHEAP, 4 * HC);
    w.heap_cells = d_hc;
    w.heap_keys = (float*)(d_hc + HC);
    w.heap_pens = (float*)(d_hc + 2 * HC);
    w.heap_admitted = d_hc + 3 * HC;
    CG_BUF(uint32_t, d_wbits, ctx, S_DEPWBITS, (size_t)w.heap_warps * w.box_words);
    w.warp_bits = d_wbits;
    void* kargs[] = {&w};
    ctx->launches++;
    CG_CUDA(ctx, cudaLaunchCooperativeKernel((void*)k_deposit_levels, cgrid, kThreads, kargs, 0, sm));
    int words[W_WORDS];
    unsigned long long timers[T_COUNT];
    CG_CUDA(ctx, cudaMemcpyAsync(words, d_words, sizeof(words), cudaMemcpyDeviceToHost, sm));
    CG_CUDA(ctx, cudaMemcpyAsync(timers, d_timers, sizeof(timers), cudaMemcpyDeviceToHost, sm));
    CG_CUDA(ctx, cudaStreamSynchronize(sm));
    if (words[W_ERROR] & 32)
        return fail(ctx, CG_INEXACT, "deposition: laying-schedule index check %d failed (value %d, bound %d)",
                    words[W_CHECK_SITE], words[W_CHECK_VALUE], words[W_CHECK_BOUND]);
    if (words[W_ERROR] & 1) return fail(ctx, CG_INEXACT, "deposition: a level's fan deposits overflowed the repair log");
    if (words[W_ERROR] & 2) return fail(ctx, CG_INEXACT, "deposition: a fan's or lobe's admission left its box");
    if (words[W_ERROR] & 4) return fail(ctx, CG_INEXACT, "deposition: the lake fans' laying waves did not converge");
    if (words[W_ERROR] & 8) return fail(ctx, CG_INEXACT, "deposition: a level's mouth refits did not converge");
    if (words[W_ERROR] & 16) return fail(ctx, CG_INEXACT, "deposition: a chunk's fan cells overflowed the schedule");
    if (counts) {
        counts->replayed = words[W_REPLAYED];
        counts->waves = words[W_WAVES];
        counts->refitted = words[W_REFITTED];
        counts->redone = words[W_RELAID];
        counts->ms_walks = timers[T_WALKS] * 1e-6;
        counts->ms_schedule = timers[T_SCHEDULE] * 1e-6;
        counts->ms_lakes = timers[T_LAKES] * 1e-6;
        counts->ms_seas = timers[T_SEAS] * 1e-6;
        counts->ms_repairs = timers[T_REPAIRS] * 1e-6;
    }
    return CG_OK;
}

cg_status deposit_settle_dev(cg_ctx* ctx, int W, int H, float* d_h) {
    const size_t N = (size_t)W * H;
    CG_BUF(float, d_sediment, ctx, S_SEDIMENT, N);
    CG_LAUNCH(ctx) k_settle<<<ctx->num_sms * 8, 256, 0, ctx->stream>>>(d_h, d_sediment, N);
    CG_CHECK_LAUNCH(ctx);
    return CG_OK;
}

cg_status open_mouths_dev(cg_ctx* ctx, const cg_erosion_params& p, float* d_h, const float* d_rain) {
    const int W = p.width, H = p.height;
    const size_t N = (size_t)W * H;
    cudaStream_t sm = ctx->stream;
    const ScaleF sc = scale_of(p);
    const RatesF rates = rates_of(p);
    const float land_half = std::fmax(sc.land_half(), 1e-6f);
    const float sea_half = std::fmax(sc.sea_half(), 1e-6f);
    CG_BUF(uint8_t, d_land, ctx, S_OM_LAND, N);
    CG_BUF(float, d_rel, ctx, S_OM_REL, N);
    CG_BUF(float, d_filled, ctx, S_OM_FILLED, N);
    CG_BUF(double, d_surface, ctx, S_SURFACE, N);
    CG_BUF(int32_t, d_recv, ctx, S_OM_RECV, N);
    CG_BUF(int32_t, d_donors, ctx, S_OM_DONORS, N);
    CG_BUF(long long, d_key, ctx, S_OM_KEY, N);
    CG_BUF(float, d_area, ctx, S_OM_AREA, N);
    CG_BUF(float, d_runoff, ctx, S_OM_RUNOFF, N);
    CG_BUF(float, d_sediment, ctx, S_SEDIMENT, N);
    // A fresh cut at today's shoreline, its fill, routing and discharge (HydraulicErosion.kt:1815-1840).
    float shoreline;
    int land_cells;
    CG_TRY_ST(percentile_cut_dev(ctx, W, H, d_h, p.sea_level, land_half, sea_half, 0.0f, d_land, d_rel, &shoreline,
                                 &land_cells));
    if (land_cells == 0) return CG_OK;
    CG_TRY_ST(fill_depressions_dev(ctx, W, H, d_land, d_rel, d_filled, nullptr, nullptr));
    FlatCounts fc{0, 0, 0};
    CG_TRY_ST(flow_directions_dev(ctx, W, H, d_land, d_rel, d_filled, p.seed, rates.cell_height_in_cell_widths,
                                  smooth_field_lattice_columns(p.world_width_km), p.facet_routing != 0,
                                  p.flat_potential != 0, d_recv, d_surface, &fc));
    CG_TRY_ST(runoff_weights_dev(ctx, W, H, d_rain, d_land, land_cells, d_runoff));
    int levels = 0;
    CG_TRY_ST(tree_walk_dev(ctx, W, H, d_land, d_recv, d_runoff, d_key, d_donors, d_area, &levels));
    if (levels <= 0) return CG_OK;
    int* d_bucket;
    int* d_start;
    CG_TRY_ST(level_buckets_dev(ctx, W, H, d_land, d_key, levels, &d_bucket, &d_start));
    MouthsDev d;
    d.W = W;
    d.pond_depth = rates.pond_depth;
    // drawnRiverCellsOn: DRAWN_RIVER_CATCHMENT_KM2 (deltaMinCatchmentKm2's 70000 / 5) in cells.
    d.drawn_river_cells = (float)(14000.0 / (sc.cell_width_km(W) * sc.cell_height_km(H)));
    d.shoreline = shoreline;
    const float step = rates.pond_depth * land_half;
    d.fall_per_cell_width = step * (0.15f / 23.4375f) * (float)sc.cell_width_km(W);   // DISTRIBUTARY_FALL_PER_KM
    d.floor_ = shoreline + step * 0.15f;                                           // LOBE_RIM
    d.step_ns = rates.step_ns;
    d.step_diag = rates.step_diag;
    d.land = d_land;
    d.filled = d_filled;
    d.rel = d_rel;
    d.area = d_area;
    d.recv = d_recv;
    d.spoil = d_sediment;
    d.working = d_h;
    d.start = d_start;
    d.bucket = d_bucket;
    d.levels = levels;
    int per_sm = 0;
    CG_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mouths_levels, 256, 0));
    if (per_sm < 1) return fail(ctx, CG_CUDA, "mouths kernel cannot be resident");
    const int cgrid = ctx->num_sms * (per_sm < 2 ? per_sm : 2);
    void* kargs[] = {&d};
    ctx->launches++;
    CG_CUDA(ctx, cudaLaunchCooperativeKernel((void*)k_mouths_levels, cgrid, 256, kargs, 0, sm));
    return CG_OK;
}

}  // namespace cg
