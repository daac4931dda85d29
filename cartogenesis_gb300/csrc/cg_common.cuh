// Shared device helpers and the context of the GB300 erosion stage.
//
// Every kernel of this library is compiled with --fmad=false and IEEE division and square root:
// the reference runs on the JVM, which never fuses a multiply and an add, and the REF32 mode
// reproduces its float arithmetic bit for bit.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <cstdio>
#include <cstring>

#include "../../include/cg_erosion.h"

namespace cg {

constexpr int kSMs = 152;   // GB300: 2 dies x 76 SMs

// Neighbour order of ErosionStage's thermal sweep (ErosionStage.kt:460-461): E, W, S, N, then the
// diagonals (+1,+1), (+1,-1), (-1,+1), (-1,-1) as (column step, row step).
__host__ __device__ constexpr int thermal_col_step(int n) { return n == 0 ? 1 : n == 1 ? -1 : n < 4 ? 0 : (n < 6 ? 1 : -1); }
__host__ __device__ constexpr int thermal_row_step(int n) { return n == 0 || n == 1 ? 0 : n == 2 ? 1 : n == 3 ? -1 : ((n & 1) == 0 ? 1 : -1); }

// Grid sides are powers of two (every entry point checks, the noalloc sweeps included), so a
// division or remainder of a non-negative index by a side is a shift or a mask, and a column wraps
// by masking (for any int column, negative ones included).
__device__ __forceinline__ int pdiv(int x, int n) { return x >> (31 - __clz(n)); }
__device__ __forceinline__ int pmod(int x, int n) { return x & (n - 1); }
__device__ __forceinline__ int wrap_col(int c, int W) { return c & (W - 1); }

// Float <-> raw bits, as Float.toRawBits.
__device__ __forceinline__ int32_t float_bits(float f) { return __float_as_int(f); }

// Growable device buffer owned by the context.
struct DevBuf {
    void* ptr = nullptr;
    size_t bytes = 0;
};

struct Timer;

// A stage whose world stays resident on the context between calls (cg_stage_begin, cg_erode_rounds,
// cg_stage_finish), and the state the round loop carries from one round to the next.
struct StageRun {
    cg_erosion_params p{};
    float* cur = nullptr;          // the working field
    float* other = nullptr;        // its ping-pong partner
    const float* uplift = nullptr; // inputs, device (or NULL)
    const float* rock = nullptr;
    const float* rain = nullptr;
    const float* veg = nullptr;
    int next_round = 0;            // rounds run so far
    int land_cells = -1;           // the last routed round's land cells (-1: none routed)
    bool done = false;             // no round is left to run (all run, or one found no land)
    bool active = false;           // a resident world is held by the round-range entry points
};

}  // namespace cg

// The library context (opaque in the C ABI).
struct cg_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    // Two more streams for work that overlaps the main one inside a call (forked from and joined
    // back into `stream` with the events), so callers only ever see `stream`.
    cudaStream_t aux = nullptr, aux2 = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr, join2 = nullptr;
    std::atomic<int> cancel{0};
    char error[512] = {0};
    // Named scratch buffers, grown on demand and reused across calls.
    cg::DevBuf bufs[200];
    // Pinned host staging.
    void* pinned = nullptr;
    size_t pinned_bytes = 0;
    int num_sms = cg::kSMs;
    // Row-weight table of the sea-level cut, cached for the last grid shape.
    int rw_w = 0, rw_h = 0;
    double rw_total = 0.0;
    // The plate flexure's twiddle tables, cached for the last line lengths; its line kernel's
    // shared-memory limit, raised once.
    int flex_tw_w = 0, flex_tw_h2 = 0;
    bool flex_attr = false;
    // Kernels launched on this context (every launch site counts itself with CG_LAUNCH).
    long long launches = 0;
    // The resident world of the round-range entry points (inactive otherwise).
    cg::StageRun run;
};

// Prefix of every kernel launch statement: `CG_LAUNCH(ctx) k<<<...>>>(...);` counts the launch.
#define CG_LAUNCH(ctx) ((ctx)->launches++),

namespace cg {

// Buffer slots of cg_ctx::bufs.
enum Slot {
    S_H0, S_H1, S_GIVE, S_UPLIFT, S_ROCK, S_RAIN, S_VEG, S_RUNOFF, S_ERODE, S_LAND, S_REL, S_FILLED,
    S_SURFACE, S_RECV, S_DONORS, S_KEY, S_ORDER, S_AREA, S_WATER, S_LABEL, S_PTR, S_PTR2, S_SCRATCH0,
    S_SCRATCH1, S_SCRATCH2, S_SCRATCH3, S_ROWW, S_HIST, S_BRACKET, S_BRACKET2, S_SMALL, S_FLATS,
    S_FLATIDX, S_FLATMEM, S_CG0, S_CG1, S_CG2, S_CG3, S_CG4, S_CG5, S_LEVELCNT, S_DEPTH, S_STATS,
    S_BASIN, S_BASIN2, S_FILLQ, S_FILLF, S_FILLFLAG, S_TILEFLAG, S_SCRATCH4, S_SCRATCH5, S_THERMFLAG,
    S_LINKS, S_SOURCES, S_FILLLIST, S_CLAIM, S_FOOT, S_BREACH,
    // profile P2's deposition: the stage's state, a round's walk, and the mouths pass's own routing
    S_SEDIMENT, S_STAMP, S_DEPWORDS, S_DEPMARK, S_SETTLED, S_LOAD, S_INCISED, S_DEPRANK, S_DEPLEVEL,
    S_HANDOFF, S_DEPUSED, S_DEPS0, S_DEPD0, S_DEPEVC, S_DEPEVK, S_DEPSEG, S_DEPEVENTS, S_DEPEVTOUCH,
    S_DEPSLOT0, S_DEPSLOT1, S_DEPSLOT2, S_DEPSLOT3, S_DEPSLOT4, S_DEPSLOT5, S_DEPSLOT6, S_DEPSLOT7,
    S_DEPHEAP, S_DEPTOUCH, S_DEPREPLAY, S_DEPSEGC,
    S_OM_LAND, S_OM_REL, S_OM_FILLED, S_OM_RECV, S_OM_KEY, S_OM_AREA, S_OM_RUNOFF, S_OM_DONORS,
    S_FILLEB, S_THERMERR, S_SL_MASK, S_SL_LABEL, S_SL_SIZE, S_SL_WORDS, S_DEPSLOT8, S_DEPSLOT9, S_DEPSLOT10,
    S_DEPCLAIM, S_DEPCANDOF, S_DEPCAND, S_DEPCANDN, S_DEPCANDOFF, S_DEPCANDW, S_DEPSLOTOFF, S_DEPACC, S_DEPOWN, S_DEPCELLCNT, S_DEPTIMERS, S_DEPRLIST, S_DEPWBITS, S_SS_EST, S_SS_SPEC, S_SS_WALK, S_SS_X, S_SS_MASK, S_SS_OUT, S_DEPFIRST, S_DEPTOUCHEV, S_RS_KEYS, S_RS_VALS, S_RS_HIST,
    S_FX_TW, S_FX_A, S_FX_B, S_FX_MEAN, S_FX_REF, S_FX_DEFL, S_FX_UPL, S_FX_LOAD,
    // the belts' replay: its inputs, the belt and its frontier, the opening's routing, a round's state
    S_BT_H, S_BT_TECT, S_BT_WEAR, S_BT_ONSET, S_BT_UPLIFT, S_BT_RAIN, S_BT_COVER, S_BT_ROCK, S_BT_UNRES,
    S_BT_BELT, S_BT_INNER, S_BT_ROUTED, S_BT_LAND, S_BT_REL, S_BT_FLAG, S_BT_POS, S_BT_LIST, S_BT_LOCAL,
    S_BT_FIRST, S_BT_RISE, S_BT_WEIGHTS, S_BT_FACTOR, S_BT_FILLED, S_BT_SURF, S_BT_RECV, S_BT_KEY,
    S_BT_DONORS, S_BT_AREA, S_BT_INFLOW, S_BT_ROUTING, S_BT_DISC, S_BT_FLUX, S_BT_CUTV, S_BT_GIVE,
    S_BT_NEXT, S_BT_ORDER, S_BT_XS, S_BT_REF, S_BT_UPLM, S_BT_RBM, S_BT_LOSS, S_BT_TMP, S_BT_TAPS,
    S_BT_SMALL, S_BT_ERODED,
    S_COUNT
};
static_assert(S_COUNT <= (int)(sizeof(((cg_ctx*)nullptr)->bufs) / sizeof(DevBuf)), "a slot past the context's buffers");

cg_status fail(cg_ctx* ctx, cg_status st, const char* fmt, ...);
cg_status cuda_fail(cg_ctx* ctx, cudaError_t e, const char* what, const char* file, int line);
// Returns a device pointer of at least `bytes` for `slot`, growing it if needed.
void* buf(cg_ctx* ctx, int slot, size_t bytes, cg_status* st);
void* pinned(cg_ctx* ctx, size_t bytes, cg_status* st);

}  // namespace cg

#define CG_CUDA(ctx, call)                                                       \
    do {                                                                         \
        cudaError_t e_ = (call);                                                 \
        if (e_ != cudaSuccess) return cg::cuda_fail((ctx), e_, #call, __FILE__, __LINE__); \
    } while (0)

#define CG_CHECK_LAUNCH(ctx) CG_CUDA(ctx, cudaGetLastError())

// Returns the status of `x` when it is not CG_OK.
#define CG_TRY_ST(x)                    \
    do {                                \
        cg_status s_ = (x);             \
        if (s_ != CG_OK) return s_;     \
    } while (0)

#define CG_BUF(T, name, ctx, slot, count)                                        \
    T* name;                                                                     \
    {                                                                            \
        cg_status st_ = CG_OK;                                                   \
        name = (T*)cg::buf((ctx), (slot), sizeof(T) * (size_t)(count), &st_);    \
        if (st_ != CG_OK) return st_;                                            \
    }
