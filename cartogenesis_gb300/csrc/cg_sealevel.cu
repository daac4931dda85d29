// SeaLevelStage.apply's cut up to the drowned basins' outlets (SeaLevelStage.kt:243-270) on the
// device: the percentile cut, the enclosure rule (markUnreachableWaterAsLand, SeaLevelStage.kt:
// 371-437) and the post-cut outlet passes (drainDrownedBasins, SeaLevelStage.kt:478-560). This is
// the reference reusing the erosion stage's routing outside it (FlowRouting.kt:14-17): each pass is
// a fill, a routing, an accumulation and the spillways over the whole grid, then the outlet notch run
// again with belowSea on, over the basins whose floor lies below the shoreline.
//
// The enclosure rule labels the water's 8-connected bodies (the same union-find labels as the
// basins, numbered by their lowest cell, which is the order the reference's scan finds them in);
// the ocean is the largest body, the first found of that size. The belowSea notch runs on one thread
// over the basins in the order spillways found them: only the drowned basins cut (a handful a pass),
// and the lake-bed walk that belowSea adds follows the ponded cells as the cutting leaves them, so
// its footprint is not known before the cut.
#include <cmath>

#include "cg_common.cuh"
#include "cg_internal.h"
#include "cg_params.h"
#include "cg_util.h"

namespace cg {
namespace {

__global__ void k_water_mask(const uint8_t* __restrict__ land, size_t N, uint8_t* __restrict__ mask) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x)
        mask[i] = land[i] ? 0 : 1;
}

__global__ void k_body_sizes(const int* __restrict__ label, size_t N, int* __restrict__ size) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x)
        if (label[i] >= 0) atomicAdd(&size[label[i]], 1);
}

// The ocean: the largest body, the lowest label (the first found) among equals.
__global__ void k_ocean(const int* __restrict__ size, int count, unsigned long long* __restrict__ best) {
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < count; b += gridDim.x * blockDim.x)
        atomicMax(best, ((unsigned long long)(unsigned)size[b] << 32) | (unsigned long long)(0xFFFFFFFFu - (unsigned)b));
}

// Every water body but the ocean, no larger than the largest lake, becomes land at its own height.
__global__ void k_enclose(uint8_t* __restrict__ land, float* __restrict__ rel, const int* __restrict__ label,
                          const int* __restrict__ size, const unsigned long long* __restrict__ best, int largest,
                          const float* __restrict__ h, float shoreline, float land_half, size_t N, int* __restrict__ added) {
    const int ocean = (int)(0xFFFFFFFFu - (unsigned)(*best & 0xFFFFFFFFull));
    int mine = 0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x) {
        const int b = label[i];
        if (b < 0 || b == ocean || size[b] > largest) continue;
        land[i] = 1;
        rel[i] = __fdiv_rn(__fsub_rn(h[i], shoreline), land_half);
        ++mine;
    }
    if (mine) atomicAdd(added, mine);
}

// SeaLevelStage.landAndWaterAt at a given shoreline.
__global__ void k_land_water_at(const float* __restrict__ h, size_t N, float shoreline, float land_half, float sea_half,
                                uint8_t* __restrict__ land, float* __restrict__ rel, int* __restrict__ count) {
    int mine = 0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x) {
        const float g = h[i];
        const bool on = g >= shoreline;
        land[i] = on ? 1 : 0;
        rel[i] = __fdiv_rn(__fsub_rn(g, shoreline), on ? land_half : sea_half);
        mine += on ? 1 : 0;
    }
    if (mine) atomicAdd(count, mine);
}

// Basins whose floor stands at or above the shoreline are the rounds' notch's: their spill is
// cleared. Counts the drowned basins that keep a spill.
__global__ void k_mark_drowned(int* __restrict__ spill, const float* __restrict__ floor_, int count,
                               int* __restrict__ drowned) {
    int mine = 0;
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < count; b += gridDim.x * blockDim.x) {
        if (floor_[b] >= 0.0f) spill[b] = -1;
        else if (spill[b] >= 0) ++mine;
    }
    if (mine) atomicAdd(drowned, mine);
}

struct NotchArgs {
    int W, H, count;
    const int* spill;
    const int* entry;
    const float* level;
    const float* floor_;
    const uint8_t* land;
    const int32_t* dirs;
    const float* area;
    float* rel;
    float* ground;
    float* surface;
    float land_cells, land_range, pond_depth, coefficient, gradient, reach, step_ns, step_diag;
    int* cells;
};

__device__ __forceinline__ float jvm_minf(float a, float b) {
    if (a != a) return a;
    if (b != b) return b;
    if (a == 0.0f && b == 0.0f) return __float_as_int(a) < 0 ? a : b;
    return a < b ? a : b;
}

__device__ __forceinline__ float step_between(const NotchArgs& a, int from, int to) {
    const bool same_row = from / a.W == to / a.W, same_col = from % a.W == to % a.W;
    return (!same_row && !same_col) ? a.step_diag : (!same_row ? a.step_ns : 1.0f);
}

// HydraulicErosion.raise with -take, and the relative fields it lowers; returns whether it cut.
__device__ bool take_down(const NotchArgs& a, int cell, float cut_level, bool lower_ground) {
    const double take = (double)(a.rel[cell] - cut_level) * (double)a.land_range;
    const bool ponded = a.ground[cell] - a.rel[cell] > a.pond_depth;
    const float prior = a.surface[cell];
    a.surface[cell] = (float)((double)prior + -take);
    const double removed = -((double)a.surface[cell] - (double)prior);
    if (removed > 0.0) {
        const float as_relative = (float)(removed / (double)a.land_range);
        a.rel[cell] -= as_relative;
        if (lower_ground && !ponded) a.ground[cell] -= as_relative;
        return true;
    }
    return false;
}

// HydraulicErosion.breach with belowSea on (HydraulicErosion.kt:1931-2171), the basins in order.
__global__ void k_notch_below_sea(NotchArgs a) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    int cells = 0;
    for (int b = 0; b < a.count; ++b) {
        const int spill = a.spill[b];
        if (spill < 0) continue;
        const float level = a.level[b], floor_ = a.floor_[b];
        if (level - floor_ <= 0.0f) continue;
        float fall = 0.0f, length = 0.0f, last_step = 1.0f;
        int walked = 0, cell = spill;
        while (cell >= 0 && a.land[cell] && length < a.reach) {
            fall = level - a.rel[cell];
            if (fall > level - floor_) break;
            const int next = a.dirs[cell];
            last_step = next >= 0 ? step_between(a, cell, next) : 1.0f;
            length += last_step;
            walked++;
            cell = next;
        }
        if (fall <= 1e-6f * (float)walked && cell >= 0 && !a.land[cell]) {   // outletFallToTheWater
            fall = level - a.rel[cell];
            length += last_step;
        }
        if (walked == 0) continue;
        float slope = fall / length * (float)a.W;
        if (slope < 0.0f) slope = 0.0f;
        const float power = a.coefficient * sqrtf(a.area[spill] / a.land_cells) * slope;
        const float drop = jvm_minf(power, level - floor_);
        if (drop <= 0.0f) continue;
        const float new_level = level - drop;
        float from_lip = 0.0f;
        cell = spill;
        while (cell >= 0 && a.land[cell] && from_lip < a.reach) {
            const float cut_level = new_level - from_lip * a.gradient;
            if (a.rel[cell] <= cut_level) break;
            if (take_down(a, cell, cut_level, true)) cells++;
            const int next = a.dirs[cell];
            from_lip += next >= 0 ? step_between(a, cell, next) : 1.0f;
            cell = next;
        }
        const int entry = a.entry[b];
        float back = 0.0f;
        if (entry >= 0 && entry != spill) {
            int margin_cells = 0, walker = entry;
            float widths = 0.0f;
            while (walker >= 0 && walker != spill && a.land[walker] && widths <= a.reach) {
                const int next = a.dirs[walker];
                widths += next >= 0 ? step_between(a, walker, next) : 1.0f;
                margin_cells++;
                walker = next;
            }
            if (walker == spill) {
                // The margin from the lip back towards the entry: the chain entry -> ... -> spill,
                // walked backwards by recounting from the entry (margin_cells stays within the reach).
                int downstream = spill;
                for (int i = margin_cells - 1; i >= 0; --i) {
                    int m = entry;
                    for (int j = 0; j < i; ++j) m = a.dirs[m];
                    back += step_between(a, m, downstream);
                    const float cut_level = new_level + back * a.gradient;
                    if (a.rel[m] <= cut_level) break;
                    if (take_down(a, m, cut_level, true)) cells++;
                    downstream = m;
                }
            }
        }
        // The sill on the basin's own side: up the inflow of the largest catchment across the bed.
        int from = entry >= 0 ? entry : spill;
        while (back <= a.reach) {
            int best = -1;
            float best_area = -1.0f;
            const int col = from % a.W, row = from / a.W;
            for (int rs = -1; rs <= 1; ++rs) {
                const int nr = row + rs;
                if (nr < 0 || nr >= a.H) continue;
                for (int cs = -1; cs <= 1; ++cs) {
                    if (rs == 0 && cs == 0) continue;
                    const int n = nr * a.W + ((col + cs) & (a.W - 1));
                    if (a.land[n] && a.dirs[n] == from && a.ground[n] - a.rel[n] > a.pond_depth) {
                        const float ar = a.area[n];
                        const bool ties = ar == best_area && (best < 0 || n < best);
                        if (ar > best_area || ties) {
                            best_area = ar;
                            best = n;
                        }
                    }
                }
            }
            if (best < 0) break;
            back += step_between(a, best, from);
            if (back > a.reach) break;
            const float cut_level = new_level + back * a.gradient;
            if (a.rel[best] <= cut_level) break;
            if (take_down(a, best, cut_level, false)) cells++;
            from = best;
        }
    }
    *a.cells = cells;
}

cg_status enclose_dev(cg_ctx* ctx, int W, int H, uint8_t* d_land, float* d_rel, const float* d_h, float shoreline,
                      float land_half, int largest_lake, int* land_cells) {
    const size_t N = (size_t)W * H;
    cudaStream_t sm = ctx->stream;
    const int grid = ctx->num_sms * 8;
    CG_BUF(uint8_t, d_mask, ctx, S_SL_MASK, N);
    CG_BUF(int, d_root, ctx, S_LABEL, N);
    CG_BUF(int, d_label, ctx, S_SL_LABEL, N);
    CG_LAUNCH(ctx) k_water_mask<<<grid, 256, 0, sm>>>(d_land, N, d_mask);
    CG_CHECK_LAUNCH(ctx);
    int bodies = 0;
    CG_TRY_ST(component_labels(ctx, W, H, d_mask, d_root, d_label, &bodies));
    if (bodies <= 1) return CG_OK;
    CG_BUF(int, d_size, ctx, S_SL_SIZE, (size_t)bodies + 4);
    unsigned long long* d_best = (unsigned long long*)(d_size + bodies + (bodies & 1));
    int* d_added = (int*)(d_best + 1);
    CG_CUDA(ctx, cudaMemsetAsync(d_size, 0, ((size_t)bodies + 4) * sizeof(int), sm));
    CG_LAUNCH(ctx) k_body_sizes<<<grid, 256, 0, sm>>>(d_label, N, d_size);
    CG_LAUNCH(ctx) k_ocean<<<(bodies + 255) / 256, 256, 0, sm>>>(d_size, bodies, d_best);
    CG_LAUNCH(ctx) k_enclose<<<grid, 256, 0, sm>>>(d_land, d_rel, d_label, d_size, d_best, largest_lake, d_h, shoreline,
                                                 land_half, N, d_added);
    CG_CHECK_LAUNCH(ctx);
    int added = 0;
    CG_CUDA(ctx, cudaMemcpyAsync(&added, d_added, sizeof(int), cudaMemcpyDeviceToHost, sm));
    CG_CUDA(ctx, cudaStreamSynchronize(sm));
    *land_cells += added;
    return CG_OK;
}

}  // namespace
}  // namespace cg

using namespace cg;

extern "C" cg_status cg_sea_level_cut(cg_ctx* ctx, const cg_erosion_params* p, const float* height,
                                      double enclosed_sea_max_share, int32_t post_cut_outlet, float* shoreline,
                                      uint8_t* is_land, float* relative, int32_t* land_cells, int32_t* passes) {
    if (!ctx || !p || !height || !shoreline || !is_land || !relative || !land_cells) return CG_BAD_ARG;
    ctx->run.active = false;   // this call reuses the resident world's buffers
    const int W = p->width, H = p->height;
    if (W <= 0 || H <= 0 || (W & (W - 1)) || (H & (H - 1)) || (int64_t)W * H > ((int64_t)1 << 30))
        return fail(ctx, CG_BAD_ARG, "width/height must be powers of two (got %d x %d)", W, H);
    if (p->abi_version != CG_ABI_VERSION) return fail(ctx, CG_BAD_ARG, "params carry ABI version %u", p->abi_version);
    if (!(enclosed_sea_max_share >= 0.0)) return fail(ctx, CG_BAD_ARG, "negative enclosed-sea share");
    CG_CUDA(ctx, cudaSetDevice(ctx->device));
    const size_t N = (size_t)W * H;
    cudaStream_t sm = ctx->stream;
    const int grid = ctx->num_sms * 8;
    const ScaleF sc = scale_of(*p);
    const RatesF rates = rates_of(*p);
    const float land_half = std::fmax(sc.land_half(), 1e-6f);
    const float sea_half = std::fmax(sc.sea_half(), 1e-6f);
    const double km2_per_cell = sc.cell_width_km(W) * sc.cell_height_km(H);
    const int largest_lake = (int)(enclosed_sea_max_share * sc.world_area_km2() / km2_per_cell);
    CG_BUF(float, d_h, ctx, S_H0, N);
    CG_BUF(float, d_terrain, ctx, S_H1, N);
    CG_BUF(uint8_t, d_land, ctx, S_LAND, N);
    CG_BUF(float, d_rel, ctx, S_REL, N);
    CG_BUF(float, d_filled, ctx, S_FILLED, N);
    CG_BUF(double, d_surface, ctx, S_SURFACE, N);
    CG_BUF(int32_t, d_recv, ctx, S_RECV, N);
    CG_BUF(int32_t, d_donors, ctx, S_DONORS, N);
    CG_BUF(long long, d_key, ctx, S_KEY, N);
    CG_BUF(float, d_area, ctx, S_AREA, N);
    CG_BUF(float, d_ones, ctx, S_RUNOFF, N);
    CG_BUF(int32_t, d_bl, ctx, S_BASIN2, N);
    CG_BUF(int, d_words, ctx, S_SL_WORDS, 4);
    CG_CUDA(ctx, cudaMemcpyAsync(d_h, height, N * 4, cudaMemcpyHostToDevice, sm));
    float s = 0.0f;
    int n = 0;
    CG_TRY_ST(percentile_cut_dev(ctx, W, H, d_h, p->sea_level, land_half, sea_half, 0.0f, d_land, d_rel, &s, &n));
    CG_TRY_ST(enclose_dev(ctx, W, H, d_land, d_rel, d_h, s, land_half, largest_lake, &n));
    int run = 0;
    bool have_terrain = false;
    for (int pass = 0; post_cut_outlet && pass < 16 && n > 0; ++pass) {   // MAX_POST_CUT_OUTLET_PASSES
        CG_TRY_ST(fill_depressions_dev(ctx, W, H, d_land, d_rel, d_filled, nullptr, nullptr));
        FlatCounts fc{0, 0, 0};
        CG_TRY_ST(flow_directions_dev(ctx, W, H, d_land, d_rel, d_filled, p->seed, rates.cell_height_in_cell_widths,
                                      smooth_field_lattice_columns(p->world_width_km), p->facet_routing != 0,
                                      p->flat_potential != 0, d_recv, d_surface, &fc));
        CG_TRY_ST(runoff_weights_dev(ctx, W, H, nullptr, d_land, n, d_ones));
        CG_TRY_ST(tree_walk_dev(ctx, W, H, d_land, d_recv, d_ones, d_key, d_donors, d_area, nullptr));
        BasinArrays bas;
        int count = 0;
        CG_TRY_ST(basins_dev(ctx, W, H, d_land, d_rel, d_filled, d_recv, rates.pond_depth, d_bl, &bas, &count));
        if (count == 0) break;
        CG_CUDA(ctx, cudaMemsetAsync(d_words, 0, 4 * sizeof(int), sm));
        CG_LAUNCH(ctx) k_mark_drowned<<<(count + 255) / 256, 256, 0, sm>>>(bas.spill, bas.floor_, count, d_words);
        CG_CHECK_LAUNCH(ctx);
        int drowned = 0;
        CG_CUDA(ctx, cudaMemcpyAsync(&drowned, d_words, sizeof(int), cudaMemcpyDeviceToHost, sm));
        CG_CUDA(ctx, cudaStreamSynchronize(sm));
        if (drowned == 0) break;
        if (!have_terrain) {
            CG_CUDA(ctx, cudaMemcpyAsync(d_terrain, d_h, N * 4, cudaMemcpyDeviceToDevice, sm));
            have_terrain = true;
        }
        run = pass + 1;
        NotchArgs a;
        a.W = W;
        a.H = H;
        a.count = count;
        a.spill = bas.spill;
        a.entry = bas.entry;
        a.level = bas.level;
        a.floor_ = bas.floor_;
        a.land = d_land;
        a.dirs = d_recv;
        a.area = d_area;
        a.rel = d_rel;
        a.ground = d_filled;
        a.surface = d_terrain;
        a.land_cells = (float)n;
        a.land_range = land_half;
        a.pond_depth = rates.pond_depth;
        a.coefficient = rates.relative_incision_coefficient * 1.125f;   // ErosionConfig.outletIncisionRatio
        a.gradient = rates.notch_fall_per_cell;
        a.reach = (float)rates.outlet_reach_cells;
        a.step_ns = rates.step_ns;
        a.step_diag = rates.step_diag;
        a.cells = d_words + 1;
        CG_LAUNCH(ctx) k_notch_below_sea<<<1, 32, 0, sm>>>(a);
        CG_CHECK_LAUNCH(ctx);
        int cut = 0;
        CG_CUDA(ctx, cudaMemcpyAsync(&cut, d_words + 1, sizeof(int), cudaMemcpyDeviceToHost, sm));
        CG_CUDA(ctx, cudaStreamSynchronize(sm));
        if (cut == 0) break;
        // The re-cut at the same shoreline over the cut terrain, and the enclosure rule again.
        CG_CUDA(ctx, cudaMemsetAsync(d_words + 2, 0, sizeof(int), sm));
        CG_LAUNCH(ctx) k_land_water_at<<<grid, 256, 0, sm>>>(d_terrain, N, s, land_half, sea_half, d_land, d_rel,
                                                           d_words + 2);
        CG_CHECK_LAUNCH(ctx);
        CG_CUDA(ctx, cudaMemcpyAsync(&n, d_words + 2, sizeof(int), cudaMemcpyDeviceToHost, sm));
        CG_CUDA(ctx, cudaStreamSynchronize(sm));
        CG_TRY_ST(enclose_dev(ctx, W, H, d_land, d_rel, d_terrain, s, land_half, largest_lake, &n));
    }
    CG_CUDA(ctx, cudaMemcpyAsync(is_land, d_land, N, cudaMemcpyDeviceToHost, sm));
    CG_CUDA(ctx, cudaMemcpyAsync(relative, d_rel, N * 4, cudaMemcpyDeviceToHost, sm));
    CG_TRY_ST(sync(ctx));
    *shoreline = s;
    *land_cells = n;
    if (passes) *passes = run;
    return CG_OK;
}
