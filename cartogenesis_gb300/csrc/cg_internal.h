// Declarations shared between the translation units of the library (not part of the C ABI).
#pragma once

#include "cg_common.cuh"

namespace cg {

// ---- thermal (cg_thermal.cu)
cg_status thermal_sweeps_dev(cg_ctx* ctx, int W, int H, float* d_a, float* d_b, cg_thermal_limits lim, int passes,
                             float rate, float** result);
// The sweeps' error word: a region copy whose bounded wait ran out sets it. Reset clears it (async);
// check reads it (synchronises) and answers CG_TIMEOUT when it is set.
cg_status thermal_error_reset_dev(cg_ctx* ctx);
cg_status thermal_error_check(cg_ctx* ctx);
// Sweeps per fused launch when `passes_left` remain (2, or 1 for the last of an odd count), and the
// number of launches that `passes` sweeps take.
int thermal_step(int passes_left);
int thermal_launches(int passes);
struct ThermalLaunch {
    float limit[8];
    float settled;
    float rate;
};
ThermalLaunch thermal_launch_args(cg_thermal_limits lim, float rate);
// One fused launch of k sweeps (k = thermal_step(...)) from src into dst.
cudaError_t thermal_launch(const float* src, float* dst, int W, int H, const ThermalLaunch& t, int k,
                           cudaStream_t stream);

// ---- sea-level cut (cg_cut.cu)
// Row weights of SeaLevelStage.shorelineForFraction and their sequential total, computed once per
// grid shape on the host (a constant table, like a plan's twiddles) and kept on the device.
cg_status row_weights_dev(cg_ctx* ctx, int W, int H, const double** d_weights, double* total);
cg_status percentile_cut_dev(cg_ctx* ctx, int W, int H, const float* d_h, float sea_level, float land_half,
                             float sea_half, float lowstand_share, uint8_t* d_land, float* d_rel, float* h_shoreline,
                             int* h_land_cells);

// ---- fill (cg_fill.cu)
cg_status fill_depressions_dev(cg_ctx* ctx, int W, int H, const uint8_t* d_land, const float* d_rel, float* d_filled,
                               int64_t* ties, int64_t* unresolved);

// ---- routing (cg_route.cu)
struct FlatCounts {
    int flats, kept, raised;
};
cg_status flow_directions_dev(cg_ctx* ctx, int W, int H, const uint8_t* d_land, const float* d_rel,
                              const float* d_filled, int64_t seed, double r, int lattice, bool by_facet,
                              bool over_potential, int32_t* d_recv, double* d_surface, FlatCounts* counts);

// FlowRouting.facetReceiver at every cell of d_mask over the routing surface d_surface (-1 elsewhere).
cg_status facet_receivers_dev(cg_ctx* ctx, int W, int H, const uint8_t* d_mask, const double* d_surface,
                              int64_t seed, double r, int32_t* d_recv);

// ---- drainage tree (cg_tree.cu)
// Donor counts, the Kahn queue keys (level << 32 | deepest source) of FlowRouting.drainageOrder and,
// if d_weights is given, FlowRouting.accumulate's areas, in one last-arriver walk. *h_levels
// (optional, synchronises) receives the number of Kahn levels.
cg_status tree_walk_dev(cg_ctx* ctx, int W, int H, const uint8_t* d_land, const int32_t* d_recv,
                        const float* d_weights, long long* d_key, int32_t* d_donors, float* d_area, int* h_levels);
// The explicit drainage order (land cells sorted by key), for callers that want it.
cg_status order_from_keys_dev(cg_ctx* ctx, int W, int H, const uint8_t* d_land, const long long* d_key,
                              int land_cells, int32_t* d_order);
struct InciseArgs {
    float courant_coefficient;
    float pond_depth;
    float land_cells;
    float land_range;
    float shoreline;
    float step_ns;
    float step_diag;
    int only_above_base;
};
// d_incised_at (may be NULL): per cell, what the incision took off it, in double (profile P2).
cg_status incise_dev(cg_ctx* ctx, int W, int H, const uint8_t* d_land, const int32_t* d_recv, const long long* d_key,
                     int levels, const float* d_ground, const float* d_rel, const float* d_area, const float* d_erod,
                     float* d_surface, const InciseArgs& a, double* d_incised_at = nullptr);
// Land cells bucketed by Kahn level (the high half of the drainage key): d_bucket (N) holds them
// level after level, d_start (levels + 1) each level's first slot. Cells within a level are in no
// particular order.
cg_status level_buckets_dev(cg_ctx* ctx, int W, int H, const uint8_t* d_land, const long long* d_key, int levels,
                            int** d_bucket, int** d_start);
// FlowRouting.spillways on the device: per basin (in the order the reference finds them) its entry,
// pour point, level, floor, fill depth and cell count, in the context's basin block; d_label
// receives each ponded cell's basin. *h_count (synchronises) receives the number of basins.
struct BasinArrays {
    int* entry = nullptr;
    int* spill = nullptr;
    float* level = nullptr;
    float* floor_ = nullptr;
    float* depth = nullptr;
    int* cells = nullptr;
};
cg_status basins_dev(cg_ctx* ctx, int W, int H, const uint8_t* d_land, const float* d_rel, const float* d_filled,
                     const int32_t* d_recv, float pond_depth, int32_t* d_label, BasinArrays* out, int* h_count);
// The same, with the basins copied into host_basins (largest and deepest as the reference keeps them).
cg_status spillways_dev(cg_ctx* ctx, int W, int H, const uint8_t* d_land, const float* d_rel, const float* d_filled,
                        const int32_t* d_recv, float pond_depth, int32_t* d_label, cg_basins* host_basins);

// ---- outlet notch (cg_breach.cu)
struct BreachRates {
    float relative_incision_coefficient;   // HydraulicErosion.Rates.relativeIncisionCoefficient
    float notch_fall_per_cell;             // HydraulicErosion.Rates.notchFallPerCell
    int outlet_reach_cells;                // HydraulicErosion.Rates.outletReachCells
    float pond_depth;
    float step_ns;
    float step_diag;
};
// HydraulicErosion.breach over the basins of this routing: d_rel, d_ground and d_surface are cut in
// place. *h_cells (optional) receives the cells cut. Where sediment is carried (profile P2's rounds)
// d_settled falls with each cut and d_load gathers what it took; both NULL otherwise.
cg_status breach_dev(cg_ctx* ctx, int W, int H, const uint8_t* d_land, float* d_rel, float* d_ground,
                     const int32_t* d_recv, const float* d_area, float land_cells, float land_range,
                     const BreachRates& rates, float* d_surface, int* h_cells, float* d_settled = nullptr,
                     double* d_load = nullptr);

// ---- weights (cg_stage.cu)
// normaliseOverLand (HydraulicErosion.kt:550-569): each cell's rain over the land's mean rain (the
// reference's sequential double sum in cell order); all ones when d_rain is NULL.
cg_status runoff_weights_dev(cg_ctx* ctx, int W, int H, const float* d_rain, const uint8_t* d_land, int land_cells,
                             float* d_runoff);

// ---- deposition, profile P2 (cg_deposit.cu)
// The stage's deposition state at its start: no sediment, fresh fan stamps.
cg_status deposit_stage_reset_dev(cg_ctx* ctx, int W, int H);
// A round's start (HydraulicErosion.kt:940-945): settled = relative + sediment, no load, nothing
// incised; returns the round's settled, load and incisedAt fields (context buffers).
cg_status deposit_round_begin_dev(cg_ctx* ctx, int W, int H, const float* d_rel, float to_relative, float** d_settled,
                                  double** d_load, double** d_incised_at);
// What one round's walk reads: the round's routing, its cut and the fields of deposit_round_begin_dev.
struct DepositRound {
    const int32_t* recv;
    const uint8_t* land;
    const float* ground;      // the filled surface
    const float* rel;
    const float* area;
    const long long* key;     // drainage keys (level << 32 | deepest source)
    int levels;
    int land_cells;
    float land_range, to_relative, shoreline;
    const float* surface;     // the working field after the incision
    float* settled;
    const double* load;       // the notch's hand-offs
    const double* incised_at;
};
struct DepositCounts {
    int redone;     // cells with a mouth refitted, the later fans of their level laid again
    int replayed;   // ponded cells whose settled height was replayed in rank order
    int waves;      // the lake fans' laying waves, over all levels (counted over the stage so far)
    int refitted;   // dry cells whose own walk was taken again with their donors as the walk saw them
    // Device-clock milliseconds of the walk's parts: own walks and listing, laying schedules, laying
    // waves, sea lobes and logs, mouth refits and last repairs.
    double ms_walks, ms_schedule, ms_lakes, ms_seas, ms_repairs;
};
// The reference's sequential double sum (`s += v` in cell order, s from 0.0) of v = x (mode 0) or
// v = 1 - 0.5 x (mode 1) over the cells of d_mask (all cells when null), into *d_out on the device,
// divided by `divisor` unless it is 0; bit for bit, in parallel (cg_seqsum.cu). d_counts (3, may be
// null) receives how the sum went: blocks of 8192 values taken whole, pieces of 1024 reduced on the
// spot, pieces added one value at a time.
cg_status seq_sum_dev(cg_ctx* ctx, const float* d_x, const uint8_t* d_mask, int mode, size_t n, double divisor,
                      double* d_out, long long* d_counts);
// The same sequential sum (`s += v`, s from 0.0) over n double terms already laid out in the order the
// reference adds them, bit for bit; a running total is carried by laying it first.
cg_status seq_sum_f64_dev(cg_ctx* ctx, const double* d_x, size_t n, double* d_out);
// The plate flexure of profile P3 (cg_flexure.cu). flexure_check refuses grids whose transform lines
// do not fit a CTA's shared memory; flexure_stage_begin_dev records the field before the rounds and
// clears the bend (and the uplift record when the world has uplift); flexure_uplifted_dev is that
// record, for k_uplift; flexure_round_dev bends the surface under the rounds' load so far.
cg_status flexure_check(cg_ctx* ctx, int W, int H);
cg_status flexure_stage_begin_dev(cg_ctx* ctx, const cg_erosion_params& p, const float* d_work, bool uplift);
float* flexure_uplifted_dev(cg_ctx* ctx, const cg_erosion_params& p);
cg_status flexure_round_dev(cg_ctx* ctx, const cg_erosion_params& p, float* d_work, const float* d_sediment,
                            bool uplift);
// The deposition walk of one round (HydraulicErosion.kt:1068-1349), the sediment in the stage's buffer.
cg_status deposit_walk_dev(cg_ctx* ctx, const cg_erosion_params& p, const DepositRound& r, DepositCounts* counts);
// settle() (HydraulicErosion.kt:1351-1364): the sediment laid on d_h; the sediment is kept as the spoil.
cg_status deposit_settle_dev(cg_ctx* ctx, int W, int H, float* d_h);
// openMouths (HydraulicErosion.kt:1804-1892) over d_h, with the spoil of deposit_settle_dev. Routes on
// buffers of its own: the stage's last routing is left as it was.
cg_status open_mouths_dev(cg_ctx* ctx, const cg_erosion_params& p, float* d_h, const float* d_rain);

// ---- the belts' replay (cg_belt.cu)
// The replay's per-cell inputs on the device: the window (tectonic, wear, onset) required, rain and
// cover always present (belt_weather_dev fills ones and zeros for null), the rest may be null.
struct BeltInputsDev {
    const float* tectonic;
    const float* wear;
    const float* onset;
    const float* uplift;
    const float* rain;
    const float* cover;
    const float* rock;
    const float* unresolved;
};
// Uploads the window's three fields into the replay's slots.
cg_status belt_window_dev(cg_ctx* ctx, const cg_erosion_params& p, const cg_belt_window& w, BeltInputsDev* in);
// Sets the replay's rain and cover to the given device fields, or to ones and zeros where null.
cg_status belt_weather_dev(cg_ctx* ctx, int W, int H, const float* d_rain, const float* d_cover, BeltInputsDev* in);
// BeltErosion.replay (BeltErosion.kt:96-425) on the device field d_h (replayed in place); d_eroded
// (N) receives the metres each cell lost. Of `opt` it reads the sea level, shield_cut, rebound and
// history_cell_km (its pointers are the host call's, unused here). Synchronises before it returns.
cg_status belt_replay_dev(cg_ctx* ctx, const cg_erosion_params& p, float* d_h, const BeltInputsDev& in,
                          double window_myr, const cg_belt_inputs& opt, float* d_eroded, cg_belt_books* books);

// ---- small helpers (cg_api.cu)
cg_status sync(cg_ctx* ctx);

}  // namespace cg
