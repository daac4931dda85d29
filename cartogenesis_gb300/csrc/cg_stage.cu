// ErosionStage.apply on the device (ErosionStage.kt:133-183 with HydraulicErosion.apply,
// HydraulicErosion.kt:596-1506) in profiles P0, P1 and P2, whole or a range of rounds at a time, and
// the C entry points that run one routing function on host buffers.
//
// The world stays resident in HBM for the whole stage: heights ping-pong between two buffers, and
// each round's masks, fields, receivers and tree live in context buffers reused round to round (P2's
// sediment too, carried from round to round). The host sequences the phases and reads back one
// shoreline and one land count per round.
#include <cmath>
#include <vector>

#include "cg_common.cuh"
#include "cg_internal.h"
#include "cg_params.h"
#include "cg_util.h"

namespace cg {

namespace {

// HydraulicErosion.kt:824-837: h += rate * upliftMetresPerRoundPerMm / metresPerFieldUnit where rate > 0.
__global__ void k_uplift(float* __restrict__ h, const float* __restrict__ rate, size_t N, float per_mm,
                         float metres_per_field, float* __restrict__ uplifted) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x) {
        float r = rate[i];
        if (r <= 0.0f) continue;
        const float metres = __fmul_rn(r, per_mm);
        h[i] = __fadd_rn(h[i], __fdiv_rn(metres, metres_per_field));
        if (uplifted) uplifted[i] = __fadd_rn(uplifted[i], metres);   // the plate flexure's record (P3)
    }
}

// The weights with no weather given: rain all 1 (mean 1, weight 1) and no cover (factor 1), times
// the rock's factor. normaliseOverLand / shieldingOverLand reduce to exactly these ones.
__global__ void k_unit_weights(const float* __restrict__ rock, size_t N, float* __restrict__ runoff,
                               float* __restrict__ erod) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x) {
        runoff[i] = 1.0f;
        erod[i] = rock ? __fmul_rn(1.0f, rock[i]) : 1.0f;
    }
}

// weights[c] = rain[c] / mean, or 0 when mean <= 0 (HydraulicErosion.kt:558-567).
__global__ void k_normalise(const float* __restrict__ rain, const double* __restrict__ sum, int land_cells, size_t N,
                            float* __restrict__ w) {
    float mean = (float)__ddiv_rn(*sum, (double)land_cells);
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x)
        w[i] = mean <= 0.0f ? 0.0f : __fdiv_rn(rain[i], mean);
}

// erod[c] = (1 - 0.5 d) / mean, or 1 when mean <= 0 (HydraulicErosion.kt:479-486), times the rock.
__global__ void k_shield(const float* __restrict__ veg, const double* __restrict__ sum, int land_cells,
                         const float* __restrict__ rock, size_t N, float* __restrict__ e) {
    float mean = (float)__ddiv_rn(*sum, (double)land_cells);
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x) {
        float v = mean <= 0.0f ? 1.0f : __fdiv_rn(__fsub_rn(1.0f, __fmul_rn(0.5f, veg[i])), mean);
        e[i] = rock ? __fmul_rn(v, rock[i]) : v;
    }
}

__global__ void k_fill_value(float* __restrict__ a, size_t N, float v) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x) a[i] = v;
}

__global__ void k_times_rock(float* __restrict__ e, const float* __restrict__ rock, size_t N) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x)
        e[i] = __fmul_rn(e[i], rock[i]);
}

bool pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

cg_status check_grid(cg_ctx* ctx, int W, int H) {
    if (!pow2(W) || !pow2(H)) return fail(ctx, CG_BAD_ARG, "width/height must be powers of two (got %d x %d)", W, H);
    if ((int64_t)W * H > ((int64_t)1 << 30)) return fail(ctx, CG_BAD_ARG, "grid of %d x %d cells is too large", W, H);
    return CG_OK;
}

cg_status up(cg_ctx* ctx, void* d, const void* h, size_t bytes) {
    CG_CUDA(ctx, cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, ctx->stream));
    return CG_OK;
}
cg_status down(cg_ctx* ctx, void* h, const void* d, size_t bytes) {
    CG_CUDA(ctx, cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    return CG_OK;
}

#define CG_TRY(x)                       \
    do {                                \
        cg_status s_ = (x);             \
        if (s_ != CG_OK) return s_;     \
    } while (0)

cg_status cancelled(cg_ctx* ctx) {
    if (ctx->cancel.exchange(0)) return fail(ctx, CG_CANCELLED, "cancelled");
    return CG_OK;
}

}  // namespace

cg_status runoff_weights_dev(cg_ctx* ctx, int W, int H, const float* d_rain, const uint8_t* d_land, int land_cells,
                             float* d_runoff) {
    const size_t N = (size_t)W * H;
    const int grid = ctx->num_sms * 8;
    if (d_rain) {
        CG_BUF(double, d_sum, ctx, S_CG3, 2);
        CG_TRY(seq_sum_dev(ctx, d_rain, d_land, 0, N, 0.0, d_sum, nullptr));
        CG_LAUNCH(ctx) k_normalise<<<grid, 256, 0, ctx->stream>>>(d_rain, d_sum, land_cells, N, d_runoff);
    } else {
        CG_LAUNCH(ctx) k_fill_value<<<grid, 256, 0, ctx->stream>>>(d_runoff, N, 1.0f);
    }
    CG_CHECK_LAUNCH(ctx);
    return CG_OK;
}

// ErosionStage.apply's opening (ErosionStage.kt:163-172): the initial thermal sweeps over the
// resident world. Marks the run done when no hydraulic round will run.
cg_status stage_begin_dev(cg_ctx* ctx, StageRun& run) {
    const cg_erosion_params& p = run.p;
    run.next_round = 0;
    run.land_cells = -1;
    run.done = false;
    if (!p.enabled) {
        run.done = true;
        return CG_OK;
    }
    CG_TRY(thermal_error_reset_dev(ctx));
    if (p.profile >= CG_PROFILE_P2) CG_TRY(deposit_stage_reset_dev(ctx, p.width, p.height));
    const int sweeps = sweeps_for(p);
    if (sweeps > 0) {
        float* res;
        CG_TRY(thermal_sweeps_dev(ctx, p.width, p.height, run.cur, run.other, thermal_limits(p), sweeps, p.rate, &res));
        if (res != run.cur) std::swap(run.cur, run.other);
    }
    // HydraulicErosion.kt:707-725: the plate flexure's field before the rounds (P3).
    if (p.profile >= CG_PROFILE_P3) CG_TRY(flexure_stage_begin_dev(ctx, p, run.cur, run.uplift != nullptr));
    if (p.hydraulic_rounds <= 0 || p.bedrock_erodibility_per_year <= 0.0f) run.done = true;
    return CG_OK;
}

// HydraulicErosion.apply's rounds [run.next_round, end_round) on the resident world, each relaxed by
// sweepsFor/rounds sweeps. `stats` (may be NULL) receives one entry per round run, the first for
// round run.next_round.
cg_status stage_rounds_dev(cg_ctx* ctx, StageRun& run, int end_round, cg_round_stats* stats) {
    const cg_erosion_params& p = run.p;
    const int W = p.width, H = p.height;
    const size_t N = (size_t)W * H;
    cudaStream_t sm = ctx->stream;
    const int grid = ctx->num_sms * 8;
    const int first_round = run.next_round;
    if (run.done || end_round <= first_round) return CG_OK;
    const float* d_uplift = run.uplift;
    const float* d_rock = run.rock;
    const float* d_rain = run.rain;
    const float* d_veg = run.veg;
    const cg_thermal_limits lim = thermal_limits(p);
    const int sweeps = sweeps_for(p);
    int per_round = sweeps / (p.hydraulic_rounds < 1 ? 1 : p.hydraulic_rounds);
    if (per_round < 1) per_round = 1;

    const ScaleF sc = scale_of(p);
    const RatesF rates = rates_of(p);
    const int lattice = smooth_field_lattice_columns(p.world_width_km);
    const float land_half = std::fmax(sc.land_half(), 1e-6f);
    const float sea_half = std::fmax(sc.sea_half(), 1e-6f);
    const float per_mm = (float)(sc.years_per_round / 1000.0);
    BreachRates brates;
    brates.relative_incision_coefficient = rates.relative_incision_coefficient;
    brates.notch_fall_per_cell = rates.notch_fall_per_cell;
    brates.outlet_reach_cells = rates.outlet_reach_cells;
    brates.pond_depth = rates.pond_depth;
    brates.step_ns = rates.step_ns;
    brates.step_diag = rates.step_diag;
    CG_BUF(uint8_t, d_land, ctx, S_LAND, N);
    CG_BUF(float, d_rel, ctx, S_REL, N);
    CG_BUF(float, d_filled, ctx, S_FILLED, N);
    CG_BUF(double, d_surface, ctx, S_SURFACE, N);
    CG_BUF(int32_t, d_recv, ctx, S_RECV, N);
    CG_BUF(int32_t, d_donors, ctx, S_DONORS, N);
    CG_BUF(long long, d_key, ctx, S_KEY, N);
    CG_BUF(float, d_area, ctx, S_AREA, N);
    CG_BUF(float, d_runoff, ctx, S_RUNOFF, N);
    CG_BUF(float, d_erod, ctx, S_ERODE, N);
    CG_BUF(double, d_sum, ctx, S_CG3, 2);

    const bool flexure = p.profile >= CG_PROFILE_P3;
    float* d_uplifted = flexure && d_uplift ? flexure_uplifted_dev(ctx, p) : nullptr;
    float* d_sediment_now = nullptr;
    if (flexure) {
        CG_BUF(float, sed, ctx, S_SEDIMENT, N);
        d_sediment_now = sed;
    }

    // Phase boundaries of a round, for the per-phase device times of cg_round_stats (ev[8]: the end
    // of the uplift and the plate flexure).
    cudaEvent_t ev[9] = {};
    if (stats)
        for (auto& e : ev) CG_CUDA(ctx, cudaEventCreate(&e));
    struct Events {
        cudaEvent_t* ev;
        bool on;
        ~Events() {
            if (on)
                for (int i = 0; i < 9; ++i) cudaEventDestroy(ev[i]);
        }
    } guard{ev, stats != nullptr};
    auto mark = [&](int i) {
        if (stats) cudaEventRecord(ev[i], sm);
    };

    for (int round = first_round; round < end_round; ++round) {
        CG_TRY(cancelled(ctx));
        float* cur = run.cur;
        const long long launches0 = ctx->launches;
        mark(0);
        if (d_uplift)
            CG_LAUNCH(ctx) k_uplift<<<grid, 256, 0, sm>>>(cur, d_uplift, N, per_mm, sc.relief_span(), d_uplifted);
        // HydraulicErosion.kt:856-884: the plate answers the whole load so far (P3).
        if (flexure) CG_TRY(flexure_round_dev(ctx, p, cur, d_sediment_now, d_uplift != nullptr));
        mark(8);
        float shoreline;
        int land_cells;
        CG_TRY(percentile_cut_dev(ctx, W, H, cur, p.sea_level, land_half, sea_half, stand_below_today(p, round),
                                  d_land, d_rel, &shoreline, &land_cells));
        if (land_cells == 0) {   // HydraulicErosion.kt:856-858: the rounds stop where the land is gone
            run.done = true;
            run.next_round = round;
            run.land_cells = 0;
            return CG_OK;
        }
        run.land_cells = land_cells;
        // normaliseOverLand / shieldingOverLand (HydraulicErosion.kt:902-911).
        if (!d_rain && (!d_veg || !p.shield_cut)) {
            CG_LAUNCH(ctx) k_unit_weights<<<grid, 256, 0, sm>>>(d_rock, N, d_runoff, d_erod);
        } else {
            if (d_rain) {
                CG_TRY(seq_sum_dev(ctx, d_rain, d_land, 0, N, 0.0, d_sum, nullptr));
                CG_LAUNCH(ctx) k_normalise<<<grid, 256, 0, sm>>>(d_rain, d_sum, land_cells, N, d_runoff);
            } else {
                CG_LAUNCH(ctx) k_fill_value<<<grid, 256, 0, sm>>>(d_runoff, N, 1.0f);
            }
            if (p.shield_cut && d_veg) {
                CG_TRY(seq_sum_dev(ctx, d_veg, d_land, 1, N, 0.0, d_sum + 1, nullptr));
                CG_LAUNCH(ctx) k_shield<<<grid, 256, 0, sm>>>(d_veg, d_sum + 1, land_cells, d_rock, N, d_erod);
            } else {
                CG_LAUNCH(ctx) k_fill_value<<<grid, 256, 0, sm>>>(d_erod, N, 1.0f);
                if (d_rock) CG_LAUNCH(ctx) k_times_rock<<<grid, 256, 0, sm>>>(d_erod, d_rock, N);
            }
        }
        CG_CHECK_LAUNCH(ctx);
        mark(1);
        int64_t ties = 0, unresolved = 0;
        CG_TRY(fill_depressions_dev(ctx, W, H, d_land, d_rel, d_filled, &ties, &unresolved));
        mark(2);
        FlatCounts fc{0, 0, 0};
        CG_TRY(flow_directions_dev(ctx, W, H, d_land, d_rel, d_filled, p.seed, rates.cell_height_in_cell_widths,
                                   lattice, p.facet_routing != 0, p.flat_potential != 0, d_recv, d_surface, &fc));
        mark(3);
        int levels = 0;
        CG_TRY(tree_walk_dev(ctx, W, H, d_land, d_recv, d_runoff, d_key, d_donors, d_area, &levels));
        mark(4);
        const bool notch = p.profile >= CG_PROFILE_P1, deposition = p.profile >= CG_PROFILE_P2;
        const bool closing = round == p.hydraulic_rounds - 1;
        const float to_relative = 1.0f / land_half;
        float* d_settled = nullptr;
        double* d_load = nullptr;
        double* d_incised_at = nullptr;
        if (deposition)
            CG_TRY(deposit_round_begin_dev(ctx, W, H, d_rel, to_relative, &d_settled, &d_load, &d_incised_at));
        if (notch)
            CG_TRY(breach_dev(ctx, W, H, d_land, d_rel, d_filled, d_recv, d_area, (float)land_cells, land_half, brates,
                              cur, nullptr, d_settled, d_load));
        InciseArgs ia;
        ia.courant_coefficient = rates.courant_coefficient;
        ia.pond_depth = rates.pond_depth;
        ia.land_cells = (float)land_cells;
        ia.land_range = land_half;
        ia.shoreline = shoreline;
        ia.step_ns = rates.step_ns;
        ia.step_diag = rates.step_diag;
        ia.only_above_base = p.receiver_clamp != 0;
        CG_TRY(incise_dev(ctx, W, H, d_land, d_recv, d_key, levels, d_filled, d_rel, d_area, d_erod, cur, ia,
                          d_incised_at));
        mark(5);
        DepositCounts dc{};
        if (deposition) {
            DepositRound dr;
            dr.recv = d_recv;
            dr.land = d_land;
            dr.ground = d_filled;
            dr.rel = d_rel;
            dr.area = d_area;
            dr.key = d_key;
            dr.levels = levels;
            dr.land_cells = land_cells;
            dr.land_range = land_half;
            dr.to_relative = to_relative;
            dr.shoreline = shoreline;
            dr.surface = cur;
            dr.settled = d_settled;
            dr.load = d_load;
            dr.incised_at = d_incised_at;
            CG_TRY(deposit_walk_dev(ctx, p, dr, &dc));
        }
        if (closing && deposition) CG_TRY(deposit_settle_dev(ctx, W, H, cur));
        if (notch && closing) {
            // The closing breach (HydraulicErosion.kt:1404-1442): a fresh cut at today's shoreline over
            // the finished surface, its own fill, routing and discharge, then one more notch. Its
            // routing is what the stage reports.
            float closing_shoreline;
            int closing_land;
            CG_TRY(percentile_cut_dev(ctx, W, H, cur, p.sea_level, land_half, sea_half, 0.0f, d_land, d_rel,
                                      &closing_shoreline, &closing_land));
            run.land_cells = closing_land;
            if (closing_land > 0) {
                if (d_rain) {
                    CG_TRY(seq_sum_dev(ctx, d_rain, d_land, 0, N, 0.0, d_sum, nullptr));
                    CG_LAUNCH(ctx) k_normalise<<<grid, 256, 0, sm>>>(d_rain, d_sum, closing_land, N, d_runoff);
                } else {
                    CG_LAUNCH(ctx) k_fill_value<<<grid, 256, 0, sm>>>(d_runoff, N, 1.0f);
                }
                CG_CHECK_LAUNCH(ctx);
                CG_TRY(fill_depressions_dev(ctx, W, H, d_land, d_rel, d_filled, nullptr, nullptr));
                FlatCounts closing_flats{0, 0, 0};
                CG_TRY(flow_directions_dev(ctx, W, H, d_land, d_rel, d_filled, p.seed, rates.cell_height_in_cell_widths,
                                           lattice, p.facet_routing != 0, p.flat_potential != 0, d_recv, d_surface,
                                           &closing_flats));
                CG_TRY(tree_walk_dev(ctx, W, H, d_land, d_recv, d_runoff, d_key, d_donors, d_area, nullptr));
                CG_TRY(breach_dev(ctx, W, H, d_land, d_rel, d_filled, d_recv, d_area, (float)closing_land, land_half,
                                  brates, cur, nullptr));
            }
        }
        // The closing mouths pass (HydraulicErosion.kt:1451-1462), ErosionConfig.deltaLobe.
        if (closing && deposition) CG_TRY(open_mouths_dev(ctx, p, cur, d_rain));
        mark(6);
        // relax = thermalErosion(config, field, accelerator, sweepsPerRound) (ErosionStage.kt:178-180).
        float* res;
        CG_TRY(thermal_sweeps_dev(ctx, W, H, run.cur, run.other, lim, per_round, p.rate, &res));
        if (res != run.cur) std::swap(run.cur, run.other);
        run.next_round = round + 1;
        mark(7);
        if (stats) {
            CG_CUDA(ctx, cudaEventSynchronize(ev[7]));
            float ms[8] = {0};
            for (int i = 1; i < 8; ++i) cudaEventElapsedTime(&ms[i], ev[i - 1], ev[i]);
            float ms_flexure = 0.0f;
            if (flexure) {
                cudaEventElapsedTime(&ms_flexure, ev[0], ev[8]);
                cudaEventElapsedTime(&ms[1], ev[8], ev[1]);
            }
            float total = 0.0f;
            cudaEventElapsedTime(&total, ev[0], ev[7]);
            cg_round_stats& s = stats[round - first_round];
            std::memset(&s, 0, sizeof(s));
            s.round = round;
            s.land_cells = land_cells;
            s.shoreline = shoreline;
            s.flats = fc.flats;
            s.flats_kept = fc.kept;
            s.raised_cells = fc.raised;
            s.levels = levels;
            s.fill_ties = ties;
            s.fill_unresolved = unresolved;
            s.kernel_launches = ctx->launches - launches0;
            s.ms_total = total;
            s.ms_cut = ms[1];
            s.ms_fill = ms[2];
            s.ms_route = ms[3];
            s.ms_tree = ms[4];
            s.ms_incise = ms[5];
            s.ms_deposit = ms[6];
            s.ms_relax = ms[7];
            s.ms_flexure = ms_flexure;
            s.deposit_replayed = dc.replayed;
            s.deposit_redone = dc.redone;
            s.deposit_refitted = dc.refitted;
            s.deposit_waves = dc.waves;
            s.ms_deposit_walks = dc.ms_walks;
            s.ms_deposit_schedule = dc.ms_schedule;
            s.ms_deposit_lakes = dc.ms_lakes;
            s.ms_deposit_seas = dc.ms_seas;
            s.ms_deposit_repairs = dc.ms_repairs;
        }
    }
    if (run.next_round >= p.hydraulic_rounds) run.done = true;
    return CG_OK;
}

// The whole stage with the world resident on the device. `d_h` holds the input heights and
// receives the result (through *d_result, which is d_h or the ping-pong partner).
cg_status erode_stage_dev(cg_ctx* ctx, const cg_erosion_params& p, float* d_h, float* d_h2, const float* d_uplift,
                          const float* d_rock, const float* d_rain, const float* d_veg, float** d_result,
                          cg_round_stats* stats, int* last_land_cells) {
    StageRun run;
    run.p = p;
    run.cur = d_h;
    run.other = d_h2;
    run.uplift = d_uplift;
    run.rock = d_rock;
    run.rain = d_rain;
    run.veg = d_veg;
    *d_result = d_h;
    *last_land_cells = -1;
    cg_status st = stage_begin_dev(ctx, run);
    if (st == CG_OK) st = stage_rounds_dev(ctx, run, p.hydraulic_rounds, stats);
    if (st == CG_OK) st = thermal_error_check(ctx);
    *d_result = run.cur;
    *last_land_cells = run.land_cells;
    return st;
}

}  // namespace cg

using namespace cg;

namespace {

// The stage's outputs (cg_outputs) from the device: the result field and, when the last round
// routed, that round's routing fields, drainage order and basins.
cg_status download_outputs(cg_ctx* ctx, const cg_erosion_params& pp, const float* d_res, int land_cells,
                           cg_outputs* out) {
    const cg_erosion_params* p = &pp;
    const int W = p->width, H = p->height;
    const size_t N = (size_t)W * H;
    CG_TRY(down(ctx, out->height, d_res, N * 4));
    const bool routed = land_cells > 0 && p->enabled && p->hydraulic_rounds > 0 && p->bedrock_erodibility_per_year > 0.0f;
    if (routed) {
        if (out->receivers) CG_TRY(down(ctx, out->receivers, ctx->bufs[S_RECV].ptr, N * 4));
        if (out->area) CG_TRY(down(ctx, out->area, ctx->bufs[S_AREA].ptr, N * 4));
        if (out->filled) CG_TRY(down(ctx, out->filled, ctx->bufs[S_FILLED].ptr, N * 4));
        if (out->relative) CG_TRY(down(ctx, out->relative, ctx->bufs[S_REL].ptr, N * 4));
        if (out->is_land) CG_TRY(down(ctx, out->is_land, ctx->bufs[S_LAND].ptr, N));
        if (out->donors) CG_TRY(down(ctx, out->donors, ctx->bufs[S_DONORS].ptr, N * 4));
        if (out->order) {
            CG_BUF(int32_t, d_order, ctx, S_ORDER, N);
            CG_CUDA(ctx, cudaMemsetAsync(d_order, 0xFF, N * 4, ctx->stream));
            CG_TRY(order_from_keys_dev(ctx, W, H, (const uint8_t*)ctx->bufs[S_LAND].ptr,
                                       (const long long*)ctx->bufs[S_KEY].ptr, land_cells, d_order));
            CG_TRY(down(ctx, out->order, d_order, N * 4));
        }
        if (out->basin_of_cell || out->basins) {
            const RatesF rates = rates_of(*p);
            CG_BUF(int32_t, d_lab, ctx, S_BASIN2, N);
            CG_TRY(spillways_dev(ctx, W, H, (const uint8_t*)ctx->bufs[S_LAND].ptr, (const float*)ctx->bufs[S_REL].ptr,
                                 (const float*)ctx->bufs[S_FILLED].ptr, (const int32_t*)ctx->bufs[S_RECV].ptr,
                                 rates.pond_depth, d_lab, out->basins));
            if (out->basin_of_cell) CG_TRY(down(ctx, out->basin_of_cell, d_lab, N * 4));
        }
    }
    return CG_OK;
}

// The parameters' checks shared by the stage's entry points. `fed_ok`: the caller can hand in the
// weather between rounds (the round-range entry points), so climate_feed is accepted.
cg_status check_params(cg_ctx* ctx, const cg_erosion_params* p, bool fed_ok) {
    if (p->abi_version != CG_ABI_VERSION)
        return fail(ctx, CG_BAD_ARG, "params carry ABI version %u, this library is %u", p->abi_version,
                    CG_ABI_VERSION);
    CG_TRY(check_grid(ctx, p->width, p->height));
    if (p->mode != CG_MODE_REF32) return fail(ctx, CG_UNSUPPORTED, "only the REF32 mode is built");
    if (p->profile < CG_PROFILE_P0 || p->profile > CG_PROFILE_P3)
        return fail(ctx, CG_UNSUPPORTED, "profile P%d is not built (P0 to P3)", p->profile);
    if (p->profile >= CG_PROFILE_P3) CG_TRY(flexure_check(ctx, p->width, p->height));
    if (p->climate_feed && !fed_ok)
        return fail(ctx, CG_UNSUPPORTED,
                    "climate_feed asks for the caller's weather halfway through the rounds: run the stage with "
                    "cg_stage_begin / cg_erode_rounds");
    return CG_OK;
}

// Copies one optional host field into its slot; *d stays NULL when the field is not given.
cg_status upload_optional(cg_ctx* ctx, int slot, const float* host, size_t N, float** d) {
    *d = nullptr;
    if (!host) return CG_OK;
    cg_status st = CG_OK;
    *d = (float*)buf(ctx, slot, N * 4, &st);
    if (st != CG_OK) return st;
    return up(ctx, *d, host, N * 4);
}

// Uploads a world's inputs into the context's slots (heights into S_H0, S_H1 reserved for the
// ping-pong partner) and fills the run's device pointers.
cg_status upload_world(cg_ctx* ctx, const cg_erosion_params* p, const cg_inputs* in, StageRun& run) {
    const size_t N = (size_t)p->width * p->height;
    CG_BUF(float, d_h, ctx, S_H0, N);
    CG_BUF(float, d_h2, ctx, S_H1, N);
    CG_TRY(up(ctx, d_h, in->height, N * 4));
    float *d_up, *d_rock, *d_rain, *d_veg;
    CG_TRY(upload_optional(ctx, S_UPLIFT, in->uplift_mm_per_year, N, &d_up));
    CG_TRY(upload_optional(ctx, S_ROCK, in->rock_erodibility, N, &d_rock));
    CG_TRY(upload_optional(ctx, S_RAIN, in->rainfall_mm, N, &d_rain));
    CG_TRY(upload_optional(ctx, S_VEG, in->vegetation_density, N, &d_veg));
    run = StageRun();
    run.p = *p;
    run.cur = d_h;
    run.other = d_h2;
    run.uplift = d_up;
    run.rock = d_rock;
    run.rain = d_rain;
    run.veg = d_veg;
    return CG_OK;
}

// cg_erode_stage without clearing the cancel flag (a batch clears it once for all its worlds).
cg_status erode_stage_host(cg_ctx* ctx, const cg_erosion_params* p, const cg_inputs* in, cg_outputs* out,
                           cg_round_stats* stats) {
    if (!ctx || !p || !in || !out || !in->height || !out->height) return CG_BAD_ARG;
    ctx->run.active = false;   // this call reuses the resident world's buffers
    CG_TRY(check_params(ctx, p, false));
    CG_CUDA(ctx, cudaSetDevice(ctx->device));
    StageRun run;
    CG_TRY(upload_world(ctx, p, in, run));
    float* d_res = run.cur;
    int land_cells = -1;
    CG_TRY(erode_stage_dev(ctx, *p, run.cur, run.other, run.uplift, run.rock, run.rain, run.veg, &d_res, stats,
                           &land_cells));
    CG_TRY(download_outputs(ctx, *p, d_res, land_cells, out));
    return sync(ctx);
}

}  // namespace

extern "C" {

cg_status cg_erode_stage(cg_ctx* ctx, const cg_erosion_params* p, const cg_inputs* in, cg_outputs* out,
                         cg_round_stats* stats) {
    if (!ctx) return CG_BAD_ARG;
    ctx->run.active = false;   // this call reuses the resident world's buffers
    ctx->cancel.store(0);
    return erode_stage_host(ctx, p, in, out, stats);
}

cg_status cg_erode_batch(cg_ctx* ctx, int32_t n_worlds, const cg_world* worlds, cg_status* status) {
    if (!ctx || n_worlds < 0 || (n_worlds > 0 && !worlds)) return CG_BAD_ARG;
    ctx->run.active = false;   // this call reuses the resident world's buffers
    ctx->cancel.store(0);
    cg_status first = CG_OK;
    for (int32_t i = 0; i < n_worlds; ++i) {
        cg_status st = cancelled(ctx);
        if (st == CG_OK) {
            cg_outputs out = worlds[i].outputs;
            st = erode_stage_host(ctx, &worlds[i].params, &worlds[i].inputs, &out, nullptr);
        }
        if (status) status[i] = st;
        if (st != CG_OK && first == CG_OK) first = st;
        if (st == CG_CANCELLED) {
            for (int32_t j = i + 1; j < n_worlds; ++j)
                if (status) status[j] = CG_CANCELLED;
            break;
        }
    }
    return first;
}

cg_status cg_erode_stage_dev(cg_ctx* ctx, const cg_erosion_params* p, const cg_inputs* in, float* out_dev,
                             cg_round_stats* stats, int32_t* land_cells_out) {
    if (!ctx || !p || !in || !in->height || !out_dev) return CG_BAD_ARG;
    ctx->run.active = false;   // this call reuses the resident world's buffers
    CG_TRY(check_params(ctx, p, false));
    CG_CUDA(ctx, cudaSetDevice(ctx->device));
    ctx->cancel.store(0);
    const size_t N = (size_t)p->width * p->height;
    CG_BUF(float, d_h, ctx, S_H0, N);
    CG_BUF(float, d_h2, ctx, S_H1, N);
    CG_CUDA(ctx, cudaMemcpyAsync(d_h, in->height, N * 4, cudaMemcpyDeviceToDevice, ctx->stream));
    float* d_res = d_h;
    int land_cells = -1;
    CG_TRY(erode_stage_dev(ctx, *p, d_h, d_h2, in->uplift_mm_per_year, in->rock_erodibility, in->rainfall_mm,
                           in->vegetation_density, &d_res, stats, &land_cells));
    CG_CUDA(ctx, cudaMemcpyAsync(out_dev, d_res, N * 4, cudaMemcpyDeviceToDevice, ctx->stream));
    if (land_cells_out) *land_cells_out = land_cells;
    return sync(ctx);
}

cg_status cg_stage_begin(cg_ctx* ctx, const cg_erosion_params* p, const cg_inputs* in) {
    if (!ctx || !p || !in || !in->height) return CG_BAD_ARG;
    ctx->run.active = false;
    CG_TRY(check_params(ctx, p, true));
    CG_CUDA(ctx, cudaSetDevice(ctx->device));
    ctx->cancel.store(0);
    StageRun run;
    CG_TRY(upload_world(ctx, p, in, run));
    CG_TRY(stage_begin_dev(ctx, run));
    CG_TRY(thermal_error_check(ctx));
    run.active = true;
    ctx->run = run;
    return CG_OK;
}

cg_status cg_erode_rounds(cg_ctx* ctx, int32_t first_round, int32_t end_round, const cg_weather* weather,
                          cg_round_stats* stats) {
    if (!ctx) return CG_BAD_ARG;
    StageRun& run = ctx->run;
    if (!run.active) return fail(ctx, CG_BAD_ARG, "no resident world: call cg_stage_begin first");
    const cg_erosion_params& p = run.p;
    if (first_round != run.next_round && !(run.done && first_round >= run.next_round))
        return fail(ctx, CG_BAD_ARG, "rounds run in order: the next round is %d, not %d", run.next_round, first_round);
    if (end_round < first_round || end_round > (p.hydraulic_rounds > 0 ? p.hydraulic_rounds : 0))
        return fail(ctx, CG_BAD_ARG, "round range [%d, %d) is outside the stage's %d rounds", first_round, end_round,
                    p.hydraulic_rounds);
    const int refresh_at = p.climate_feed && p.hydraulic_rounds > 1 ? p.hydraulic_rounds / 2 : -1;
    if (refresh_at > first_round && refresh_at < end_round)
        return fail(ctx, CG_BAD_ARG, "climate_feed: round %d takes the refreshed weather, so a call may not run across it",
                    refresh_at);
    if (p.climate_feed && (first_round == 0 || first_round == refresh_at) && !weather && end_round > first_round)
        return fail(ctx, CG_BAD_ARG, "climate_feed: round %d needs the caller's weather", first_round);
    CG_CUDA(ctx, cudaSetDevice(ctx->device));
    ctx->cancel.store(0);
    const size_t N = (size_t)p.width * p.height;
    if (weather) {   // replaces the rounds' weather from first_round on; a NULL field is the default
        float *d_rain, *d_veg;
        CG_TRY(upload_optional(ctx, S_RAIN, weather->rainfall_mm, N, &d_rain));
        CG_TRY(upload_optional(ctx, S_VEG, weather->vegetation_density, N, &d_veg));
        run.rain = d_rain;
        run.veg = d_veg;
    }
    cg_status st = stage_rounds_dev(ctx, run, end_round, stats);
    if (st == CG_OK) st = thermal_error_check(ctx);
    if (st != CG_OK) {
        run.active = false;   // a round stopped part way: the world is no longer a whole terrain
        return st;
    }
    return sync(ctx);
}

cg_status cg_stage_replay_belts(cg_ctx* ctx, const cg_belt_window* window, const cg_weather* weather,
                                int32_t rebound, double history_cell_km, float* eroded_meters,
                                cg_belt_books* books) {
    if (!ctx || !window || !books || !window->tectonic_km || !window->wear_km || !window->onset_myr_ago)
        return CG_BAD_ARG;
    StageRun& run = ctx->run;
    if (!run.active) return fail(ctx, CG_BAD_ARG, "no resident world: call cg_stage_begin first");
    if (run.next_round != 0) return fail(ctx, CG_BAD_ARG, "the belts replay before round 0, not after round %d",
                                         run.next_round);
    const cg_erosion_params& p = run.p;
    const size_t N = (size_t)p.width * p.height;
    *books = cg_belt_books{};
    CG_CUDA(ctx, cudaSetDevice(ctx->device));
    ctx->cancel.store(0);
    // HydraulicErosion.apply returns before the replay when the stage erodes nothing
    // (HydraulicErosion.kt:632): run.done is set then, and the terrain is left as the sweeps left it.
    if (run.done) {
        if (eroded_meters) std::memset(eroded_meters, 0, N * 4);
        return CG_OK;
    }
    BeltInputsDev in{};
    CG_TRY(belt_window_dev(ctx, p, *window, &in));
    in.uplift = run.uplift;
    in.rock = run.rock;
    const float* d_rain = run.rain;
    const float* d_veg = run.veg;
    if (weather) {   // the opening weather, when the caller solves it (climate_feed); NULL fields are the defaults
        float *r = nullptr, *v = nullptr;
        CG_TRY(upload_optional(ctx, S_BT_RAIN, weather->rainfall_mm, N, &r));
        CG_TRY(upload_optional(ctx, S_BT_COVER, weather->vegetation_density, N, &v));
        d_rain = r;
        d_veg = v;
    }
    CG_TRY(belt_weather_dev(ctx, p.width, p.height, d_rain, d_veg, &in));
    cg_belt_inputs opt{};
    opt.provisional_sea_level = p.sea_level;   // ErosionStage.apply hands config.seaLevel (ErosionStage.kt:174)
    opt.shield_cut = p.shield_cut;
    opt.rebound = rebound;
    opt.history_cell_km = history_cell_km;
    CG_BUF(float, d_eroded, ctx, S_BT_ERODED, N);
    cg_status st = belt_replay_dev(ctx, p, run.cur, in, window->window_myr, opt, d_eroded, books);
    if (st != CG_OK) {
        run.active = false;   // the replay stopped part way: the world is no longer a whole terrain
        return st;
    }
    // HydraulicErosion.kt:707-725: the flexure's field before the rounds is the replayed one (P3).
    if (p.profile >= CG_PROFILE_P3) CG_TRY(flexure_stage_begin_dev(ctx, p, run.cur, run.uplift != nullptr));
    if (eroded_meters) CG_TRY(down(ctx, eroded_meters, d_eroded, N * 4));
    return sync(ctx);
}

cg_status cg_stage_height(cg_ctx* ctx, float* height) {
    if (!ctx || !height) return CG_BAD_ARG;
    if (!ctx->run.active) return fail(ctx, CG_BAD_ARG, "no resident world: call cg_stage_begin first");
    CG_CUDA(ctx, cudaSetDevice(ctx->device));
    CG_TRY(down(ctx, height, ctx->run.cur, (size_t)ctx->run.p.width * ctx->run.p.height * 4));
    return sync(ctx);
}

cg_status cg_stage_finish(cg_ctx* ctx, cg_outputs* out) {
    if (!ctx || !out || !out->height) return CG_BAD_ARG;
    StageRun& run = ctx->run;
    if (!run.active) return fail(ctx, CG_BAD_ARG, "no resident world: call cg_stage_begin first");
    if (!run.done) return fail(ctx, CG_BAD_ARG, "round %d of %d is still to run", run.next_round, run.p.hydraulic_rounds);
    CG_CUDA(ctx, cudaSetDevice(ctx->device));
    run.active = false;
    CG_TRY(download_outputs(ctx, run.p, run.cur, run.land_cells, out));
    return sync(ctx);
}

cg_status cg_percentile_cut(cg_ctx* ctx, int32_t W, int32_t H, const float* heights, float sea_level,
                            float highest_land, float deepest_ocean, float lowstand_share, float* shoreline,
                            uint8_t* is_land, float* relative, int32_t* land_cells) {
    if (!ctx || !heights || !shoreline || !is_land || !relative || !land_cells) return CG_BAD_ARG;
    ctx->run.active = false;   // this call reuses the resident world's buffers
    CG_TRY(check_grid(ctx, W, H));
    CG_CUDA(ctx, cudaSetDevice(ctx->device));
    size_t N = (size_t)W * H;
    CG_BUF(float, d_h, ctx, S_H0, N);
    CG_BUF(uint8_t, d_land, ctx, S_LAND, N);
    CG_BUF(float, d_rel, ctx, S_REL, N);
    CG_TRY(up(ctx, d_h, heights, N * 4));
    ScaleF sc{40075.0, highest_land, deepest_ocean, 0.0};
    float s;
    int n;
    CG_TRY(percentile_cut_dev(ctx, W, H, d_h, sea_level, std::fmax(sc.land_half(), 1e-6f),
                              std::fmax(sc.sea_half(), 1e-6f), lowstand_share, d_land, d_rel, &s, &n));
    CG_TRY(down(ctx, is_land, d_land, N));
    CG_TRY(down(ctx, relative, d_rel, N * 4));
    CG_TRY(sync(ctx));
    *shoreline = s;
    *land_cells = n;
    return CG_OK;
}

cg_status cg_fill_depressions(cg_ctx* ctx, int32_t W, int32_t H, const uint8_t* is_land, const float* relative,
                              float* filled, int64_t* ties, int64_t* unresolved) {
    if (!ctx || !is_land || !relative || !filled) return CG_BAD_ARG;
    ctx->run.active = false;   // this call reuses the resident world's buffers
    CG_TRY(check_grid(ctx, W, H));
    CG_CUDA(ctx, cudaSetDevice(ctx->device));
    size_t N = (size_t)W * H;
    CG_BUF(uint8_t, d_land, ctx, S_LAND, N);
    CG_BUF(float, d_rel, ctx, S_REL, N);
    CG_BUF(float, d_filled, ctx, S_FILLED, N);
    CG_TRY(up(ctx, d_land, is_land, N));
    CG_TRY(up(ctx, d_rel, relative, N * 4));
    CG_TRY(fill_depressions_dev(ctx, W, H, d_land, d_rel, d_filled, ties, unresolved));
    CG_TRY(down(ctx, filled, d_filled, N * 4));
    return sync(ctx);
}

cg_status cg_flow_directions(cg_ctx* ctx, int32_t W, int32_t H, const uint8_t* is_land, const float* relative,
                             const float* filled, int64_t seed, double r, int32_t lattice, int32_t by_facet,
                             int32_t over_potential, int32_t* receivers, double* surface, int32_t* flat_counts) {
    if (!ctx || !is_land || !relative || !filled || !receivers) return CG_BAD_ARG;
    ctx->run.active = false;   // this call reuses the resident world's buffers
    CG_TRY(check_grid(ctx, W, H));
    if (!(r > 0.0) || lattice < 1) return fail(ctx, CG_BAD_ARG, "bad cell aspect %g or lattice %d", r, lattice);
    CG_CUDA(ctx, cudaSetDevice(ctx->device));
    size_t N = (size_t)W * H;
    CG_BUF(uint8_t, d_land, ctx, S_LAND, N);
    CG_BUF(float, d_rel, ctx, S_REL, N);
    CG_BUF(float, d_filled, ctx, S_FILLED, N);
    CG_BUF(double, d_surface, ctx, S_SURFACE, N);
    CG_BUF(int32_t, d_recv, ctx, S_RECV, N);
    CG_TRY(up(ctx, d_land, is_land, N));
    CG_TRY(up(ctx, d_rel, relative, N * 4));
    CG_TRY(up(ctx, d_filled, filled, N * 4));
    FlatCounts fc{0, 0, 0};
    CG_TRY(flow_directions_dev(ctx, W, H, d_land, d_rel, d_filled, seed, r, lattice, by_facet != 0,
                               over_potential != 0, d_recv, d_surface, &fc));
    CG_TRY(down(ctx, receivers, d_recv, N * 4));
    if (surface) CG_TRY(down(ctx, surface, d_surface, N * 8));
    CG_TRY(sync(ctx));
    if (flat_counts) {
        flat_counts[0] = fc.flats;
        flat_counts[1] = fc.kept;
        flat_counts[2] = fc.raised;
    }
    return CG_OK;
}

cg_status cg_drainage_order(cg_ctx* ctx, int32_t W, int32_t H, const uint8_t* is_land, const int32_t* receivers,
                            int32_t land_cells, int32_t* order) {
    if (!ctx || !is_land || !receivers || !order || land_cells < 0) return CG_BAD_ARG;
    ctx->run.active = false;   // this call reuses the resident world's buffers
    CG_TRY(check_grid(ctx, W, H));
    CG_CUDA(ctx, cudaSetDevice(ctx->device));
    size_t N = (size_t)W * H;
    CG_BUF(uint8_t, d_land, ctx, S_LAND, N);
    CG_BUF(int32_t, d_recv, ctx, S_RECV, N);
    CG_BUF(int32_t, d_donors, ctx, S_DONORS, N);
    CG_BUF(long long, d_key, ctx, S_KEY, N);
    CG_BUF(int32_t, d_order, ctx, S_ORDER, N);
    CG_TRY(up(ctx, d_land, is_land, N));
    CG_TRY(up(ctx, d_recv, receivers, N * 4));
    CG_TRY(tree_walk_dev(ctx, W, H, d_land, d_recv, nullptr, d_key, d_donors, nullptr, nullptr));
    CG_TRY(order_from_keys_dev(ctx, W, H, d_land, d_key, land_cells, d_order));
    if (land_cells > 0) CG_TRY(down(ctx, order, d_order, (size_t)land_cells * 4));
    return sync(ctx);
}

cg_status cg_accumulate(cg_ctx* ctx, int32_t W, int32_t H, const uint8_t* is_land, const int32_t* receivers,
                        int32_t land_cells, const float* weights, float* area) {
    if (!ctx || !is_land || !receivers || !weights || !area) return CG_BAD_ARG;
    ctx->run.active = false;   // this call reuses the resident world's buffers
    CG_TRY(check_grid(ctx, W, H));
    CG_CUDA(ctx, cudaSetDevice(ctx->device));
    size_t N = (size_t)W * H;
    CG_BUF(uint8_t, d_land, ctx, S_LAND, N);
    CG_BUF(int32_t, d_recv, ctx, S_RECV, N);
    CG_BUF(int32_t, d_donors, ctx, S_DONORS, N);
    CG_BUF(long long, d_key, ctx, S_KEY, N);
    CG_BUF(float, d_w, ctx, S_RUNOFF, N);
    CG_BUF(float, d_area, ctx, S_AREA, N);
    CG_TRY(up(ctx, d_land, is_land, N));
    CG_TRY(up(ctx, d_recv, receivers, N * 4));
    CG_TRY(up(ctx, d_w, weights, N * 4));
    CG_TRY(tree_walk_dev(ctx, W, H, d_land, d_recv, d_w, d_key, d_donors, d_area, nullptr));
    CG_TRY(down(ctx, area, d_area, N * 4));
    (void)land_cells;
    return sync(ctx);
}

cg_status cg_route_cut(cg_ctx* ctx, const cg_erosion_params* p, const uint8_t* is_land, const float* relative,
                       int32_t land_cells, const float* weights, float* filled, int32_t* receivers, float* area,
                       int32_t* order) {
    if (!ctx || !p || !is_land || !relative || !receivers || land_cells < 0) return CG_BAD_ARG;
    ctx->run.active = false;   // this call reuses the resident world's buffers
    if (p->abi_version != CG_ABI_VERSION)
        return fail(ctx, CG_BAD_ARG, "params carry ABI version %u, this library is %u", p->abi_version,
                    CG_ABI_VERSION);
    const int W = p->width, H = p->height;
    CG_TRY(check_grid(ctx, W, H));
    CG_CUDA(ctx, cudaSetDevice(ctx->device));
    const size_t N = (size_t)W * H;
    const int grid = ctx->num_sms * 8;
    CG_BUF(uint8_t, d_land, ctx, S_LAND, N);
    CG_BUF(float, d_rel, ctx, S_REL, N);
    CG_BUF(float, d_filled, ctx, S_FILLED, N);
    CG_BUF(double, d_surface, ctx, S_SURFACE, N);
    CG_BUF(int32_t, d_recv, ctx, S_RECV, N);
    CG_TRY(up(ctx, d_land, is_land, N));
    CG_TRY(up(ctx, d_rel, relative, N * 4));
    // FlowRouting.fillDepressions, then flowDirections over it (FlowRouting.kt:52-111, 179-216).
    CG_TRY(fill_depressions_dev(ctx, W, H, d_land, d_rel, d_filled, nullptr, nullptr));
    const ScaleF sc = scale_of(*p);
    FlatCounts fc{0, 0, 0};
    CG_TRY(flow_directions_dev(ctx, W, H, d_land, d_rel, d_filled, p->seed, sc.cell_height_km(H) / sc.cell_width_km(W),
                               smooth_field_lattice_columns(p->world_width_km), p->facet_routing != 0,
                               p->flat_potential != 0, d_recv, d_surface, &fc));
    // accumulate (weights, or { 1f }) and drainageOrder over those receivers (FlowRouting.kt:485-511, 695-729).
    if (area || order) {
        CG_BUF(int32_t, d_donors, ctx, S_DONORS, N);
        CG_BUF(long long, d_key, ctx, S_KEY, N);
        float *d_w = nullptr, *d_area = nullptr;
        if (area) {
            CG_BUF(float, w, ctx, S_RUNOFF, N);
            CG_BUF(float, a, ctx, S_AREA, N);
            d_w = w;
            d_area = a;
            if (weights) CG_TRY(up(ctx, d_w, weights, N * 4));
            else CG_LAUNCH(ctx) k_fill_value<<<grid, 256, 0, ctx->stream>>>(d_w, N, 1.0f);
            CG_CHECK_LAUNCH(ctx);
        }
        CG_TRY(tree_walk_dev(ctx, W, H, d_land, d_recv, d_w, d_key, d_donors, d_area, nullptr));
        if (order) {
            CG_BUF(int32_t, d_order, ctx, S_ORDER, N);
            CG_TRY(order_from_keys_dev(ctx, W, H, d_land, d_key, land_cells, d_order));
            if (land_cells > 0) CG_TRY(down(ctx, order, d_order, (size_t)land_cells * 4));
        }
        if (area) CG_TRY(down(ctx, area, d_area, N * 4));
    }
    if (filled) CG_TRY(down(ctx, filled, d_filled, N * 4));
    CG_TRY(down(ctx, receivers, d_recv, N * 4));
    return sync(ctx);
}

cg_status cg_breach(cg_ctx* ctx, const cg_erosion_params* p, const uint8_t* is_land, float* relative, float* ground,
                    const int32_t* receivers, const float* area, float land_cells, float land_range, float* surface,
                    int32_t* cells_cut) {
    if (!ctx || !p || !is_land || !relative || !ground || !receivers || !area || !surface) return CG_BAD_ARG;
    ctx->run.active = false;   // this call reuses the resident world's buffers
    if (p->abi_version != CG_ABI_VERSION)
        return fail(ctx, CG_BAD_ARG, "params carry ABI version %u, this library is %u", p->abi_version,
                    CG_ABI_VERSION);
    CG_TRY(check_grid(ctx, p->width, p->height));
    CG_CUDA(ctx, cudaSetDevice(ctx->device));
    const int W = p->width, H = p->height;
    const size_t N = (size_t)W * H;
    const RatesF rates = rates_of(*p);
    BreachRates br;
    br.relative_incision_coefficient = rates.relative_incision_coefficient;
    br.notch_fall_per_cell = rates.notch_fall_per_cell;
    br.outlet_reach_cells = rates.outlet_reach_cells;
    br.pond_depth = rates.pond_depth;
    br.step_ns = rates.step_ns;
    br.step_diag = rates.step_diag;
    CG_BUF(uint8_t, d_land, ctx, S_LAND, N);
    CG_BUF(float, d_rel, ctx, S_REL, N);
    CG_BUF(float, d_filled, ctx, S_FILLED, N);
    CG_BUF(int32_t, d_recv, ctx, S_RECV, N);
    CG_BUF(float, d_area, ctx, S_AREA, N);
    CG_BUF(float, d_h, ctx, S_H0, N);
    CG_TRY(up(ctx, d_land, is_land, N));
    CG_TRY(up(ctx, d_rel, relative, N * 4));
    CG_TRY(up(ctx, d_filled, ground, N * 4));
    CG_TRY(up(ctx, d_recv, receivers, N * 4));
    CG_TRY(up(ctx, d_area, area, N * 4));
    CG_TRY(up(ctx, d_h, surface, N * 4));
    int cells = 0;
    CG_TRY(breach_dev(ctx, W, H, d_land, d_rel, d_filled, d_recv, d_area, land_cells, land_range, br, d_h, &cells));
    CG_TRY(down(ctx, relative, d_rel, N * 4));
    CG_TRY(down(ctx, ground, d_filled, N * 4));
    CG_TRY(down(ctx, surface, d_h, N * 4));
    CG_TRY(sync(ctx));
    if (cells_cut) *cells_cut = cells;
    return CG_OK;
}

cg_status cg_spillways(cg_ctx* ctx, int32_t W, int32_t H, const uint8_t* is_land, const float* relative,
                       const float* filled, const int32_t* receivers, float pond_depth, int32_t* basin_of_cell,
                       cg_basins* basins) {
    if (!ctx || !is_land || !relative || !filled || !receivers) return CG_BAD_ARG;
    ctx->run.active = false;   // this call reuses the resident world's buffers
    CG_TRY(check_grid(ctx, W, H));
    CG_CUDA(ctx, cudaSetDevice(ctx->device));
    size_t N = (size_t)W * H;
    CG_BUF(uint8_t, d_land, ctx, S_LAND, N);
    CG_BUF(float, d_rel, ctx, S_REL, N);
    CG_BUF(float, d_filled, ctx, S_FILLED, N);
    CG_BUF(int32_t, d_recv, ctx, S_RECV, N);
    CG_BUF(int32_t, d_lab, ctx, S_BASIN2, N);
    CG_TRY(up(ctx, d_land, is_land, N));
    CG_TRY(up(ctx, d_rel, relative, N * 4));
    CG_TRY(up(ctx, d_filled, filled, N * 4));
    CG_TRY(up(ctx, d_recv, receivers, N * 4));
    CG_TRY(spillways_dev(ctx, W, H, d_land, d_rel, d_filled, d_recv, pond_depth, d_lab, basins));
    if (basin_of_cell) CG_TRY(down(ctx, basin_of_cell, d_lab, N * 4));
    return sync(ctx);
}

}  // extern "C"
