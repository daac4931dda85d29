// TEST INFRASTRUCTURE ONLY - the oracle.
//
// A CPU restatement of Cartogenesis's per-round erosion stage, written to follow the Kotlin
// reference statement by statement: the same float and double rounding points, the same loop and
// neighbour orders, the same sequential sums, heap keys, FIFO queue and DFS stacks. Built with
// -O2 -ffp-contract=off so that, as on the JVM, no multiply-add is fused.
//
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it, and there
// only as the checker (or the timed CPU stand-in for the Kotlin path, which cannot run without a
// JVM). The product path never calls it.
//
// Reference files (paths inside the Cartogenesis project; P = worldgen/src/commonMain/kotlin/
// com/cartogenesis/worldgen/pipeline, M = .../worldgen/model, MA = .../worldgen/math):
//   P/ErosionStage.kt, P/HydraulicErosion.kt, P/FlowRouting.kt, P/FlatRouting.kt,
//   P/SeaLevelStage.kt, P/Runoff.kt, MA/GroundSteps.kt, MA/LongMinHeap.kt, M/WorldGenConfig.kt.
// Parity of this restatement with the Kotlin code is pinned through the reference's own
// known-answer tests (tests/test_oracle_pins.py); no golden arrays exist in the reference.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <queue>
#include <vector>

#include "../include/cg_erosion.h"

namespace {

using u8 = uint8_t;

// ---------------------------------------------------------------- scale and config (M/WorldGenConfig.kt)

struct Scale {
    double world_width_km;
    float highest_land;
    float deepest_ocean;
    double years_per_round;
    // WorldScale.reliefSpanMetres: a Float sum (WorldGenConfig.kt:178).
    float relief_span() const { return highest_land + deepest_ocean; }
    // WorldGenConfig.kt:206-207.
    float land_half() const { return highest_land / relief_span(); }
    float sea_half() const { return deepest_ocean / relief_span(); }
    // WorldGenConfig.kt:146, 161.
    float relief_share_of_metres(float m) const { return m / highest_land; }
    float field_share_of_metres(float m) const { return m / relief_span(); }
    // WorldGenConfig.kt:210-231.
    double cell_width_km(int w) const { return world_width_km / w; }
    double cell_height_km(int h) const { return world_width_km * 0.5 / h; }
    double world_area_km2() const { return world_width_km * world_width_km * 0.5; }
};

Scale scale_of(const cg_erosion_params& p) {
    return Scale{p.world_width_km, p.highest_land_metres, p.deepest_ocean_metres, p.years_per_hydraulic_round};
}

// kotlin.math.round on Float/Double rounds half to even (rint).
// WorldGenConfig.cellsFor / wholeCellsFor (WorldGenConfig.kt:3331, 3340-3341).
int whole_cells_for(const cg_erosion_params& p, double km, int at_least) {
    float cells = (float)(km * p.width / p.world_width_km);
    int r = (int)std::nearbyint(cells);
    return r < at_least ? at_least : r;
}

// ErosionStage.sweepsFor (ErosionStage.kt:412-413).
int sweeps_for(const cg_erosion_params& p) { return whole_cells_for(p, p.debris_travel_km, 0); }

// ErosionStage.thermalLimits (ErosionStage.kt:428-437).
cg_thermal_limits thermal_limits(const cg_erosion_params& p) {
    Scale s = scale_of(p);
    double critical_per_km = (double)p.critical_fall_metres_per_km / (double)s.relief_span();
    double cw = s.cell_width_km(p.width);
    double ch = s.cell_height_km(p.height);
    cg_thermal_limits l;
    l.east_west = (float)(critical_per_km * cw);
    l.north_south = (float)(critical_per_km * ch);
    l.diagonal = (float)(critical_per_km * std::sqrt(cw * cw + ch * ch));
    return l;
}

// GroundLattice.wholeCycles(worldWidthKm, 187.5) (noise/GroundLattice.kt:81-82,
// FlowRouting.kt:407-414).
int smooth_field_lattice_columns(double world_width_km) {
    int r = (int)std::nearbyint(world_width_km / 187.5);
    return r < 1 ? 1 : r;
}

// ---------------------------------------------------------------- GroundSteps (MA/GroundSteps.kt:20-59)

struct GroundSteps {
    float east_west = 1.0f;
    float north_south;
    float diagonal;
    explicit GroundSteps(double r)
        : north_south((float)r), diagonal((float)std::sqrt(1.0 + r * r)) {}
    float of(int dc, int dr) const {
        if (dc != 0 && dr != 0) return diagonal;
        if (dr != 0) return north_south;
        return east_west;
    }
    float between(int from, int to, int width) const {
        bool same_row = from / width == to / width;
        bool same_col = from % width == to % width;
        if (!same_row && !same_col) return diagonal;
        if (!same_row) return north_south;
        return east_west;
    }
};

// ---------------------------------------------------------------- thermal sweep (ErosionStage.kt:235-403)

const int kThermalColStep[8] = {1, -1, 0, 0, 1, 1, -1, -1};   // ErosionStage.kt:460
const int kThermalRowStep[8] = {0, 0, 1, -1, 1, -1, 1, -1};   // ErosionStage.kt:461
const int kTile = 32;                                          // ErosionStage.kt:76

std::vector<u8> dilate(const std::vector<u8>& mask, int ta, int td) {   // ErosionStage.kt:440-457
    std::vector<u8> grown(mask.size(), 0);
    for (int tr = 0; tr < td; ++tr)
        for (int tc = 0; tc < ta; ++tc) {
            if (!mask[tr * ta + tc]) continue;
            for (int rs = -1; rs <= 1; ++rs) {
                int nr = tr + rs;
                if (nr < 0 || nr >= td) continue;
                for (int cs = -1; cs <= 1; ++cs) {
                    int nc = (tc + cs + ta) % ta;
                    grown[nr * ta + nc] = 1;
                }
            }
        }
    return grown;
}

void thermal_sweep(int W, int H, const float* in, float* out, cg_thermal_limits lim, int sweeps,
                   float rate, bool skip_settled) {
    size_t N = (size_t)W * H;
    std::vector<float> heights(in, in + N), next(N, 0.0f), give(N, 0.0f);
    if (sweeps <= 0) {
        std::memcpy(out, in, N * sizeof(float));
        return;
    }
    float limit_by[8];
    for (int n = 0; n < 8; ++n)
        limit_by[n] = n >= 4 ? lim.diagonal : (kThermalRowStep[n] != 0 ? lim.north_south : lim.east_west);
    const float settled = lim.east_west * 1e-3f;   // SETTLED_SHARE_OF_CRITICAL_SLOPE
    int ta = (W + kTile - 1) / kTile, td = (H + kTile - 1) / kTile;
    std::vector<u8> has_excess(ta * td, 0), can_change(ta * td, 1), can_hold(ta * td, 1);

    for (int s = 0; s < sweeps; ++s) {
        const float* cur = heights.data();
        // parallelChunks over tile rows (ErosionStage.kt:292): cells are independent within a pass.
#pragma omp parallel for schedule(dynamic)
        for (int tr = 0; tr < td; ++tr)
            for (int tc = 0; tc < ta; ++tc) {
                int tile = tr * ta + tc;
                if (skip_settled && !can_hold[tile]) continue;
                bool tile_excess = false;
                int row_end = std::min((tr + 1) * kTile, H), col_end = std::min((tc + 1) * kTile, W);
                for (int row = tr * kTile; row < row_end; ++row)
                    for (int col = tc * kTile; col < col_end; ++col) {
                        int cell = row * W + col;
                        float here = cur[cell];
                        float excess = 0.0f, steepest = 0.0f;
                        for (int n = 0; n < 8; ++n) {
                            int nr = row + kThermalRowStep[n];
                            if (nr < 0 || nr >= H) continue;
                            int nc = (col + kThermalColStep[n] + W) % W;
                            float drop = here - cur[nr * W + nc];
                            if (drop <= 0.0f) continue;
                            if (drop > steepest) steepest = drop;
                            float limit = limit_by[n];
                            if (drop > limit) excess += drop - limit;
                        }
                        if (excess <= settled) {
                            give[cell] = 0.0f;
                        } else {
                            float a = rate * excess, b = steepest * 0.5f;   // MAX_SHARE_OF_STEEPEST_DROP
                            give[cell] = (a <= b ? a : b) / excess;
                            tile_excess = true;
                        }
                    }
                has_excess[tile] = tile_excess;
            }
        can_change = dilate(has_excess, ta, td);
        can_hold = dilate(can_change, ta, td);
        float* wr = next.data();
#pragma omp parallel for schedule(dynamic)
        for (int tr = 0; tr < td; ++tr)
            for (int tc = 0; tc < ta; ++tc) {
                int tile = tr * ta + tc;
                int row_end = std::min((tr + 1) * kTile, H), col_end = std::min((tc + 1) * kTile, W);
                if (skip_settled && !can_change[tile]) {
                    for (int row = tr * kTile; row < row_end; ++row)
                        for (int col = tc * kTile; col < col_end; ++col) wr[row * W + col] = cur[row * W + col];
                    continue;
                }
                for (int row = tr * kTile; row < row_end; ++row)
                    for (int col = tc * kTile; col < col_end; ++col) {
                        int cell = row * W + col;
                        float here = cur[cell];
                        float received = 0.0f, given = 0.0f;
                        for (int n = 0; n < 8; ++n) {
                            int nr = row + kThermalRowStep[n];
                            if (nr < 0 || nr >= H) continue;
                            int nc = (col + kThermalColStep[n] + W) % W;
                            float limit = limit_by[n];
                            int ncell = nr * W + nc;
                            float incoming = cur[ncell] - here;
                            if (incoming > limit) {
                                received += give[ncell] * (incoming - limit);
                            } else if (-incoming > limit) {
                                given += give[cell] * (-incoming - limit);
                            }
                        }
                        wr[cell] = here - given + received;
                    }
            }
        heights.swap(next);
    }
    std::memcpy(out, heights.data(), N * sizeof(float));
}

// ---------------------------------------------------------------- percentile cut (SeaLevelStage.kt)

int32_t float_bits(float f) {
    int32_t b;
    std::memcpy(&b, &f, 4);
    return b;
}

// SeaLevelStage.sortableBits (SeaLevelStage.kt:648-651).
int32_t sortable_bits(float v) {
    int32_t bits = float_bits(v);
    return bits < 0 ? (bits ^ 0x7FFFFFFF) : bits;
}

// shorelineForFraction's row weights (SeaLevelStage.kt:580-584) and their sequential total.
void row_weights(int W, int H, std::vector<double>& w, double& total) {
    const double PI = 3.141592653589793;
    w.resize(H);
    for (int row = 0; row < H; ++row) w[row] = std::cos(PI / 2 - (row + 0.5) / H * PI);
    total = 0.0;
    for (int row = 0; row < H; ++row) total += w[row] * W;
}

// SeaLevelStage.thresholdAtWeight (SeaLevelStage.kt:600-645).
float threshold_at_weight(int W, int H, const float* h, const std::vector<double>& rw, double target) {
    size_t N = (size_t)W * H;
    float lowest = h[0], highest = h[0];
    for (size_t i = 1; i < N; ++i) {
        if (h[i] < lowest) lowest = h[i];
        if (h[i] > highest) highest = h[i];
    }
    if (highest - lowest <= 0.0f) return lowest;
    if (target <= 0.0) return lowest;
    const int BINS = 4096;   // HISTOGRAM_BINS
    float per = (float)(BINS - 1) / (highest - lowest);
    auto bin_of = [&](float v) {
        float x = (v - lowest) * per;
        // Kotlin Float.toInt(): truncation, NaN -> 0, saturating.
        int b;
        if (x != x) b = 0;
        else if (x >= 2147483647.0f) b = 2147483647;
        else if (x <= -2147483648.0f) b = (-2147483647 - 1);
        else b = (int)x;
        return b < 0 ? 0 : (b > BINS - 1 ? BINS - 1 : b);
    };
    std::vector<double> hist(BINS, 0.0);
    for (size_t c = 0; c < N; ++c) hist[bin_of(h[c])] += rw[c / W];
    double below_bracket = 0.0;
    int bracket_bin = BINS - 1;
    for (int b = 0; b < BINS; ++b) {
        if (below_bracket + hist[b] >= target) {
            bracket_bin = b;
            break;
        }
        below_bracket += hist[b];
    }
    std::vector<int64_t> bracket;
    for (size_t c = 0; c < N; ++c)
        if (bin_of(h[c]) == bracket_bin)
            bracket.push_back((int64_t)((uint64_t)(int64_t)sortable_bits(h[c]) << 32) | (int64_t)c);
    if (bracket.empty()) return highest;
    std::sort(bracket.begin(), bracket.end());
    double below = below_bracket;
    for (int64_t e : bracket) {
        int cell = (int)(e & 0xFFFFFFFFLL);
        if (below >= target) return h[cell];
        below += rw[cell / W];
    }
    return h[(int)(bracket.back() & 0xFFFFFFFFLL)];
}

struct Cut {
    float shoreline;
    std::vector<u8> is_land;
    std::vector<float> relative;
    int land_cells;
};

// SeaLevelStage.percentileCut + landAndWaterAt (SeaLevelStage.kt:146-200).
void percentile_cut(int W, int H, const float* h, float sea_level, const Scale& sc, float lowstand_share,
                    Cut& out) {
    float submerged = sea_level < 0.0f ? 0.0f : (sea_level > 1.0f ? 1.0f : sea_level);
    std::vector<double> rw;
    double total;
    row_weights(W, H, rw, total);
    float todays = threshold_at_weight(W, H, h, rw, submerged * total);
    float shoreline = todays - lowstand_share;
    size_t N = (size_t)W * H;
    out.shoreline = shoreline;
    out.is_land.assign(N, 0);
    out.relative.assign(N, 0.0f);
    float land_half = std::max(sc.land_half(), 1e-6f);   // MIN_RANGE
    float sea_half = std::max(sc.sea_half(), 1e-6f);
    int land = 0;
    for (size_t c = 0; c < N; ++c) {
        float g = h[c];
        if (g >= shoreline) {
            out.is_land[c] = 1;
            ++land;
            out.relative[c] = (g - shoreline) / land_half;
        } else {
            out.relative[c] = (g - shoreline) / sea_half;
        }
    }
    out.land_cells = land;
}

// ---------------------------------------------------------------- FlowRouting

const float kFlatGradientStep = 1e-6f;   // FlowRouting.kt:34
const float kElevationBias = 4.0f;       // FlowRouting.kt:753

// FlowRouting.encode (FlowRouting.kt:739-742).
int64_t encode(float elevation, int index) {
    int32_t bits = float_bits(elevation + kElevationBias);
    return (int64_t)((uint64_t)(int64_t)bits << 32) | (int64_t)(uint32_t)index;
}
int decode_index(int64_t e) { return (int)(e & 0xFFFFFFFFLL); }

// FlowRouting.forEachNeighbour (FlowRouting.kt:755-772): rows -1..1, columns -1..1, x wraps.
template <class F>
inline void for_each_neighbour(int W, int H, int col, int row, F&& f) {
    for (int rs = -1; rs <= 1; ++rs) {
        int nr = row + rs;
        if (nr < 0 || nr >= H) continue;
        for (int cs = -1; cs <= 1; ++cs) {
            if (cs == 0 && rs == 0) continue;
            int nc = (col + cs) % W;
            if (nc < 0) nc += W;
            f(nr * W + nc, cs, rs);
        }
    }
}

// FlowRouting.fillDepressions (FlowRouting.kt:52-111). LongMinHeap (MA/LongMinHeap.kt) pops the
// smallest key; every cell is pushed at most once, so keys are unique and any min-heap pops the
// same sequence.
void fill_depressions(int W, int H, const u8* is_land, const float* elev, float* filled) {
    size_t N = (size_t)W * H;
    std::memcpy(filled, elev, N * sizeof(float));
    std::vector<u8> visited(N, 0);
    std::priority_queue<int64_t, std::vector<int64_t>, std::greater<int64_t>> heap;
    for (size_t c = 0; c < N; ++c)
        if (!is_land[c]) visited[c] = 1;
    for (int row = 0; row < H; ++row)
        for (int col = 0; col < W; ++col) {
            int cell = row * W + col;
            if (!is_land[cell]) {
                bool touches = false;
                for_each_neighbour(W, H, col, row, [&](int n, int, int) {
                    if (is_land[n]) touches = true;
                });
                if (touches) heap.push(encode(filled[cell], cell));
                continue;
            }
            if (row == 0 || row == H - 1) {
                if (!visited[cell]) {
                    visited[cell] = 1;
                    heap.push(encode(filled[cell], cell));
                }
            }
        }
    while (!heap.empty()) {
        int64_t lowest = heap.top();
        heap.pop();
        int cell = decode_index(lowest);
        float ce = filled[cell];
        int cc = cell % W, cr = cell / W;
        for_each_neighbour(W, H, cc, cr, [&](int n, int, int) {
            if (!visited[n]) {
                visited[n] = 1;
                if (filled[n] <= ce) filled[n] = ce + kFlatGradientStep;
                heap.push(encode(filled[n], n));
            }
        });
    }
}

// FlowRouting.seededNoise (FlowRouting.kt:426-436): SplitMix64 rounds on wrapping 64-bit ints.
float seeded_noise(int lc, int lr, int64_t seed) {
    uint64_t mixed = (uint64_t)seed ^ ((uint64_t)(int64_t)lc * (uint64_t)(-0x61c8864680b583ebLL)) ^
                     ((uint64_t)(int64_t)lr * (uint64_t)0x27220a951d5a2b1fLL);
    mixed ^= mixed >> 30;
    mixed *= (uint64_t)(-0x40a7b892e31b1a47LL);
    mixed ^= mixed >> 27;
    mixed *= (uint64_t)(-0x6b2fb644ecceee15LL);
    mixed ^= mixed >> 31;
    int top = (int)(mixed >> 40);
    return (float)top / 8388608.0f - 1.0f;
}

float lerpf(float from, float to, float at) { return from + (to - from) * at; }

// FlowRouting.smoothSeededField (FlowRouting.kt:377-399).
float smooth_seeded_field(int W, int lattice, int col, int row, int64_t seed) {
    int cal = col * lattice, ral = row * lattice;
    int ccol = cal / W, crow = ral / W;
    float ac = (float)(cal - ccol * W) / (float)W;
    float ar = (float)(ral - crow * W) / (float)W;
    float ec = ac * ac * (3.0f - 2.0f * ac);
    float er = ar * ar * (3.0f - 2.0f * ar);
    int west = ccol % lattice, east = (ccol + 1) % lattice;
    float north = lerpf(seeded_noise(west, crow, seed), seeded_noise(east, crow, seed), ec);
    float south = lerpf(seeded_noise(west, crow + 1, seed), seeded_noise(east, crow + 1, seed), ec);
    return lerpf(north, south, er);
}

const int64_t kSubGridDrawSalt = 0x5f3a91c72b64d8e3LL;   // FlowRouting.kt:358
const int64_t kRainReliefSalt = 0x3c6ef372fe94f82bLL;    // FlatRouting.kt:507

// FlowRouting.subGridDraw (FlowRouting.kt:355-356).
double sub_grid_draw(int col, int row, int64_t seed) {
    return (double)((seeded_noise(col, row, seed ^ kSubGridDrawSalt) + 1.0f) * 0.5f);
}

// FlowRouting.neighbourAt (FlowRouting.kt:443-448).
int neighbour_at(int W, int H, int col, int row) {
    if (row < 0 || row >= H) return -1;
    int wc = col % W;
    if (wc < 0) wc += W;
    return row * W + wc;
}

const int kCardColStep[4] = {1, 0, -1, 0};   // FlowRouting.kt:451
const int kCardRowStep[4] = {0, -1, 0, 1};   // FlowRouting.kt:452

// FlowRouting.facetReceiver (FlowRouting.kt:223-310).
int facet_receiver(int W, int H, const double* rs, int col, int row, const GroundSteps& steps, int64_t seed) {
    double here = rs[row * W + col];
    double steepest = 0.0;
    int fcard = -1, fdiag = -1;
    double dshare = 0.0;
    for (int side = 0; side < 4; ++side) {
        int ccs = kCardColStep[side], crs = kCardRowStep[side];
        int card = neighbour_at(W, H, col + ccs, row + crs);
        if (card < 0) continue;
        double cdrop = here - rs[card];
        double to_card = (double)steps.of(ccs, crs);
        double on_to_diag = (double)(ccs == 0 ? steps.east_west : steps.north_south);
        for (int turn = -1; turn <= 1; turn += 2) {
            int dcs = ccs == 0 ? turn : ccs;
            int drs = crs == 0 ? turn : crs;
            int diag = neighbour_at(W, H, col + dcs, row + drs);
            if (diag < 0) continue;
            double dfall = here - rs[diag];
            double dslope = dfall / (double)steps.diagonal;
            double outward = dfall - cdrop;
            double cslope = cdrop / to_card;
            double oslope = outward / on_to_diag;
            double share_edge = cdrop > 0.0 ? outward * to_card * to_card / (cdrop * on_to_diag * on_to_diag) : 1.0;
            bool to_cardinal = cdrop > 0.0 && outward <= 0.0;
            bool to_diagonal = !to_cardinal && share_edge >= 1.0;
            double fslope = to_cardinal ? cslope : (to_diagonal ? dslope : std::sqrt(cslope * cslope + oslope * oslope));
            double share = to_cardinal ? 0.0 : (to_diagonal ? 1.0 : share_edge);
            if (fslope > steepest) {
                steepest = fslope;
                fcard = card;
                fdiag = diag;
                dshare = share;
            }
        }
    }
    if (steepest <= 0.0) return -1;
    if (dshare <= 0.0) return fcard;
    if (dshare >= 1.0) return fdiag;
    if (sub_grid_draw(col, row, seed) < dshare) return fdiag;
    return fcard;
}

// FlowRouting.steepestNeighbourOf (FlowRouting.kt:320-343).
int steepest_neighbour_of(int W, int H, const double* rs, int col, int row, const GroundSteps& steps) {
    int steepest = -1;
    double sd = 0.0;
    double here = rs[row * W + col];
    for_each_neighbour(W, H, col, row, [&](int n, int cs, int rs_) {
        double there = rs[n];
        double drop = (here - there) / (double)steps.of(cs, rs_);
        if (drop > sd) {
            sd = drop;
            steepest = n;
        }
    });
    return steepest;
}

// ---------------------------------------------------------------- FlatRouting (FlatRouting.kt)

struct Stencil {
    double ew, ns, diag;
};

// FlatRouting.stencil (FlatRouting.kt:177-186).
Stencil stencil_of(double r) {
    if (r <= 1.0) {
        double d = 2.0 / (1.0 + r * r);
        return Stencil{1.0, (1.0 + 2.0 * d) / (r * r) - 2.0 * d, d};
    }
    double d = 2.0 / (1.0 + 1.0 / (r * r));
    return Stencil{r * r * (1.0 + 2.0 * d) - 2.0 * d, 1.0, d};
}

const int kLaid = 0x7FFFFFFF;   // FlatRouting.kt:141

// FlatRouting.ColumnRuns (FlatRouting.kt:350-414).
struct ColumnRuns {
    std::vector<int> order, run_start;
    std::vector<double> pivot;
    double ns;
    ColumnRuns(int W, const std::vector<int>& members, int mc, const std::vector<int>& local,
               const std::vector<double>& degree, double northSouth)
        : order(mc), pivot(mc), ns(northSouth) {
        auto member_at = [&](long cell) -> int {
            if (cell < 0 || cell >= (long)local.size()) return -1;
            int l = local[cell];
            return (l >= 0 && l < mc) ? l : -1;
        };
        int placed = 0;
        for (int m = 0; m < mc; ++m) {
            if (member_at((long)members[m] - W) >= 0) continue;
            run_start.push_back(placed);
            int here = m;
            while (here >= 0) {
                order[placed++] = here;
                here = member_at((long)members[here] + W);
            }
        }
        run_start.push_back(placed);
        for (size_t run = 0; run + 1 < run_start.size(); ++run)
            for (int pos = run_start[run]; pos < run_start[run + 1]; ++pos) {
                double d = degree[order[pos]];
                pivot[pos] = pos == run_start[run] ? d : d - ns * ns / pivot[pos - 1];
            }
    }
    void solve(const std::vector<double>& right, std::vector<double>& into) const {
        for (size_t run = 0; run + 1 < run_start.size(); ++run) {
            int first = run_start[run], last = run_start[run + 1] - 1;
            for (int pos = first; pos <= last; ++pos) {
                double carried = pos == first ? 0.0 : ns * into[order[pos - 1]];
                into[order[pos]] = (right[order[pos]] + carried) / pivot[pos];
            }
            for (int pos = last - 1; pos >= first; --pos)
                into[order[pos]] += ns / pivot[pos] * into[order[pos + 1]];
        }
    }
};

// FlatRouting.solvePotential (FlatRouting.kt:215-337). Returns false for null.
bool solve_potential(int W, int H, const std::vector<int>& members, int mc, const std::vector<int>& local,
                     const std::vector<double>& surface, double entry_level, int64_t seed, double r, int lattice,
                     std::vector<double>& x) {
    Stencil st = stencil_of(r);
    std::vector<double> degree(mc);
    std::vector<int> nstart(mc + 1), nbrs((size_t)mc * 8);
    std::vector<double> wts((size_t)mc * 8);
    int written = 0;
    for (int m = 0; m < mc; ++m) {
        int cell = members[m];
        int col = cell % W, row = cell / W;
        nstart[m] = written;
        double total = 0.0;
        for (int rs = -1; rs <= 1; ++rs) {
            int nr = row + rs;
            if (nr < 0 || nr >= H) continue;
            for (int cs = -1; cs <= 1; ++cs) {
                if (cs == 0 && rs == 0) continue;
                int nc = (col + cs) % W;
                if (nc < 0) nc += W;
                int n = nr * W + nc;
                double w = (cs != 0 && rs != 0) ? st.diag : (rs != 0 ? st.ns : st.ew);
                int l = local[n];
                if (l >= 0 && l < mc && l != kLaid) {
                    nbrs[written] = l;
                    wts[written] = w;
                    ++written;
                    total += w;
                } else if (l < 0 && surface[n] < entry_level) {
                    total += w;
                }
            }
        }
        degree[m] = total;
    }
    nstart[mc] = written;
    auto apply_laplacian = [&](const std::vector<double>& xx, std::vector<double>& into) {
        for (int m = 0; m < mc; ++m) {
            double sum = degree[m] * xx[m];
            for (int s = nstart[m]; s < nstart[m + 1]; ++s) sum -= wts[s] * xx[nbrs[s]];
            into[m] = sum;
        }
    };
    x.assign(mc, 0.0);
    std::vector<double> residual(mc);
    for (int m = 0; m < mc; ++m) {
        int cell = members[m];
        residual[m] = 1.0 + 0.5 * (double)smooth_seeded_field(W, lattice, cell % W, cell / W, seed ^ kRainReliefSalt);
    }
    ColumnRuns runs(W, members, mc, local, degree, st.ns);
    std::vector<double> pre(mc, 0.0);
    runs.solve(residual, pre);
    std::vector<double> direction = pre, product(mc, 0.0);
    double rnorm = 0.0, rap = 0.0;
    for (int m = 0; m < mc; ++m) {
        rnorm += residual[m] * residual[m];
        rap += residual[m] * pre[m];
    }
    const double tol = 1e-7;   // RESIDUAL_TOLERANCE
    double stop_at = rnorm * tol * tol;
    int most = 64 + (int)(8.0 * std::sqrt((double)mc));   // MOST_ITERATIONS_FLOOR, _PER_ROOT_CELL
    int it = 0;
    while (rnorm > stop_at && it < most) {
        apply_laplacian(direction, product);
        double energy = 0.0;
        for (int m = 0; m < mc; ++m) energy += direction[m] * product[m];
        if (energy <= 0.0 || rap <= 0.0) break;
        double step = rap / energy;
        double next_norm = 0.0;
        for (int m = 0; m < mc; ++m) {
            x[m] += step * direction[m];
            residual[m] -= step * product[m];
            next_norm += residual[m] * residual[m];
        }
        runs.solve(residual, pre);
        double next_ap = 0.0;
        for (int m = 0; m < mc; ++m) next_ap += residual[m] * pre[m];
        double improvement = next_ap / rap;
        for (int m = 0; m < mc; ++m) direction[m] = pre[m] + improvement * direction[m];
        rnorm = next_norm;
        rap = next_ap;
        ++it;
    }
    for (int m = 0; m < mc; ++m)
        if (!(x[m] > 0.0)) return false;
    return true;
}

// FlatRouting.highestEntryOf (FlatRouting.kt:427-445).
double highest_entry_of(int W, int H, const std::vector<int>& members, int mc, const std::vector<int>& local,
                        const std::vector<double>& surface, double entry_level) {
    double highest = -INFINITY;
    for (int m = 0; m < mc; ++m) {
        int cell = members[m];
        for_each_neighbour(W, H, cell % W, cell / W, [&](int n, int, int) {
            double there = surface[n];
            if (local[n] < 0 && there < entry_level && there > highest) highest = there;
        });
    }
    return highest;
}

// FlatRouting.layInBand (FlatRouting.kt:455-489).
bool lay_in_band(int W, int H, const std::vector<int>& members, int mc, std::vector<double>& surface,
                 const std::vector<double>& potential, double entry_height, double entry_level) {
    double highest = 0.0;
    for (int m = 0; m < mc; ++m)
        if (potential[m] > highest) highest = potential[m];
    if (highest <= 0.0 || entry_height >= entry_level) return false;
    std::vector<double> staircase(mc);
    for (int m = 0; m < mc; ++m) staircase[m] = surface[members[m]];
    double floor_ = entry_height;
    double band = (entry_level - entry_height) * 0.9;   // BAND_SHARE_OF_THE_GAP
    for (int m = 0; m < mc; ++m) surface[members[m]] = floor_ + band * (potential[m] / highest);
    for (int m = 0; m < mc; ++m) {
        int cell = members[m];
        double here = surface[cell];
        bool has_lower = false;
        for_each_neighbour(W, H, cell % W, cell / W, [&](int n, int, int) {
            if (!has_lower && surface[n] < here) has_lower = true;
        });
        if (!has_lower) {
            for (int u = 0; u < mc; ++u) surface[members[u]] = staircase[u];
            return false;
        }
    }
    return true;
}

struct FlatCounts {
    int flats = 0, kept = 0, raised = 0;
};

// FlatRouting.surfaceOf (FlatRouting.kt:58-138).
void surface_of(int W, int H, const u8* is_land, const float* elev, const float* filled, int64_t seed, double r,
                int lattice, std::vector<double>& surface, FlatCounts& counts) {
    size_t N = (size_t)W * H;
    surface.resize(N);
    for (size_t c = 0; c < N; ++c) surface[c] = (double)(is_land[c] ? filled[c] : elev[c]);
    std::vector<u8> raised(N);
    for (size_t c = 0; c < N; ++c) raised[c] = is_land[c] && filled[c] > elev[c];
    std::vector<int> local(N, -1), stack, members;
    counts = FlatCounts{};
    for (size_t start = 0; start < N; ++start) {
        if (!raised[start] || local[start] >= 0) continue;
        members.clear();
        stack.clear();
        stack.push_back((int)start);
        local[start] = 0;
        members.push_back((int)start);
        float lowest = filled[start];
        while (!stack.empty()) {
            int cell = stack.back();
            stack.pop_back();
            if (filled[cell] < lowest) lowest = filled[cell];
            for_each_neighbour(W, H, cell % W, cell / W, [&](int n, int, int) {
                if (raised[n] && local[n] < 0) {
                    local[n] = (int)members.size();
                    members.push_back(n);
                    stack.push_back(n);
                }
            });
        }
        int mc = (int)members.size();
        counts.flats++;
        counts.raised += mc;
        double entry_level = (double)lowest;
        double entry_height = highest_entry_of(W, H, members, mc, local, surface, entry_level);
        std::vector<double> potential;
        bool ok = solve_potential(W, H, members, mc, local, surface, entry_level, seed, r, lattice, potential);
        if (!(ok && lay_in_band(W, H, members, mc, surface, potential, entry_height, entry_level))) counts.kept++;
        for (int m = 0; m < mc; ++m) {
            raised[members[m]] = 0;
            local[members[m]] = kLaid;
        }
    }
}

// FlowRouting.flowDirections (FlowRouting.kt:179-216).
void flow_directions(int W, int H, const u8* is_land, const float* elev, const float* filled, int64_t seed, double r,
                     int lattice, bool by_facet, bool over_potential, int32_t* receiver, std::vector<double>* surf_out,
                     FlatCounts* counts_out) {
    size_t N = (size_t)W * H;
    std::vector<double> surface;
    FlatCounts counts;
    if (over_potential) {
        surface_of(W, H, is_land, elev, filled, seed, r, lattice, surface, counts);
    } else {
        surface.resize(N);
        for (size_t c = 0; c < N; ++c) surface[c] = (double)(is_land[c] ? filled[c] : elev[c]);
    }
    GroundSteps steps(r);
    for (int row = 0; row < H; ++row)
        for (int col = 0; col < W; ++col) {
            int cell = row * W + col;
            receiver[cell] = -1;
            if (!is_land[cell]) continue;
            receiver[cell] = by_facet ? facet_receiver(W, H, surface.data(), col, row, steps, seed)
                                      : steepest_neighbour_of(W, H, surface.data(), col, row, steps);
        }
    if (surf_out) surf_out->swap(surface);
    if (counts_out) *counts_out = counts;
}

// FlowRouting.drainageOrder (FlowRouting.kt:695-729).
void drainage_order(int W, int H, const u8* is_land, const int32_t* target, int land_cells, int32_t* order) {
    size_t N = (size_t)W * H;
    std::vector<int> feeding(N, 0);
    for (size_t c = 0; c < N; ++c) {
        if (!is_land[c]) continue;
        int r = target[c];
        if (r >= 0 && is_land[r]) feeding[r]++;
    }
    int tail = 0;
    for (size_t c = 0; c < N; ++c)
        if (is_land[c] && feeding[c] == 0) order[tail++] = (int)c;
    int head = 0;
    while (head < tail) {
        int r = target[order[head++]];
        if (r >= 0 && is_land[r] && --feeding[r] == 0) order[tail++] = r;
    }
    if (tail < land_cells)
        for (size_t c = 0; c < N; ++c)
            if (is_land[c] && feeding[c] > 0) order[tail++] = (int)c;
}

// FlowRouting.accumulate (FlowRouting.kt:485-511).
void accumulate(int W, int H, const u8* is_land, const int32_t* target, int land_cells, const float* weights,
                float* area) {
    size_t N = (size_t)W * H;
    for (size_t c = 0; c < N; ++c) area[c] = is_land[c] ? weights[c] : 0.0f;
    std::vector<int32_t> order(land_cells > 0 ? land_cells : 1);
    drainage_order(W, H, is_land, target, land_cells, order.data());
    for (int i = 0; i < land_cells; ++i) {
        int c = order[i];
        int r = target[c];
        if (r >= 0 && is_land[r]) area[r] += area[c];
    }
}

struct Spillways {
    int count = 0;
    std::vector<int> spill, entry, cells;
    std::vector<float> level, floor_;
    int largest = -1, largest_cells = 0;
    float largest_depth = 0.0f, deepest = 0.0f;
};

// FlowRouting.spillways (FlowRouting.kt:573-677). basin_of_cell, if given, receives each ponded
// cell's basin index (the order basins are found in), -1 elsewhere.
void spillways(int W, int H, const u8* is_land, const float* elev, const float* filled, const int32_t* target,
               float pond_depth, Spillways& out, int32_t* basin_of_cell) {
    size_t N = (size_t)W * H;
    std::vector<u8> ponded(N), seen(N, 0);
    for (size_t c = 0; c < N; ++c) ponded[c] = is_land[c] && filled[c] - elev[c] > pond_depth;
    if (basin_of_cell)
        for (size_t c = 0; c < N; ++c) basin_of_cell[c] = -1;
    out = Spillways{};
    std::vector<int> stack;
    for (size_t start = 0; start < N; ++start) {
        if (!ponded[start] || seen[start]) continue;
        stack.clear();
        stack.push_back((int)start);
        seen[start] = 1;
        int cells = 0;
        float basin_floor = 3.402823466e+38f;   // Float.MAX_VALUE
        int spill = -1;
        float spill_level = 3.402823466e+38f;
        while (!stack.empty()) {
            int cell = stack.back();
            stack.pop_back();
            cells++;
            if (basin_of_cell) basin_of_cell[cell] = out.count;
            if (elev[cell] < basin_floor) basin_floor = elev[cell];
            int r = target[cell];
            if (r >= 0 && is_land[r] && !ponded[r]) {
                float exit_level = filled[r];
                if (exit_level < spill_level || (exit_level == spill_level && r < spill)) {
                    spill_level = exit_level;
                    spill = r;
                }
            }
            for_each_neighbour(W, H, cell % W, cell / W, [&](int n, int, int) {
                if (ponded[n] && !seen[n]) {
                    seen[n] = 1;
                    stack.push_back(n);
                }
            });
        }
        int pour = spill;
        if (spill >= 0) {
            int cell = spill;
            long steps = 0;
            while (cell >= 0 && is_land[cell] && filled[cell] > elev[cell] && steps < (long)N) {
                cell = target[cell];
                steps++;
            }
            if (cell >= 0 && is_land[cell]) pour = cell;
        }
        float pour_level = pour >= 0 ? filled[pour] : spill_level;
        out.entry.push_back(spill);
        out.spill.push_back(pour);
        out.level.push_back(pour >= 0 ? pour_level : basin_floor);
        out.floor_.push_back(basin_floor);
        out.cells.push_back(cells);
        float fill_depth = pour >= 0 ? pour_level - basin_floor : 0.0f;
        if (cells > out.largest_cells) {
            out.largest = out.count;
            out.largest_cells = cells;
            out.largest_depth = fill_depth;
        }
        if (fill_depth > out.deepest) out.deepest = fill_depth;
        out.count++;
    }
}

// ---------------------------------------------------------------- HydraulicErosion

const float kPondDepthMetres = 24.0f;    // HydraulicErosion.kt:192
const float kVegetationShielding = 0.5f; // HydraulicErosion.kt:1716

struct Rates {   // HydraulicErosion.Rates (HydraulicErosion.kt:203-312), the P0 and P1 members
    float incision_coefficient;
    float courant_coefficient;
    float pond_depth;
    float relative_incision_coefficient;   // HydraulicErosion.kt:246-247
    float notch_fall_per_cell;             // HydraulicErosion.kt:281-282, NOTCH_FALL_METRES_PER_KM 0.0025
    int outlet_reach_cells;                // HydraulicErosion.kt:303, ErosionConfig.outletReachKm 1500
    GroundSteps steps;
    explicit Rates(const cg_erosion_params& p) : steps(0.0) {
        Scale s = scale_of(p);
        double sl = (double)p.sea_level;
        sl = sl < 0.0 ? 0.0 : (sl > 1.0 ? 1.0 : sl);
        double land_area = (1.0 - sl) * s.world_area_km2();
        double per_year = (double)p.bedrock_erodibility_per_year * s.years_per_round;
        double geometry = std::sqrt(land_area) / s.world_width_km;
        double ratio = (double)s.highest_land / (double)s.relief_span();
        incision_coefficient = (float)(per_year * geometry * ratio);
        courant_coefficient = incision_coefficient / s.land_half() * (float)p.width;
        pond_depth = s.relief_share_of_metres(kPondDepthMetres);
        relative_incision_coefficient = incision_coefficient * s.relief_span() / s.highest_land;
        notch_fall_per_cell = s.relief_share_of_metres(0.0025f * (float)s.cell_width_km(p.width));
        outlet_reach_cells = whole_cells_for(p, 1500.0, 1);
        steps = GroundSteps(s.cell_height_km(p.height) / s.cell_width_km(p.width));
    }
};

// HydraulicErosion.standBelowToday (HydraulicErosion.kt:365-373).
float stand_below_today(const cg_erosion_params& p, int round) {
    Scale s = scale_of(p);
    float lowstand = s.field_share_of_metres(p.lowstand_metres);
    int rounds = p.hydraulic_rounds;
    if (lowstand <= 0.0f || rounds <= 1) return 0.0f;
    int rising = (int)((float)rounds * 0.25f);   // TRANSGRESSION_SHARE
    if (rising < 1) rising = 1;
    int held = rounds - rising;
    if (round < held) return lowstand;
    return lowstand * (float)(rounds - 1 - round) / (float)rising;
}

// HydraulicErosion.normaliseOverLand (HydraulicErosion.kt:550-569).
void normalise_over_land(const float* rain, const u8* is_land, int land_cells, size_t N, float* weights) {
    double summed = 0.0;
    for (size_t c = 0; c < N; ++c)
        if (is_land[c]) summed += (double)rain[c];
    float mean = (float)(summed / land_cells);
    if (mean <= 0.0f) {
        for (size_t c = 0; c < N; ++c) weights[c] = 0.0f;
        return;
    }
    for (size_t c = 0; c < N; ++c) weights[c] = rain[c] / mean;
}

// HydraulicErosion.shieldingOverLand (HydraulicErosion.kt:469-487).
void shielding_over_land(const float* density, const u8* is_land, int land_cells, size_t N, float* erod) {
    double summed = 0.0;
    for (size_t c = 0; c < N; ++c)
        if (is_land[c]) summed += (double)(1.0f - kVegetationShielding * density[c]);
    float mean = (float)(summed / land_cells);
    if (mean <= 0.0f) {
        for (size_t c = 0; c < N; ++c) erod[c] = 1.0f;
        return;
    }
    for (size_t c = 0; c < N; ++c) erod[c] = (1.0f - kVegetationShielding * density[c]) / mean;
}

// HydraulicErosion.baseLevel (HydraulicErosion.kt:2380-2390).
inline float base_level(int r, const float* surface, const u8* is_land, const float* water, float shoreline) {
    if (!is_land[r]) return shoreline;
    if (!std::isnan(water[r])) return std::max(surface[r], water[r]);
    return surface[r];
}

// HydraulicErosion.incise (HydraulicErosion.kt:2298-2371), without the watch and incisedAt.
void incise(const Rates& rates, int W, size_t N, const int32_t* order, int order_len, const int32_t* directions,
            const u8* is_land, const float* ground, const float* relative, const float* discharge, float land_cells,
            float land_range, float shoreline, const float* erodibility, float* surface, bool only_above_base,
            const float* unresolved) {
    std::vector<float> water(N, NAN);
    for (int rank = order_len - 1; rank >= 0; --rank) {
        int cell = order[rank];
        int r = directions[cell];
        bool under = ground[cell] - relative[cell] > rates.pond_depth;
        if (r < 0) {
            if (under) water[cell] = shoreline + ground[cell] * land_range;
            continue;
        }
        float base_after = base_level(r, surface, is_land, water.data(), shoreline);
        if (under) {
            float filled_level = shoreline + ground[cell] * land_range;
            float downstream = (is_land[r] && !std::isnan(water[r])) ? water[r] : base_after;
            water[cell] = std::min(filled_level, downstream);
        }
        float height = surface[cell];
        float step = rates.steps.between(cell, r, W);
        float courant = rates.courant_coefficient * std::sqrt(discharge[cell] / land_cells) * erodibility[cell] / step;
        float offset = 0.0f;
        if (unresolved)
            offset = unresolved[cell] - ((is_land[r] && std::isnan(water[r])) ? unresolved[r] : 0.0f);
        float grades_to = base_after + offset;
        bool submerged = under && height <= water[cell];
        float after;
        if (submerged || (height <= grades_to && only_above_base)) after = height;
        else after = (float)((double)grades_to + (double)(height - grades_to) / (1.0 + (double)courant));
        if (after != height) surface[cell] = after;
    }
}

// Math.min(float, float) on the JVM: NaN if either is, and -0 below +0.
inline float jvm_min(float a, float b) {
    if (a != a) return a;
    if (b != b) return b;
    if (a == 0.0f && b == 0.0f) return std::signbit(a) ? a : b;
    return a < b ? a : b;
}

// HydraulicErosion.raise (HydraulicErosion.kt:2535-2539): the change actually made, in double.
inline double raise(float* field, int cell, double amount) {
    float prior = field[cell];
    field[cell] = (float)((double)prior + amount);
    return (double)field[cell] - (double)prior;
}

struct Breached {
    double moved = 0.0;
    int cells = 0;
};

// HydraulicErosion.breach (HydraulicErosion.kt:1931-2171) as the rounds and the closing pass run it:
// belowSea false, no settled field and no load (nothing is carried in profile P1), and
// ErosionConfig's outletIncisionRatio 1.125 and outletFallToTheWater on. Basins are taken in the
// order spillways found them; `relative`, `ground` and `surface` are cut in place.
Breached breach(const Rates& rates, int W, const Spillways& notch, const u8* is_land, float* relative, float* ground,
                const int32_t* dirs, const float* area, float land_cells, float land_range, float* surface) {
    Breached out;
    const GroundSteps& steps = rates.steps;
    const float reach = (float)rates.outlet_reach_cells;   // Float < Int compares as floats
    const float gradient = rates.notch_fall_per_cell;
    auto take_down_to = [&](int cell, float cut_level) {
        double take = (double)(relative[cell] - cut_level) * (double)land_range;
        bool ponded = ground[cell] - relative[cell] > rates.pond_depth;
        double removed = -raise(surface, cell, -take);
        if (removed > 0.0) {
            float as_relative = (float)(removed / (double)land_range);
            relative[cell] -= as_relative;
            if (!ponded) ground[cell] -= as_relative;
            out.moved += removed;
            out.cells++;
        }
    };
    for (int b = 0; b < notch.count; ++b) {
        int spill = notch.spill[b];
        if (spill < 0) continue;
        float level = notch.level[b];
        float floor_ = notch.floor_[b];
        if (level - floor_ <= 0.0f) continue;
        // The channel's fall and length below the lip.
        float fall = 0.0f, length = 0.0f, last_step = steps.east_west;
        int walked = 0;
        int cell = spill;
        while (cell >= 0 && is_land[cell] && length < reach) {
            fall = level - relative[cell];
            if (fall > level - floor_) break;
            int next = dirs[cell];
            last_step = next >= 0 ? steps.between(cell, next, W) : steps.east_west;
            length += last_step;
            walked++;
            cell = next;
        }
        // A sill level to the water measures the step into it (FlowRouting.FLAT_GRADIENT_STEP 1e-6).
        if (fall <= 1e-6f * (float)walked && cell >= 0 && !is_land[cell]) {
            fall = level - relative[cell];
            length += last_step;
        }
        if (walked == 0) continue;
        float slope = fall / length * (float)W;
        if (slope < 0.0f) slope = 0.0f;
        float power = rates.relative_incision_coefficient * 1.125f * std::sqrt(area[spill] / land_cells) * slope;
        float drop = jvm_min(power, jvm_min(level - floor_, level));
        if (drop <= 0.0f) continue;
        float new_level = level - drop;
        // Down the channel from the lip, falling `gradient` a cell width, never below the shoreline.
        float from_lip = 0.0f;
        cell = spill;
        while (cell >= 0 && is_land[cell] && from_lip < reach) {
            float falling = new_level - from_lip * gradient;
            float cut_level = falling < 0.0f ? 0.0f : falling;
            if (relative[cell] <= cut_level) break;
            take_down_to(cell, cut_level);
            int next = dirs[cell];
            from_lip += next >= 0 ? steps.between(cell, next, W) : steps.east_west;
            cell = next;
        }
        // Back across the shallow margin, from the lip towards the entry, rising by the same gradient.
        int entry = notch.entry[b];
        if (entry >= 0 && entry != spill) {
            int margin_cells = 0;
            int walker = entry;
            float widths = 0.0f;
            while (walker >= 0 && walker != spill && is_land[walker] && widths <= reach) {
                int next = dirs[walker];
                widths += next >= 0 ? steps.between(walker, next, W) : steps.east_west;
                margin_cells++;
                walker = next;
            }
            if (walker == spill) {
                std::vector<int> margin(margin_cells);
                walker = entry;
                for (int i = 0; i < margin_cells; ++i) {
                    margin[i] = walker;
                    walker = dirs[walker];
                }
                float back = 0.0f;
                int downstream = spill;
                for (int i = margin_cells - 1; i >= 0; --i) {
                    int m = margin[i];
                    back += steps.between(m, downstream, W);
                    float cut_level = new_level + back * gradient;
                    if (relative[m] <= cut_level) break;
                    take_down_to(m, cut_level);
                    downstream = m;
                }
            }
        }
    }
    return out;
}

struct StageOut {
    std::vector<float> height;
    Cut cut;
    std::vector<float> filled, area;
    std::vector<int32_t> receivers, order;
    FlatCounts flats;
};

// ErosionStage.apply (ErosionStage.kt:133-183) with HydraulicErosion.apply (HydraulicErosion.kt:596-1506)
// for profiles P0 and P1: no provisional climate (the given weather is held), no belt replay, no
// flexure, no deposition; P1 adds the outlet notch (ErosionConfig.outletIncision): each round's breach
// before the incision (HydraulicErosion.kt:1002-1028) and the closing breach before the last
// relaxation (HydraulicErosion.kt:1404-1442). P1's routing outputs are the closing pass's, as its
// breach left them.
// run_rounds >= 0 stops after that many rounds (the relaxation keeps the whole stage's share per
// round) and initial = false leaves out the initial sweeps: a bounded sample of a stage.
int erode_stage(const cg_erosion_params& p, const cg_inputs& in, cg_outputs* out, cg_round_stats* stats,
                bool with_thermal = true, bool initial = true, int run_rounds = -1) {
    int W = p.width, H = p.height;
    size_t N = (size_t)W * H;
    Scale sc = scale_of(p);
    std::vector<float> working(in.height, in.height + N);
    if (!p.enabled) {
        std::memcpy(out->height, in.height, N * sizeof(float));
        return CG_OK;
    }
    cg_thermal_limits lim = thermal_limits(p);
    int sweeps = sweeps_for(p);
    // thermalErosion -> thermalSweep(skipSettled = true) (ErosionStage.kt:189-222).
    if (with_thermal && initial && sweeps > 0)
        thermal_sweep(W, H, working.data(), working.data(), lim, sweeps, p.rate, true);
    int rounds_for_relax = p.hydraulic_rounds < 1 ? 1 : p.hydraulic_rounds;
    int per_round = sweeps / rounds_for_relax;
    if (per_round < 1) per_round = 1;

    if (p.hydraulic_rounds <= 0 || p.bedrock_erodibility_per_year <= 0.0f) {
        std::memcpy(out->height, working.data(), N * sizeof(float));
        return CG_OK;
    }
    Rates rates(p);
    double r = sc.cell_height_km(H) / sc.cell_width_km(W);   // cellHeightInCellWidths
    int lattice = smooth_field_lattice_columns(p.world_width_km);
    std::vector<float> ones(N, 1.0f), zeros(N, 0.0f);
    const float* rain = in.rainfall_mm ? in.rainfall_mm : ones.data();
    const float* veg = in.vegetation_density ? in.vegetation_density : zeros.data();
    std::vector<float> runoff(N), erod(N);
    float metres_per_field = sc.relief_span();
    float uplift_per_mm = (float)(sc.years_per_round / 1000.0);   // MILLIMETRES_PER_METRE

    Cut cut;
    std::vector<float> filled(N), area(N);
    std::vector<int32_t> dirs(N), order;
    FlatCounts flats;
    bool routed = true;
    const int last = run_rounds >= 0 && run_rounds < p.hydraulic_rounds ? run_rounds : p.hydraulic_rounds;
    for (int round = 0; round < last; ++round) {
        if (in.uplift_mm_per_year) {
            const float* rate = in.uplift_mm_per_year;
            for (size_t c = 0; c < N; ++c) {
                if (rate[c] <= 0.0f) continue;
                float metres = rate[c] * uplift_per_mm;
                working[c] += metres / metres_per_field;
            }
        }
        percentile_cut(W, H, working.data(), p.sea_level, sc, stand_below_today(p, round), cut);
        if (cut.land_cells == 0) {
            std::memcpy(out->height, working.data(), N * sizeof(float));
            return CG_OK;
        }
        normalise_over_land(rain, cut.is_land.data(), cut.land_cells, N, runoff.data());
        if (p.shield_cut) shielding_over_land(veg, cut.is_land.data(), cut.land_cells, N, erod.data());
        else std::fill(erod.begin(), erod.end(), 1.0f);
        if (in.rock_erodibility)
            for (size_t c = 0; c < N; ++c) erod[c] *= in.rock_erodibility[c];
        fill_depressions(W, H, cut.is_land.data(), cut.relative.data(), filled.data());
        flow_directions(W, H, cut.is_land.data(), cut.relative.data(), filled.data(), p.seed, r, lattice,
                        p.facet_routing != 0, p.flat_potential != 0, dirs.data(), nullptr, &flats);
        accumulate(W, H, cut.is_land.data(), dirs.data(), cut.land_cells, runoff.data(), area.data());
        order.assign(cut.land_cells, 0);
        drainage_order(W, H, cut.is_land.data(), dirs.data(), cut.land_cells, order.data());
        float land_cells = (float)cut.land_cells;
        float land_range = std::max(sc.land_half(), 1e-6f);
        if (p.profile == CG_PROFILE_P1) {
            Spillways notch;
            spillways(W, H, cut.is_land.data(), cut.relative.data(), filled.data(), dirs.data(), rates.pond_depth,
                      notch, nullptr);
            breach(rates, W, notch, cut.is_land.data(), cut.relative.data(), filled.data(), dirs.data(), area.data(),
                   land_cells, land_range, working.data());
        }
        incise(rates, W, N, order.data(), cut.land_cells, dirs.data(), cut.is_land.data(), filled.data(),
               cut.relative.data(), area.data(), land_cells, land_range, cut.shoreline, erod.data(), working.data(),
               p.receiver_clamp != 0, nullptr);
        if (stats) {
            cg_round_stats& s = stats[round];
            std::memset(&s, 0, sizeof(s));
            s.round = round;
            s.land_cells = cut.land_cells;
            s.shoreline = cut.shoreline;
            s.flats = flats.flats;
            s.flats_kept = flats.kept;
            s.raised_cells = flats.raised;
        }
        if (p.profile == CG_PROFILE_P1 && round == p.hydraulic_rounds - 1) {
            // The closing breach over the finished surface: a fresh cut at today's shoreline, its own
            // fill, routing and discharge, then one more notch.
            Cut after;
            percentile_cut(W, H, working.data(), p.sea_level, sc, 0.0f, after);
            if (after.land_cells == 0) {
                routed = false;
            } else {
                fill_depressions(W, H, after.is_land.data(), after.relative.data(), filled.data());
                FlatCounts closing_flats;
                flow_directions(W, H, after.is_land.data(), after.relative.data(), filled.data(), p.seed, r, lattice,
                                p.facet_routing != 0, p.flat_potential != 0, dirs.data(), nullptr, &closing_flats);
                normalise_over_land(rain, after.is_land.data(), after.land_cells, N, runoff.data());
                accumulate(W, H, after.is_land.data(), dirs.data(), after.land_cells, runoff.data(), area.data());
                Spillways notch;
                spillways(W, H, after.is_land.data(), after.relative.data(), filled.data(), dirs.data(),
                          rates.pond_depth, notch, nullptr);
                breach(rates, W, notch, after.is_land.data(), after.relative.data(), filled.data(), dirs.data(),
                       area.data(), (float)after.land_cells, land_range, working.data());
                order.assign(after.land_cells, 0);
                drainage_order(W, H, after.is_land.data(), dirs.data(), after.land_cells, order.data());
                cut = std::move(after);
            }
        }
        // relax = thermalErosion(config, field, accelerator, sweepsPerRound) (ErosionStage.kt:178-180).
        if (with_thermal) thermal_sweep(W, H, working.data(), working.data(), lim, per_round, p.rate, true);
    }
    std::memcpy(out->height, working.data(), N * sizeof(float));
    if (!routed) return CG_OK;
    if (out->receivers) std::memcpy(out->receivers, dirs.data(), N * sizeof(int32_t));
    if (out->area) std::memcpy(out->area, area.data(), N * sizeof(float));
    if (out->filled) std::memcpy(out->filled, filled.data(), N * sizeof(float));
    if (out->relative) std::memcpy(out->relative, cut.relative.data(), N * sizeof(float));
    if (out->is_land) std::memcpy(out->is_land, cut.is_land.data(), N);
    if (out->order) {
        for (size_t c = 0; c < N; ++c) out->order[c] = -1;
        std::memcpy(out->order, order.data(), order.size() * sizeof(int32_t));
    }
    if (out->donors) {
        for (size_t c = 0; c < N; ++c) out->donors[c] = 0;
        for (size_t c = 0; c < N; ++c) {
            if (!cut.is_land[c]) continue;
            int rr = dirs[c];
            if (rr >= 0 && cut.is_land[rr]) out->donors[rr]++;
        }
    }
    if (out->basin_of_cell || out->basins) {
        Spillways sw;
        spillways(W, H, cut.is_land.data(), cut.relative.data(), filled.data(), dirs.data(), rates.pond_depth, sw,
                  out->basin_of_cell);
        if (out->basins) {
            cg_basins* b = out->basins;
            b->count = sw.count;
            int n = std::min(sw.count, b->capacity);
            for (int i = 0; i < n; ++i) {
                if (b->spill) b->spill[i] = sw.spill[i];
                if (b->entry) b->entry[i] = sw.entry[i];
                if (b->level) b->level[i] = sw.level[i];
                if (b->floor) b->floor[i] = sw.floor_[i];
                if (b->cells) b->cells[i] = sw.cells[i];
            }
            b->largest = sw.largest;
            b->largest_cells = sw.largest_cells;
            b->largest_depth = sw.largest_depth;
            b->deepest = sw.deepest;
        }
    }
    return CG_OK;
}

}  // namespace

// ================================================================ C entry points (ctypes)

extern "C" {

void or_default_params(cg_erosion_params* p, int32_t width, int32_t height, int64_t seed) {
    std::memset(p, 0, sizeof(*p));
    p->abi_version = CG_ABI_VERSION;
    p->width = width;
    p->height = height;
    p->mode = CG_MODE_REF32;
    p->seed = seed;
    p->world_width_km = 40075.0;
    p->highest_land_metres = 6000.0f;
    p->deepest_ocean_metres = 10000.0f;
    p->years_per_hydraulic_round = 336476.4;
    p->enabled = 1;
    p->critical_fall_metres_per_km = 60.0f;
    p->debris_travel_km = 1875.0;
    p->rate = 0.25f;
    p->hydraulic_rounds = 12;
    p->bedrock_erodibility_per_year = 1e-6f;
    p->facet_routing = 1;
    p->flat_potential = 1;
    p->sea_level = 0.71f;
    p->lowstand_metres = 120.0f;
    p->receiver_clamp = 1;
    p->shield_cut = 1;
    p->profile = CG_PROFILE_P0;
}

void or_thermal_limits(const cg_erosion_params* p, cg_thermal_limits* lim, int32_t* sweeps) {
    *lim = thermal_limits(*p);
    *sweeps = sweeps_for(*p);
}

void or_thermal_sweep(int32_t W, int32_t H, const float* in, float* out, float ew, float ns, float diag,
                      int32_t sweeps, float rate, int32_t skip) {
    cg_thermal_limits l{ew, ns, diag};
    thermal_sweep(W, H, in, out, l, sweeps, rate, skip != 0);
}

int32_t or_percentile_cut(int32_t W, int32_t H, const float* h, float sea_level, float highest_land,
                          float deepest_ocean, float lowstand_share, float* shoreline, uint8_t* is_land,
                          float* relative) {
    Scale sc{40075.0, highest_land, deepest_ocean, 336476.4};
    Cut cut;
    percentile_cut(W, H, h, sea_level, sc, lowstand_share, cut);
    *shoreline = cut.shoreline;
    std::memcpy(is_land, cut.is_land.data(), cut.is_land.size());
    std::memcpy(relative, cut.relative.data(), cut.relative.size() * sizeof(float));
    return cut.land_cells;
}

void or_fill_depressions(int32_t W, int32_t H, const uint8_t* is_land, const float* elev, float* filled) {
    fill_depressions(W, H, is_land, elev, filled);
}

void or_flow_directions(int32_t W, int32_t H, const uint8_t* is_land, const float* elev, const float* filled,
                        int64_t seed, double r, int32_t lattice, int32_t by_facet, int32_t over_potential,
                        int32_t* receivers, double* surface, int32_t* flat_counts) {
    std::vector<double> surf;
    FlatCounts fc;
    flow_directions(W, H, is_land, elev, filled, seed, r, lattice, by_facet != 0, over_potential != 0, receivers,
                    surface ? &surf : nullptr, &fc);
    if (surface) std::memcpy(surface, surf.data(), surf.size() * sizeof(double));
    if (flat_counts) {
        flat_counts[0] = fc.flats;
        flat_counts[1] = fc.kept;
        flat_counts[2] = fc.raised;
    }
}

void or_drainage_order(int32_t W, int32_t H, const uint8_t* is_land, const int32_t* target, int32_t land_cells,
                       int32_t* order) {
    drainage_order(W, H, is_land, target, land_cells, order);
}

void or_accumulate(int32_t W, int32_t H, const uint8_t* is_land, const int32_t* target, int32_t land_cells,
                   const float* weights, float* area) {
    accumulate(W, H, is_land, target, land_cells, weights, area);
}

int32_t or_spillways(int32_t W, int32_t H, const uint8_t* is_land, const float* elev, const float* filled,
                     const int32_t* target, float pond_depth, int32_t* basin_of_cell, cg_basins* basins) {
    Spillways sw;
    spillways(W, H, is_land, elev, filled, target, pond_depth, sw, basin_of_cell);
    if (basins) {
        basins->count = sw.count;
        int n = std::min(sw.count, basins->capacity);
        for (int i = 0; i < n; ++i) {
            if (basins->spill) basins->spill[i] = sw.spill[i];
            if (basins->entry) basins->entry[i] = sw.entry[i];
            if (basins->level) basins->level[i] = sw.level[i];
            if (basins->floor) basins->floor[i] = sw.floor_[i];
            if (basins->cells) basins->cells[i] = sw.cells[i];
        }
        basins->largest = sw.largest;
        basins->largest_cells = sw.largest_cells;
        basins->largest_depth = sw.largest_depth;
        basins->deepest = sw.deepest;
    }
    return sw.count;
}

// HydraulicErosion.incise on caller arrays; `rates` come from params.
void or_incise(const cg_erosion_params* p, const int32_t* order, int32_t order_len, const int32_t* directions,
               const uint8_t* is_land, const float* ground, const float* relative, const float* discharge,
               float land_cells, float land_range, float shoreline, const float* erodibility, float* surface,
               int32_t only_above_base, const float* unresolved) {
    Rates rates(*p);
    incise(rates, p->width, (size_t)p->width * p->height, order, order_len, directions, is_land, ground, relative,
           discharge, land_cells, land_range, shoreline, erodibility, surface, only_above_base != 0, unresolved);
}

// HydraulicErosion.breach over the basins FlowRouting.spillways finds on the given routing; relative,
// ground and surface are cut in place. Returns the cells cut; *moved receives the amount taken.
int32_t or_breach(const cg_erosion_params* p, const uint8_t* is_land, float* relative, float* ground,
                  const int32_t* directions, const float* area, float land_cells, float land_range, float* surface,
                  double* moved) {
    Rates rates(*p);
    Spillways notch;
    spillways(p->width, p->height, is_land, relative, ground, directions, rates.pond_depth, notch, nullptr);
    Breached b = breach(rates, p->width, notch, is_land, relative, ground, directions, area, land_cells, land_range,
                        surface);
    if (moved) *moved = b.moved;
    return b.cells;
}

void or_outlet_rates(const cg_erosion_params* p, float* relative_incision_coefficient, float* notch_fall_per_cell,
                     int32_t* outlet_reach_cells) {
    Rates rates(*p);
    *relative_incision_coefficient = rates.relative_incision_coefficient;
    *notch_fall_per_cell = rates.notch_fall_per_cell;
    *outlet_reach_cells = rates.outlet_reach_cells;
}

void or_rates(const cg_erosion_params* p, float* incision_coefficient, float* courant_coefficient,
              float* pond_depth) {
    Rates rates(*p);
    *incision_coefficient = rates.incision_coefficient;
    *courant_coefficient = rates.courant_coefficient;
    *pond_depth = rates.pond_depth;
}

float or_stand_below_today(const cg_erosion_params* p, int32_t round) { return stand_below_today(*p, round); }

float or_seeded_noise(int32_t c, int32_t r, int64_t seed) { return seeded_noise(c, r, seed); }

float or_smooth_seeded_field(int32_t W, int32_t lattice, int32_t c, int32_t r, int64_t seed) {
    return smooth_seeded_field(W, lattice, c, r, seed);
}

int32_t or_erode_stage(const cg_erosion_params* p, const cg_inputs* in, cg_outputs* out, cg_round_stats* stats) {
    return erode_stage(*p, *in, out, stats);
}

// HydraulicErosion.apply(config, height, seaLevel) { it }: the rounds alone, with no initial sweeps
// and an identity relaxation, as the reference's incision tests drive it.
int32_t or_hydraulic_apply(const cg_erosion_params* p, const cg_inputs* in, cg_outputs* out,
                           cg_round_stats* stats) {
    return erode_stage(*p, *in, out, stats, false);
}

// The first `rounds` rounds of ErosionStage.apply from heights already swept (no initial sweeps),
// each with its relaxation: a bounded sample of the stage for timing.
int32_t or_stage_rounds(const cg_erosion_params* p, const cg_inputs* in, cg_outputs* out, int32_t rounds) {
    return erode_stage(*p, *in, out, nullptr, true, false, rounds);
}

}  // extern "C"
