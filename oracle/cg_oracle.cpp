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
#include <memory>
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
            const float* unresolved, double* incised_at = nullptr) {
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
        if (after != height) {
            surface[cell] = after;
            if (incised_at && after < height) incised_at[cell] = (double)height - (double)after;
        }
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
// belowSea false; `settled` and `load` given where sediment is carried (profile P2's rounds), and
// ErosionConfig's outletIncisionRatio 1.125 and outletFallToTheWater on. Basins are taken in the
// order spillways found them; `relative`, `ground` and `surface` are cut in place.
Breached breach(const Rates& rates, int W, const Spillways& notch, const u8* is_land, float* relative, float* ground,
                const int32_t* dirs, const float* area, float land_cells, float land_range, float* surface,
                float* settled = nullptr, double* load = nullptr, bool below_sea = false, int rows = 0) {
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
            if (settled) settled[cell] -= as_relative;
            if (load) load[cell] += removed;
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
        // Never below the basin's floor; inside the rounds never below the sea either (belowSea off).
        float drop = below_sea ? jvm_min(power, level - floor_) : jvm_min(power, jvm_min(level - floor_, level));
        if (drop <= 0.0f) continue;
        float new_level = level - drop;
        // Down the channel from the lip, falling `gradient` a cell width, never below the shoreline
        // (belowSea: down to wherever the falling surface goes).
        float from_lip = 0.0f;
        cell = spill;
        while (cell >= 0 && is_land[cell] && from_lip < reach) {
            float falling = new_level - from_lip * gradient;
            float cut_level = below_sea ? falling : (falling < 0.0f ? 0.0f : falling);
            if (relative[cell] <= cut_level) break;
            take_down_to(cell, cut_level);
            int next = dirs[cell];
            from_lip += next >= 0 ? steps.between(cell, next, W) : steps.east_west;
            cell = next;
        }
        // Back across the shallow margin, from the lip towards the entry, rising by the same gradient.
        int entry = notch.entry[b];
        float back = 0.0f;
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
        // belowSea: the sill on the basin's own side too (HydraulicErosion.kt:2099-2168), the same
        // surface continued back across the lake bed up the inflow of the largest catchment (ties to
        // the lower index), rising by the gradient, never leaving the water, within the reach.
        if (below_sea) {
            const int H = rows;
            int from = entry >= 0 ? entry : spill;
            while (back <= reach) {
                int best = -1;
                float best_area = -1.0f;
                for_each_neighbour(W, H, from % W, from / W, [&](int n, int, int) {
                    if (is_land[n] && dirs[n] == from && ground[n] - relative[n] > rates.pond_depth) {
                        float a = area[n];
                        bool ties = a == best_area && (best < 0 || n < best);
                        if (a > best_area || ties) {
                            best_area = a;
                            best = n;
                        }
                    }
                });
                if (best < 0) break;
                back += steps.between(best, from, W);
                if (back > reach) break;
                float cut_level = new_level + back * gradient;
                if (relative[best] <= cut_level) break;
                double take = (double)(relative[best] - cut_level) * (double)land_range;
                double taken = -raise(surface, best, -take);
                if (taken > 0.0) {
                    float as_relative = (float)(taken / (double)land_range);
                    relative[best] -= as_relative;
                    if (settled) settled[best] -= as_relative;
                    if (load) load[best] += taken;
                    out.moved += taken;
                    out.cells++;
                }
                from = best;
            }
        }
    }
    return out;
}

// ---------------------------------------------------------------- SeaLevelStage's drowned basins

// SeaLevelStage.landAndWaterAt (SeaLevelStage.kt:175-200): the cut at a given shoreline.
void land_and_water_at(int W, int H, const float* h, float shoreline, const Scale& sc, Cut& out) {
    const size_t N = (size_t)W * H;
    const float land_half = std::max(sc.land_half(), 1e-6f), sea_half = std::max(sc.sea_half(), 1e-6f);
    out.shoreline = shoreline;
    out.is_land.assign(N, 0);
    out.relative.assign(N, 0.0f);
    out.land_cells = 0;
    for (size_t c = 0; c < N; ++c) {
        if (h[c] >= shoreline) {
            out.is_land[c] = 1;
            out.land_cells++;
            out.relative[c] = (h[c] - shoreline) / land_half;
        } else {
            out.relative[c] = (h[c] - shoreline) / sea_half;
        }
    }
}

// SeaLevelStage.markUnreachableWaterAsLand (SeaLevelStage.kt:371-437): the water bodies (8-connected,
// found from ascending start cells by a stack), the largest the ocean (the first found of that size);
// every other body no larger than the largest lake Earth has becomes land at its own height.
void mark_unreachable_water_as_land(int W, int H, Cut& cut, const float* h, const Scale& sc, double km2_per_cell,
                                    double enclosed_max_share) {
    const size_t N = (size_t)W * H;
    const int water = (int)N - cut.land_cells;
    if (water == 0) return;
    std::vector<int> body_of(N, -1), frontier(water);
    std::vector<int> cells_in;
    int bodies = 0, ocean = -1, ocean_cells = 0;
    for (size_t start = 0; start < N; ++start) {
        if (cut.is_land[start] || body_of[start] >= 0) continue;
        const int body = bodies++;
        int fs = 0;
        body_of[start] = body;
        frontier[fs++] = (int)start;
        int found = 0;
        while (fs > 0) {
            const int c = frontier[--fs];
            found++;
            for_each_neighbour(W, H, c % W, c / W, [&](int n, int, int) {
                if (!cut.is_land[n] && body_of[n] < 0) {
                    body_of[n] = body;
                    frontier[fs++] = n;
                }
            });
        }
        cells_in.push_back(found);
        if (found > ocean_cells) {
            ocean_cells = found;
            ocean = body;
        }
    }
    if (bodies <= 1) return;
    const int largest_lake = (int)(enclosed_max_share * sc.world_area_km2() / km2_per_cell);
    const float land_half = std::max(sc.land_half(), 1e-6f);
    for (size_t c = 0; c < N; ++c) {
        const int body = body_of[c];
        if (body < 0 || body == ocean || cells_in[body] > largest_lake) continue;
        cut.is_land[c] = 1;
        cut.land_cells++;
        cut.relative[c] = (h[c] - cut.shoreline) / land_half;
    }
}

// SeaLevelStage.drainDrownedBasins (SeaLevelStage.kt:478-560): the outlet notch once more, belowSea,
// over only the basins whose floor lies below the shoreline, up to MAX_POST_CUT_OUTLET_PASSES times,
// each pass re-cut at the same shoreline with the enclosure rule. The terrain it cuts is a copy.
void drain_drowned_basins(const cg_erosion_params& p, Cut& current, const float* height, double enclosed_max_share,
                          int* passes_run) {
    const int W = p.width, H = p.height;
    const size_t N = (size_t)W * H;
    const Scale sc = scale_of(p);
    const float land_half = std::max(sc.land_half(), 1e-6f);
    const Rates rates(p);
    const double r = sc.cell_height_km(H) / sc.cell_width_km(W);
    const int lattice = smooth_field_lattice_columns(p.world_width_km);
    const double km2_per_cell = sc.cell_width_km(W) * sc.cell_height_km(H);
    std::vector<float> terrain;
    std::vector<float> ones(N, 1.0f), filled(N), area(N);
    std::vector<int32_t> dirs(N);
    *passes_run = 0;
    for (int pass = 0; pass < 16; ++pass) {   // SeaLevelStage.MAX_POST_CUT_OUTLET_PASSES
        if (current.land_cells == 0) return;
        std::vector<float> relative = current.relative;
        fill_depressions(W, H, current.is_land.data(), relative.data(), filled.data());
        FlatCounts fc;
        flow_directions(W, H, current.is_land.data(), relative.data(), filled.data(), p.seed, r, lattice,
                        p.facet_routing != 0, p.flat_potential != 0, dirs.data(), nullptr, &fc);
        accumulate(W, H, current.is_land.data(), dirs.data(), current.land_cells, ones.data(), area.data());
        Spillways sw;
        spillways(W, H, current.is_land.data(), relative.data(), filled.data(), dirs.data(), rates.pond_depth, sw,
                  nullptr);
        int drowned = 0;
        for (int b = 0; b < sw.count; ++b) {
            if (sw.floor_[b] >= 0.0f) sw.spill[b] = -1;
            else if (sw.spill[b] >= 0) drowned++;
        }
        if (drowned == 0) return;
        if (terrain.empty()) terrain.assign(height, height + N);
        *passes_run = pass + 1;
        Breached b = breach(rates, W, sw, current.is_land.data(), relative.data(), filled.data(), dirs.data(),
                            area.data(), (float)current.land_cells, land_half, terrain.data(), nullptr, nullptr, true, H);
        if (b.cells == 0) return;
        Cut next;
        land_and_water_at(W, H, terrain.data(), current.shoreline, sc, next);
        mark_unreachable_water_as_land(W, H, next, terrain.data(), sc, km2_per_cell, enclosed_max_share);
        current = std::move(next);
    }
}

// ---------------------------------------------------------------- deposition (profile P2)

// The switches the round tail reads (ErosionConfig, M:WorldGenConfig.kt:2068-2496) and the knobs of
// the deposition beside them. A profile sets the switches; tests may change the knobs.
struct Switches {
    bool outlet_incision = false;     // ErosionConfig.outletIncision
    bool deposition = false;          // ErosionConfig.deposition
    bool delta_lobe = false;          // ErosionConfig.deltaLobe (the closing mouths pass runs on it)
    bool delta_outline = false;       // ErosionConfig.deltaOutline: best-first outlined fans, else square ones
    bool graded_aggradation = false;  // ErosionConfig.gradedAggradation
    float transport_capacity = 20.0f;        // ErosionConfig.transportCapacity
    float deposition_rate = 0.06f;           // ErosionConfig.depositionRate
    float delta_share = 0.15f;               // ErosionConfig.deltaShare
    float lake_share = 0.1f;                 // ErosionConfig.lakeShare
    double delta_min_catchment_km2 = 70000.0;   // ErosionConfig.deltaMinCatchmentKm2
    double delta_reach_km = 140.625;         // ErosionConfig.deltaReachKm
    float delta_freeboard_metres = 48.0f;    // ErosionConfig.deltaFreeboardMetres
    bool flexure = false;             // IsostasyConfig.flexure (with IsostasyConfig.enabled)
};

// P0: the plain core; P1 adds the outlet notch; P2 adds deposition with the lobed, outlined and
// graded deltas.
Switches switches_of(const cg_erosion_params& p) {
    Switches s;
    s.outlet_incision = p.profile >= CG_PROFILE_P1;
    s.deposition = s.delta_lobe = s.delta_outline = s.graded_aggradation = p.profile >= CG_PROFILE_P2;
    s.flexure = p.profile >= CG_PROFILE_P3;
    return s;
}

const float kLobeRim = 0.15f;                       // HydraulicErosion.LOBE_RIM
const float kLobeSides = 0.38f;                     // HydraulicErosion.LOBE_SIDES
const float kLobeWobble = 0.18f;                    // HydraulicErosion.LOBE_WOBBLE
const float kDepthCost = 1.0f;                      // HydraulicErosion.DEPTH_COST
const float kGrooveKeep = 0.45f;                    // HydraulicErosion.GROOVE_KEEP
const float kLakeFanSlope = 1.5f;                   // HydraulicErosion.LAKE_FAN_SLOPE
const float kDistributaryFallPerKm = 0.15f / 23.4375f;   // HydraulicErosion.DISTRIBUTARY_FALL_PER_KM
const float kMinDistributaryFall = 1e-7f;           // HydraulicErosion.MIN_DISTRIBUTARY_FALL
const int kMouthKeyRowStride = 0x2000;              // HydraulicErosion.MOUTH_KEY_ROW_STRIDE
const double kDrawnRiverCatchmentKm2 = 70000.0 / 5; // HydraulicErosion.DRAWN_RIVER_CATCHMENT_KM2
const float kShelfBreakMetres = 130.0f;             // HydraulicErosion.SHELF_BREAK_METRES

// The deposition members of HydraulicErosion.Rates (HydraulicErosion.kt:285-300) and the stage's own
// cell counts (HydraulicErosion.kt:639-640, 1673-1674).
struct DepositionRates {
    float delta_freeboard;
    int delta_reach_cells;
    float shelf_break;
    float delta_min_cells;
    float drawn_river_cells;
    DepositionRates(const cg_erosion_params& p, const Switches& sw) {
        Scale s = scale_of(p);
        delta_freeboard = s.relief_share_of_metres(sw.delta_freeboard_metres);
        delta_reach_cells = whole_cells_for(p, sw.delta_reach_km, 1);
        shelf_break = s.field_share_of_metres(kShelfBreakMetres);
        double km2 = s.cell_width_km(p.width) * s.cell_height_km(p.height);   // squareKilometresPerCell
        delta_min_cells = (float)(sw.delta_min_catchment_km2 / km2);
        drawn_river_cells = (float)(kDrawnRiverCatchmentKm2 / km2);
    }
};

// Math.min(double, double) on the JVM.
inline double jvm_min(double a, double b) {
    if (a != a) return a;
    if (b != b) return b;
    if (a == 0.0 && b == 0.0) return std::signbit(a) ? a : b;
    return a < b ? a : b;
}

// HydraulicErosion.shortestX / DeltaFan.wrapDx: a column difference taken the short way round.
inline int shortest_x(int dx, int W) {
    if (dx > W / 2) return dx - W;
    if (dx < -W / 2) return dx + W;
    return dx;
}

// HydraulicErosion.wobble (HydraulicErosion.kt:1574-1581): Int arithmetic, wrapping.
inline float cell_wobble(int cell) {
    uint32_t bits = (uint32_t)cell * 0x9E3779B9u;
    bits ^= bits >> 15;
    bits *= 0x2c1b3c6du;
    bits ^= bits >> 12;
    return (float)((bits >> 8) & 0xFFFFu) / 65535.0f;
}

// HydraulicErosion.mouthKey (HydraulicErosion.kt:1567-1571).
inline int mouth_key(int apex, int reach_cells, int W) {
    int block = reach_cells < 1 ? 1 : reach_cells;
    return (apex / W / block) * kMouthKeyRowStride + (apex % W / block);
}

// HydraulicErosion.lobeLevel (HydraulicErosion.kt:1519-1527): a square lobe's surface `d` cells out.
inline float lobe_level(float apex_level, float shoreline, int reach_cells, int distance_cells) {
    float rim = shoreline + (apex_level - shoreline) * kLobeRim;
    return apex_level + (rim - apex_level) * (float)distance_cells / (float)(reach_cells + 1);
}

// HydraulicErosion.lobeReach (HydraulicErosion.kt:1539-1556): how far a square lobe may grow towards a cell.
int lobe_reach(int reach_cells, int apex, int cell, float out_x, float out_y, int W) {
    float co = (float)shortest_x(cell % W - apex % W, W);
    float ro = (float)(cell / W - apex / W);
    float distance = std::sqrt(co * co + ro * ro);
    float out_length = std::sqrt(out_x * out_x + out_y * out_y);
    float ahead = (distance <= 0.0f || out_length <= 0.0f) ? 1.0f : (co * out_x + ro * out_y) / (distance * out_length);
    float shape = kLobeSides + (1.0f - kLobeSides) * (ahead < 0.0f ? 0.0f : ahead);
    return (int)((float)reach_cells * (shape + kLobeWobble * cell_wobble(cell)));
}

// HydraulicErosion.fallToReceiver (HydraulicErosion.kt:2229-2230).
inline float fall_to_receiver(const float* ground, const u8* is_land, int cell, int receiver) {
    return ground[cell] - (is_land[receiver] ? ground[receiver] : 0.0f);
}

// HydraulicErosion.headroom (HydraulicErosion.kt:2400-2424).
float headroom(int W, int H, int cell, float drop, const int32_t* dirs, const float* settled, float grade,
               const GroundSteps& steps) {
    float room = 3.402823466e+38f;
    bool fed = false;
    for_each_neighbour(W, H, cell % W, cell / W, [&](int n, int, int) {
        if (dirs[n] != cell) return;
        fed = true;
        float step = steps.between(n, cell, W);
        float margin = settled[n] - settled[cell] - grade * step;
        if (margin < room) room = margin;
    });
    return fed ? room : drop - grade;
}

// DeltaFan.hash (DeltaFan.kt): SplitMix64-style mixing of the seed and a mouth's key, Long wrapping.
int32_t fan_hash(int64_t seed, int32_t index) {
    uint64_t mixed = (uint64_t)seed * (uint64_t)(-0x61c8864680b583ebLL) +
                     (uint64_t)(int64_t)index * (uint64_t)(-0x7ee3623a03d3c83fLL) + (uint64_t)0x5DE17A11;
    mixed = (mixed ^ (mixed >> 30)) * (uint64_t)(-0x40a7b892e31b1a47LL);
    mixed = (mixed ^ (mixed >> 27)) * (uint64_t)(-0x6b2fb644ecceee15LL);
    mixed = mixed ^ (mixed >> 31);
    return (int32_t)(uint32_t)(mixed >> 17);
}

// DeltaFan.draw: a number in 0..1 for (hash, slot), Int wrapping.
float fan_draw(int32_t hash, int slot) {
    uint32_t mixed = (uint32_t)hash + (uint32_t)slot * 0x9E3779B9u;
    mixed ^= mixed >> 15;
    mixed *= 0x2c1b3c6du;
    mixed ^= mixed >> 12;
    mixed *= 0x297a2d39u;
    mixed ^= mixed >> 15;
    return (float)((mixed >> 8) & 0xFFFFu) / 65535.0f;
}

const float kSideReachShare = 0.38f;   // DeltaFan.SIDE_REACH_SHARE
const float kFanWobble = 0.30f;        // DeltaFan.WOBBLE
const float kWobbleW2 = 1.0f, kWobbleW3 = 0.7f, kWobbleW5 = 0.5f, kWobbleW7 = 0.45f;
const float kWobbleTotalInverse = 1.0f / (kWobbleW2 + kWobbleW3 + kWobbleW5 + kWobbleW7);
const float kDistributarySpread = 1.1f;
const float kGrooveHalfWidthShare = 0.05f;
const int kGrooveMinReachCells = 4;
const float kMinGrooveHalfWidthCells = 0.55f;
const int kGrooveDrawSlot = 10;
const float kGrooveJitterShare = 0.8f;

// DeltaFan.Rim: a lobe's outline around its apex, its bearing, its wobble and its grooves.
struct Rim {
    int apex, width;
    float reach_cells;
    int apex_column, apex_row;
    float ahead_x = 0.0f, ahead_y = 0.0f;
    float ph2x, ph2y, ph3x, ph3y, ph5x, ph5y, ph7x, ph7y;
    int distributaries = 0, live = 0;
    float groove_x[5] = {0}, groove_y[5] = {0};
    float groove_half_width;
    GroundSteps steps;
    float row_scale;
    float wobble = kFanWobble;   // DeltaFan.Rim's wobble (DeltaFan.WOBBLE unless a caller sets it)

    static void phase(int32_t hash, int slot, float& x, float& y) {
        float hx = fan_draw(hash, slot * 2) * 2.0f - 1.0f;
        float hy = fan_draw(hash, slot * 2 + 1) * 2.0f - 1.0f;
        float len = std::sqrt(hx * hx + hy * hy);
        if (len < 1e-4f) {
            x = 1.0f;
            y = 0.0f;
        } else {
            x = hx / len;
            y = hy / len;
        }
    }

    Rim(int apex_, int width_, double r, float reach, float out_x, float out_y, int32_t hash, bool grooved)
        : apex(apex_), width(width_), reach_cells(reach), apex_column(apex_ % width_), apex_row(apex_ / width_),
          steps(r), row_scale((float)r) {
        groove_half_width = reach * kGrooveHalfWidthShare > kMinGrooveHalfWidthCells ? reach * kGrooveHalfWidthShare
                                                                                    : kMinGrooveHalfWidthCells;
        float out_down = out_y * row_scale;
        float out_length = std::sqrt(out_x * out_x + out_down * out_down);
        if (out_length > 0.0f) {
            ahead_x = out_x / out_length;
            ahead_y = out_down / out_length;
        }
        phase(hash, 1, ph2x, ph2y);
        phase(hash, 2, ph3x, ph3y);
        phase(hash, 3, ph5x, ph5y);
        phase(hash, 4, ph7x, ph7y);
        distributaries = (!grooved || reach < (float)kGrooveMinReachCells || out_length <= 0.0f)
                             ? 0
                             : 2 + (int)(((uint32_t)hash >> 3) & 3u);
        if (distributaries > 0) {
            int n = distributaries;
            float left_x = -ahead_y, left_y = ahead_x;
            float span = n > 1 ? 2.0f * kDistributarySpread / (float)(n - 1) : 0.0f;
            for (int g = 0; g < n; ++g) {
                float jitter = (fan_draw(hash, kGrooveDrawSlot + g) - 0.5f) * kGrooveJitterShare * span;
                float off_axis = n > 1 ? -kDistributarySpread + span * (float)g + jitter : jitter;
                float ray_x = ahead_x + left_x * off_axis;
                float ray_y = ahead_y + left_y * off_axis;
                float ray_length = std::sqrt(ray_x * ray_x + ray_y * ray_y);
                if (ray_length < 1e-6f) ray_length = 1e-6f;
                groove_x[g] = ray_x / ray_length;
                groove_y[g] = ray_y / ray_length;
            }
        }
        live = distributaries;
    }

    float radius(float column_offset, float row_offset, float distance) const {
        if (distance <= 0.0f) return reach_cells;
        float c1 = column_offset / distance, s1 = row_offset / distance;
        float ahead = c1 * ahead_x + s1 * ahead_y;
        float nose = kSideReachShare + (1.0f - kSideReachShare) * (ahead > 0.0f ? ahead : 0.0f);
        float c2 = c1 * c1 - s1 * s1, s2 = 2.0f * c1 * s1;
        float c3 = c2 * c1 - s2 * s1, s3 = s2 * c1 + c2 * s1;
        float c5 = c3 * c2 - s3 * s2, s5 = s3 * c2 + c3 * s2;
        float c7 = c5 * c2 - s5 * s2, s7 = s5 * c2 + c5 * s2;
        float term = (kWobbleW2 * (c2 * ph2x - s2 * ph2y) + kWobbleW3 * (c3 * ph3x - s3 * ph3y) +
                      kWobbleW5 * (c5 * ph5x - s5 * ph5y) + kWobbleW7 * (c7 * ph7x - s7 * ph7y)) *
                     kWobbleTotalInverse;
        return reach_cells * nose * (1.0f + wobble * term);
    }

    bool grooved(float column_offset, float row_offset) const {
        for (int g = 0; g < live; ++g) {
            if (column_offset * groove_x[g] + row_offset * groove_y[g] < 0.0f) continue;
            float across = column_offset * groove_y[g] - row_offset * groove_x[g];
            if (across > -groove_half_width && across < groove_half_width) return true;
        }
        return false;
    }

    template <class Open>
    void prune_grooves(int height, Open&& open) {
        int kept = 0;
        for (int g = 0; g < distributaries; ++g) {
            float rx = groove_x[g], ry = groove_y[g];
            float ray_reach = radius(rx, ry, 1.0f);
            bool blocked = false;
            float stride = std::min(1.0f, row_scale);
            float along = stride;
            while (along <= (float)(int)ray_reach) {
                int row = apex_row + (int)(ry * along / row_scale);
                if (row < 0 || row >= height) {
                    blocked = true;
                    break;
                }
                int column = (apex_column + (int)(rx * along)) % width;
                if (column < 0) column += width;
                if (!open(row * width + column)) {
                    blocked = true;
                    break;
                }
                along += stride;
            }
            if (blocked) continue;
            if (kept != g) {
                groove_x[kept] = groove_x[g];
                groove_y[kept] = groove_y[g];
            }
            kept++;
        }
        live = kept;
    }

    float column_offset(int cell) const { return (float)shortest_x(cell % width - apex_column, width); }
    float row_offset(int cell) const { return (float)(cell / width - apex_row) * row_scale; }
};

// DeltaFan.Scratch: the stamps, a binary min-heap on (key, cell) and the admitted list.
struct FanScratch {
    std::vector<int> stamp;
    int capacity;
    std::vector<int> cells;
    std::vector<float> keys, penalties;
    int size = 0;
    std::vector<int> admitted;
    int admitted_count = 0;
    int out_cell = -1;
    float out_penalty = 0.0f;

    FanScratch(size_t n, int reach_cells, double r) : stamp(n, 0) {
        int reach_rows = (int)std::ceil(reach_cells / r);
        capacity = std::max((2 * reach_cells + 1) * (2 * reach_rows + 1), 9);
        cells.assign(capacity, 0);
        keys.assign(capacity, 0.0f);
        penalties.assign(capacity, 0.0f);
        admitted.assign(capacity, 0);
    }
    bool less(int a, int b) const { return keys[a] < keys[b] || (keys[a] == keys[b] && cells[a] < cells[b]); }
    void swap_slots(int a, int b) {
        std::swap(cells[a], cells[b]);
        std::swap(keys[a], keys[b]);
        std::swap(penalties[a], penalties[b]);
    }
    void admit(int cell) {
        if (admitted_count < capacity) admitted[admitted_count++] = cell;
    }
    void push(int cell, float key, float penalty) {
        if (size >= capacity) return;
        int slot = size++;
        cells[slot] = cell;
        keys[slot] = key;
        penalties[slot] = penalty;
        while (slot > 0) {
            int parent = (slot - 1) / 2;
            if (!less(slot, parent)) break;
            swap_slots(slot, parent);
            slot = parent;
        }
    }
    bool pop() {
        if (size == 0) return false;
        out_cell = cells[0];
        out_penalty = penalties[0];
        size--;
        if (size > 0) {
            cells[0] = cells[size];
            keys[0] = keys[size];
            penalties[0] = penalties[size];
            int slot = 0;
            while (true) {
                int left = 2 * slot + 1;
                if (left >= size) break;
                int right = left + 1;
                int smaller = left;
                if (right < size && less(right, left)) smaller = right;
                if (!less(smaller, slot)) break;
                swap_slots(slot, smaller);
                slot = smaller;
            }
        }
        return true;
    }
};

// A cell a fan laid into: its settled height and sediment before, and what its settled height gained.
struct FanTouch {
    int cell;
    float settled_before, sediment_before, increment;
};

// raise() of a fan's deposit into one cell, its settled height following; recorded if asked.
inline double lay(float* sediment, float* settled, int cell, double amount, float to_relative,
                  std::vector<FanTouch>* touched) {
    if (touched) touched->push_back({cell, settled[cell], sediment[cell], 0.0f});
    double moved = raise(sediment, cell, amount);
    float increment = (float)(moved * (double)to_relative);
    settled[cell] += increment;
    if (touched) touched->back().increment = increment;
    return moved;
}

// growFan (DeltaFan.kt): best-first admission of cells inside the rim, distance bent by `advance`,
// then laying `budget` into the admitted cells nearest first, each up to `level_of` and no higher.
template <class Accepts, class Advance, class LevelOf>
double grow_fan(int W, int H, double budget, const Rim& rim, FanScratch& scratch, int id, const float* surface,
                float* sediment, float* settled, float to_relative, bool whole_cells,
                std::vector<FanTouch>* touched, Accepts&& accepts, Advance&& advance, LevelOf&& level_of) {
    int apex = rim.apex;
    if (budget <= 0.0 || !accepts(apex)) return 0.0;
    scratch.size = 0;
    scratch.admitted_count = 0;
    scratch.stamp[apex] = id;
    scratch.push(apex, 0.0f, 0.0f);
    while (scratch.pop()) {
        int cell = scratch.out_cell;
        float penalty = scratch.out_penalty;
        scratch.admit(cell);
        int column = cell % W, row = cell / W;
        for (int sy = -1; sy <= 1; ++sy) {
            int nr = row + sy;
            if (nr < 0 || nr >= H) continue;
            for (int sx = -1; sx <= 1; ++sx) {
                if (sx == 0 && sy == 0) continue;
                int nc = (column + sx) % W;
                if (nc < 0) nc += W;
                int n = nr * W + nc;
                if (scratch.stamp[n] == id || !accepts(n)) continue;
                float co = rim.column_offset(n), ro = rim.row_offset(n);
                float distance = std::sqrt(co * co + ro * ro);
                float step = rim.steps.of(sx, sy);
                float np = penalty + step * (advance(n) - 1.0f);
                float rim_here = rim.radius(co, ro, distance);
                if (distance + np > rim_here) continue;
                scratch.stamp[n] = id;
                scratch.push(n, distance + np, np);
            }
        }
    }
    int count = scratch.admitted_count;
    scratch.size = 0;
    for (int k = 0; k < count; ++k) {
        int cell = scratch.admitted[k];
        float co = rim.column_offset(cell), ro = rim.row_offset(cell);
        scratch.push(cell, std::sqrt(co * co + ro * ro), 0.0f);
    }
    double remaining = budget, laid = 0.0;
    while (remaining > 0.0 && scratch.pop()) {
        int cell = scratch.out_cell;
        float co = rim.column_offset(cell), ro = rim.row_offset(cell);
        float distance = std::sqrt(co * co + ro * ro);
        float fraction = distance / rim.reach_cells;
        if (fraction > 1.0f) fraction = 1.0f;
        double need = (double)level_of(cell, fraction) - (double)surface[cell] - (double)sediment[cell];
        if (need <= 0.0) continue;
        if (whole_cells && need > remaining) break;
        double moved = lay(sediment, settled, cell, need < remaining ? need : remaining, to_relative, touched);
        remaining -= moved;
        laid += moved;
    }
    return laid;
}

// HydraulicErosion.fan (HydraulicErosion.kt:2446-2525): the square fan, breadth-first from the mouth
// out to the reach, each cell built up to `level_of` and no higher, nearest first. The stamps are
// the stage's own array (ids only ever increase); the queue holds (2 reach + 1)^2 cells.
template <class Accepts, class LevelOf>
double square_fan(int W, int H, int start, double budget, int reach_cells, std::vector<int>& stamp, int id,
                  std::vector<int>& queue, std::vector<int>& distance_at, const float* surface, float* sediment,
                  float* settled, float to_relative, bool whole_cells, std::vector<FanTouch>* touched,
                  Accepts&& accepts, LevelOf&& level_of) {
    if (budget <= 0.0 || !accepts(start, 0)) return 0.0;
    double remaining = budget, laid = 0.0;
    int head = 0, tail = 0;
    queue[tail] = start;
    distance_at[tail] = 0;
    tail++;
    stamp[start] = id;
    while (head < tail && remaining > 0.0) {
        int cell = queue[head];
        int steps = distance_at[head];
        head++;
        double need = (double)level_of(cell, steps) - (double)surface[cell] - (double)sediment[cell];
        if (need > 0.0) {
            if (whole_cells && need > remaining) break;
            double moved = lay(sediment, settled, cell, need < remaining ? need : remaining, to_relative, touched);
            remaining -= moved;
            laid += moved;
        }
        if (steps >= reach_cells) continue;
        int column = cell % W, row = cell / W;
        for (int rs = -1; rs <= 1; ++rs) {
            int nr = row + rs;
            if (nr < 0 || nr >= H) continue;
            for (int cs = -1; cs <= 1; ++cs) {
                if (cs == 0 && rs == 0) continue;
                int nc = (column + cs) % W;
                if (nc < 0) nc += W;
                int n = nr * W + nc;
                if (stamp[n] == id || !accepts(n, steps + 1)) continue;
                stamp[n] = id;
                if (tail < (int)queue.size()) {
                    queue[tail] = n;
                    distance_at[tail] = steps + 1;
                    tail++;
                }
            }
        }
    }
    return laid;
}

// Scratch of the square fans (HydraulicErosion.kt:773-776): present where some fan is square.
struct SquareScratch {
    std::vector<int> stamp, queue, distance_at;
    SquareScratch(size_t n, int reach_cells)
        : stamp(n, 0), queue((size_t)(2 * reach_cells + 1) * (2 * reach_cells + 1)),
          distance_at((size_t)(2 * reach_cells + 1) * (2 * reach_cells + 1)) {}
};

// One round's deposition walk captured for tests of the device's walk: its inputs just before the
// walk and the fields it changed just after (the reference's order).
struct WalkCapture {
    int round = -1;
    bool taken = false;
    std::vector<int32_t> order, dirs;
    std::vector<u8> land;
    std::vector<float> ground, relative, area, surface, sediment, settled;
    std::vector<double> load, incised_at;
    float land_cells = 0, land_range = 0, to_relative = 0, shoreline = 0;
    int mouth_id = 0;
    std::vector<float> sediment_after, settled_after;
    std::vector<double> load_after;
};

struct Tally {   // one round's mass budget (RoundMass, HydraulicErosion.kt:1477-1484)
    double incised = 0.0, deposited = 0.0, lost = 0.0, field_drop = 0.0;
};

// The deposition walk (HydraulicErosion.kt:1068-1349) over one round's drainage order, sources first:
// each cell picks up what the incision took off it, settles any surplus over the flow's capacity on a
// floodplain (never above the ground that feeds it), and hands the rest on; at the sea a river's
// share builds a lobe, at a lake a share builds a fan. The walk's two halves are kept apart (a cell's
// own walk, then its mouth) so that the level schedule below can reorder them.
struct DepositionWalk {
    enum { OFF_MAP = -1, ON = 0, SEA = 1, LAKE = 2 };
    const cg_erosion_params& p;
    const Switches& sw;
    const Rates& rates;
    const int32_t* dirs;
    const u8* is_land;
    const float *ground, *relative, *area;
    float land_cells, land_range, to_relative, shoreline;
    float *surface, *sediment, *settled;
    const double* incised_at;
    FanScratch* scratch;
    SquareScratch* square;
    int& mouth_id;
    Tally& t;
    int W, H, reach_cells;
    double r;
    float delta_top, rim_top, shelf_depth, delta_min_cells;
    // Fan deposits of the current mouth as (cell, settled increment), when a caller wants them.
    std::vector<FanTouch>* touched = nullptr;

    DepositionWalk(const cg_erosion_params& p_, const Switches& sw_, const DepositionRates& dr, const Rates& rates_,
                   const int32_t* dirs_, const u8* is_land_, const float* ground_, const float* relative_,
                   const float* area_, float land_cells_, float land_range_, float to_relative_, float shoreline_,
                   float* surface_, float* sediment_, float* settled_, const double* incised_at_, FanScratch* scratch_,
                   SquareScratch* square_, int& mouth_id_, Tally& t_)
        : p(p_), sw(sw_), rates(rates_), dirs(dirs_), is_land(is_land_), ground(ground_), relative(relative_),
          area(area_), land_cells(land_cells_), land_range(land_range_), to_relative(to_relative_),
          shoreline(shoreline_), surface(surface_), sediment(sediment_), settled(settled_), incised_at(incised_at_),
          scratch(scratch_), square(square_), mouth_id(mouth_id_), t(t_) {
        W = p.width;
        H = p.height;
        r = scale_of(p).cell_height_km(H) / scale_of(p).cell_width_km(W);
        reach_cells = dr.delta_reach_cells < 0 ? 0 : dr.delta_reach_cells;
        delta_top = shoreline + dr.delta_freeboard * land_range;
        rim_top = shoreline + (delta_top - shoreline) * kLobeRim;
        shelf_depth = dr.shelf_break < 1e-9f ? 1e-9f : dr.shelf_break;
        delta_min_cells = dr.delta_min_cells;
    }

    bool ponded(int c) const { return ground[c] - relative[c] > rates.pond_depth; }

    // A cell's own walk (HydraulicErosion.kt:1068-1186), `carried` arriving: returns what it carries on
    // and where it goes. *used_headroom (if given) says whether it read its donors' settled heights.
    int own(int cell, double& carried, bool* used_headroom = nullptr) {
        int receiver = dirs[cell];
        if (used_headroom) *used_headroom = false;
        if (receiver < 0) return OFF_MAP;
        bool to_sea = !is_land[receiver];
        float drop = fall_to_receiver(ground, is_land, cell, receiver);
        bool wet = ponded(cell);
        float distance = rates.steps.between(cell, receiver, W);
        float slope = drop > 0.0f ? drop / distance * (float)W : 0.0f;
        double capacity = (double)(sw.transport_capacity * std::sqrt(area[cell] / land_cells) * slope);
        double moved = incised_at[cell];
        if (moved > 0.0) {
            settled[cell] -= (float)(moved * (double)to_relative);
            carried += moved;
            t.incised += moved;
        }
        if (!wet && carried > capacity) {
            float grade = 0.0f;
            if (sw.graded_aggradation) {
                double conveyance = (double)(sw.transport_capacity * std::sqrt(area[cell] / land_cells));
                grade = conveyance > 1e-12 ? (float)(carried / conveyance / (double)W) : 0.0f;
            }
            if (used_headroom) *used_headroom = true;
            float room = headroom(W, H, cell, drop, dirs, settled, grade, rates.steps) * land_range;
            double give = jvm_min(carried - capacity, (double)room) * (double)sw.deposition_rate;
            if (give > 0.0) {
                double laid = raise(sediment, cell, give);
                settled[cell] += (float)(laid * (double)to_relative);
                carried -= laid;
                t.deposited += laid;
            }
        }
        if (to_sea) return SEA;
        if (!wet && ponded(receiver)) return LAKE;
        return ON;
    }

    // A cell's mouth (HydraulicErosion.kt:1187-1349): the lobe at the sea or the fan in a lake. Returns
    // what it laid; the caller hands the rest on (lake) or counts it lost (sea).
    double mouth(int cell, double carried, int kind) {
        int receiver = dirs[cell];
        float out_x = (float)shortest_x(receiver % W - cell % W, W);
        float out_y = (float)(receiver / W - cell / W);
        double laid;
        if (kind == SEA) {
            bool river = area[cell] >= delta_min_cells;
            double budget = river ? carried * (double)sw.delta_share : 0.0;
            if (!(sw.delta_lobe && sw.delta_outline)) {
                // The square lobe, or with the lobe off the flat slab (HydraulicErosion.kt:1230-1253).
                laid = square_fan(
                    W, H, receiver, budget, reach_cells, square->stamp, ++mouth_id, square->queue, square->distance_at,
                    surface, sediment, settled, to_relative, sw.delta_lobe, touched,
                    [&](int c, int steps) {
                        return !is_land[c] &&
                               (!sw.delta_lobe || steps <= lobe_reach(reach_cells, receiver, c, out_x, out_y, W));
                    },
                    [&](int, int steps) {
                        return sw.delta_lobe ? lobe_level(delta_top, shoreline, reach_cells, steps) : delta_top;
                    });
            } else {
                Rim rim(receiver, W, r, (float)reach_cells, out_x, out_y,
                        fan_hash(p.seed, mouth_key(receiver, reach_cells, W)), true);
                rim.prune_grooves(H, [&](int c) { return !is_land[c]; });
                laid = grow_fan(
                    W, H, budget, rim, *scratch, ++mouth_id, surface, sediment, settled, to_relative, true, touched,
                    [&](int c) { return !is_land[c]; },
                    [&](int c) {
                        float depth = shoreline - (surface[c] + sediment[c]);
                        return 1.0f + kDepthCost * (depth > 0.0f ? depth : 0.0f) / shelf_depth;
                    },
                    [&](int c, float fraction) {
                        float level = delta_top + (rim_top - delta_top) * fraction;
                        if (rim.grooved(rim.column_offset(c), rim.row_offset(c)))
                            return shoreline + (level - shoreline) * kGrooveKeep;
                        return level;
                    });
            }
            t.deposited += laid;
            t.lost += carried - laid;
            return laid;
        }
        if (!sw.delta_outline) {   // the square lake fan (HydraulicErosion.kt:1321-1344)
            laid = square_fan(
                W, H, receiver, carried * (double)sw.lake_share, reach_cells, square->stamp, ++mouth_id,
                square->queue, square->distance_at, surface, sediment, settled, to_relative, false, touched,
                [&](int c, int) { return is_land[c] && ponded(c); },
                [&](int c, int steps) {
                    float depth = 2.0f * rates.pond_depth *
                                  (1.0f + kLakeFanSlope * (float)steps / (float)(reach_cells < 1 ? 1 : reach_cells)) *
                                  (0.9f + 0.35f * cell_wobble(c));
                    return shoreline + (ground[c] - depth) * land_range;
                });
        } else {
            Rim rim(receiver, W, r, (float)reach_cells, out_x, out_y,
                    fan_hash(p.seed, mouth_key(receiver, reach_cells, W)), false);
            laid = grow_fan(
                W, H, carried * (double)sw.lake_share, rim, *scratch, ++mouth_id, surface, sediment, settled,
                to_relative, false, touched,
                [&](int c) { return is_land[c] && ponded(c); },
                [&](int c) {
                    float depth = (ground[c] - relative[c]) * land_range;
                    return 1.0f + kDepthCost * (depth > 0.0f ? depth : 0.0f) / shelf_depth;
                },
                [&](int c, float fraction) {
                    float depth = 2.0f * rates.pond_depth * (1.0f + kLakeFanSlope * fraction) *
                                  (0.9f + 0.35f * cell_wobble(c));
                    return shoreline + (ground[c] - depth) * land_range;
                });
        }
        t.deposited += laid;
        return laid;
    }

    // The reference's order: one cell after another, load[] gathering each hand-off as it is made.
    void run(const int32_t* order, int order_len, double* load) {
        for (int rank = 0; rank < order_len; ++rank) {
            int cell = order[rank];
            double carried = load[cell];
            int kind = own(cell, carried);
            if (kind == OFF_MAP) t.lost += carried;   // off the polar edge, with whatever it carries
            else if (kind == SEA) mouth(cell, carried, kind);
            else if (kind == LAKE) load[dirs[cell]] += carried - mouth(cell, carried, kind);
            else load[dirs[cell]] += carried;
        }
    }
};

// How often the level schedule had to repair a level (see run_levels).
struct LevelRepairs {
    long replayed = 0;   // ponded cells of a fan's own level, ranked after it, whose settled height was replayed
    long redone = 0;     // levels restored and walked again one cell after another
};

// The same walk in the order a device runs it, to show that this order gives the reference's bits.
// The Kahn order is level-major, so the walk goes level by level from the sources. In a level every
// cell first does its own walk (cells of one level never read one another: a cell reads its own state
// and its donors', which are lower), its load being its notch hand-off plus its donors' hand-offs in
// rank order, the reference's additions in the reference's order. Then the level's mouths run in rank
// order. A fan changes only sea cells and ponded land cells, which no own walk reads, except (a) a
// ponded cell of the fan's level ranked after it, whose settled height took its own subtraction before
// the fan's addition instead of after: replayed in rank order; and (b) a donor whose settled height a
// later cell of the level read in its headroom: the level is restored and walked one cell after another.
void run_levels(DepositionWalk& w, const int32_t* order, int order_len, const double* notch_load, size_t N,
                LevelRepairs& repairs) {
    const int32_t* dirs = w.dirs;
    const u8* land = w.is_land;
    std::vector<int> level(N, -1), rank_of(N, -1);
    for (int k = 0; k < order_len; ++k) {
        level[order[k]] = 0;
        rank_of[order[k]] = k;
    }
    for (int k = 0; k < order_len; ++k) {
        int c = order[k], rr = dirs[c];
        if (rr >= 0 && land[rr]) level[rr] = std::max(level[rr], level[c] + 1);
    }
    std::vector<int> dstart(N + 1, 0), donors;   // donors in rank order
    for (int k = 0; k < order_len; ++k) {
        int rr = dirs[order[k]];
        if (rr >= 0 && land[rr]) dstart[rr + 1]++;
    }
    for (size_t c = 0; c < N; ++c) dstart[c + 1] += dstart[c];
    donors.resize(dstart[N]);
    {
        std::vector<int> next(dstart.begin(), dstart.end() - 1);
        for (int k = 0; k < order_len; ++k) {
            int c = order[k], rr = dirs[c];
            if (rr >= 0 && land[rr]) donors[next[rr]++] = c;
        }
    }
    std::vector<double> handoff(N, 0.0);
    std::vector<char> used(N, 0);
    auto arriving = [&](int c) {
        double carried = notch_load[c];
        for (int k = dstart[c]; k < dstart[c + 1]; ++k) carried += handoff[donors[k]];
        return carried;
    };
    auto walk_one = [&](int c) {   // a cell's whole step, the reference's way
        double carried = arriving(c);
        int kind = w.own(c, carried);
        if (kind == DepositionWalk::OFF_MAP) w.t.lost += carried;
        else if (kind == DepositionWalk::SEA) w.mouth(c, carried, kind);
        else if (kind == DepositionWalk::LAKE) handoff[c] = carried - w.mouth(c, carried, kind);
        else handoff[c] = carried;
    };
    struct Event {
        int rank, cell, kind;
        double carried;
        std::vector<FanTouch> touched;
    };
    int lo = 0;
    while (lo < order_len) {
        const int L = level[order[lo]];
        int hi = lo;
        while (hi < order_len && level[order[hi]] == L) ++hi;
        const Tally t0 = w.t;
        std::vector<float> settled0(hi - lo), sediment0(hi - lo);
        for (int k = lo; k < hi; ++k) {
            settled0[k - lo] = w.settled[order[k]];
            sediment0[k - lo] = w.sediment[order[k]];
        }
        std::vector<Event> events;
        for (int k = lo; k < hi; ++k) {   // every own walk of the level, as if at once
            int c = order[k];
            double carried = arriving(c);
            bool used_headroom = false;
            int kind = w.own(c, carried, &used_headroom);
            used[c] = used_headroom;
            if (kind == DepositionWalk::OFF_MAP) w.t.lost += carried;
            else if (kind == DepositionWalk::ON) handoff[c] = carried;
            else events.push_back({k, c, kind, carried, {}});
        }
        for (Event& e : events) {   // the mouths, in rank order
            w.touched = &e.touched;
            double laid = w.mouth(e.cell, e.carried, e.kind);
            w.touched = nullptr;
            if (e.kind == DepositionWalk::LAKE) handoff[e.cell] = e.carried - laid;
        }
        bool redo = false;
        std::vector<int> replay;
        for (const Event& e : events)
            for (const FanTouch& f : e.touched) {
                int x = f.cell;
                if (!land[x]) continue;
                if (level[x] == L && rank_of[x] > e.rank) replay.push_back(x);
                int rr = dirs[x];
                if (rr >= 0 && land[rr] && level[rr] == L && rank_of[rr] > e.rank && used[rr]) redo = true;
            }
        if (redo) {
            repairs.redone++;
            for (auto e = events.rbegin(); e != events.rend(); ++e)
                for (auto f = e->touched.rbegin(); f != e->touched.rend(); ++f) {
                    w.settled[f->cell] = f->settled_before;
                    w.sediment[f->cell] = f->sediment_before;
                }
            for (int k = lo; k < hi; ++k) {
                w.settled[order[k]] = settled0[k - lo];
                w.sediment[order[k]] = sediment0[k - lo];
            }
            w.t = t0;
            for (int k = lo; k < hi; ++k) walk_one(order[k]);
        } else if (!replay.empty()) {
            std::sort(replay.begin(), replay.end());
            replay.erase(std::unique(replay.begin(), replay.end()), replay.end());
            for (int x : replay) {
                repairs.replayed++;
                // The cell's own subtraction and the fans' increments, in rank order.
                std::vector<std::pair<int, float>> ops;   // (rank, increment); the own op marked by rank_of[x]
                for (const Event& e : events)
                    for (const FanTouch& f : e.touched)
                        if (f.cell == x) ops.push_back({e.rank, f.increment});
                float v = settled0[rank_of[x] - lo];
                bool own_done = false;
                auto own_op = [&]() {
                    double moved = w.incised_at[x];
                    if (moved > 0.0) v -= (float)(moved * (double)w.to_relative);
                    own_done = true;
                };
                for (const auto& op : ops) {
                    if (!own_done && op.first > rank_of[x]) own_op();
                    v += op.second;
                }
                if (!own_done) own_op();
                w.settled[x] = v;
            }
        }
        lo = hi;
    }
}

// HydraulicErosion.openMouths (HydraulicErosion.kt:1804-1892): a fresh cut, fill, routing and
// discharge over the finished surface, then each drawn river's path across raised ground (or its own
// fresh spoil) cut to a surface falling a fixed step a cell, receivers before their donors.
double open_mouths(const cg_erosion_params& p, float* working, const float* spoil, float pond_depth,
                   const float* rain, double r, int lattice, const DepositionRates& dr) {
    const int W = p.width, H = p.height;
    const size_t N = (size_t)W * H;
    Scale sc = scale_of(p);
    Cut sea;
    percentile_cut(W, H, working, p.sea_level, sc, 0.0f, sea);
    if (sea.land_cells == 0) return 0.0;
    const float land_range = std::max(sc.land_half(), 1e-6f);
    const float step = pond_depth * land_range;
    const float fall_per_cell_width = step * kDistributaryFallPerKm * (float)sc.cell_width_km(W);
    GroundSteps steps(r);
    const float floor_ = sea.shoreline + step * kLobeRim;
    std::vector<float> filled(N), runoff(N), area(N);
    std::vector<int32_t> flow(N);
    fill_depressions(W, H, sea.is_land.data(), sea.relative.data(), filled.data());
    FlatCounts fc;
    flow_directions(W, H, sea.is_land.data(), sea.relative.data(), filled.data(), p.seed, r, lattice,
                    p.facet_routing != 0, p.flat_potential != 0, flow.data(), nullptr, &fc);
    normalise_over_land(rain, sea.is_land.data(), sea.land_cells, N, runoff.data());
    accumulate(W, H, sea.is_land.data(), flow.data(), sea.land_cells, runoff.data(), area.data());
    std::vector<int32_t> order(sea.land_cells);
    drainage_order(W, H, sea.is_land.data(), flow.data(), sea.land_cells, order.data());
    double removed = 0.0;
    for (int rank = sea.land_cells - 1; rank >= 0; --rank) {
        int cell = order[rank];
        if (area[cell] < dr.drawn_river_cells) continue;
        float standing = filled[cell] - sea.relative[cell];
        bool on_flat = standing > 0.0f && (standing <= pond_depth || spoil[cell] > 0.0f);
        if (!on_flat) continue;
        int receiver = flow[cell];
        if (receiver < 0) continue;
        float below = sea.is_land[receiver] ? working[receiver] : sea.shoreline;
        float fall = fall_per_cell_width * steps.between(cell, receiver, W);
        if (fall < kMinDistributaryFall) fall = kMinDistributaryFall;
        float want = jvm_min(working[cell], below + fall);
        if (want < floor_) want = floor_;
        if (working[cell] > want) removed += -raise(working, cell, (double)(want - working[cell]));
    }
    return removed;
}

// ---------------------------------------------------------------- plate flexure (profile P3)

// Fft1D (math/Fft.kt:12-97): in-place radix-2 decimation in time over a strided line, twiddles
// tabulated once per length; `inverse` flips the sign of the twiddles' imaginary parts only.
struct Fft1D {
    int n;
    std::vector<double> cos_t, sin_t;
    explicit Fft1D(int length) : n(length), cos_t(length / 2), sin_t(length / 2) {
        for (int i = 0; i < length / 2; ++i) {
            cos_t[i] = std::cos(2.0 * M_PI * (double)i / (double)length);
            sin_t[i] = std::sin(2.0 * M_PI * (double)i / (double)length);
        }
    }
    void transform(double* re, double* im, size_t offset, size_t stride, bool inverse) const {
        int reversed = 0;
        for (int index = 1; index < n; ++index) {
            int bit = n >> 1;
            while (reversed & bit) {
                reversed ^= bit;
                bit >>= 1;
            }
            reversed |= bit;
            if (index < reversed) {
                const size_t a = offset + (size_t)index * stride, b = offset + (size_t)reversed * stride;
                std::swap(re[a], re[b]);
                std::swap(im[a], im[b]);
            }
        }
        for (int block = 2; block <= n; block <<= 1) {
            const int half = block >> 1, tw_stride = n / block;
            for (int start = 0; start < n; start += block)
                for (int pair = 0; pair < half; ++pair) {
                    const int t = pair * tw_stride;
                    const double wr = cos_t[t], wi = inverse ? sin_t[t] : -sin_t[t];
                    const size_t e = offset + (size_t)(start + pair) * stride;
                    const size_t o = offset + (size_t)(start + pair + half) * stride;
                    const double rr = re[o] * wr - im[o] * wi;
                    const double ri = re[o] * wi + im[o] * wr;
                    const double er = re[e], ei = im[e];
                    re[e] = er + rr;
                    im[e] = ei + ri;
                    re[o] = er - rr;
                    im[o] = ei - ri;
                }
        }
    }
};

// Fft2D (math/Fft.kt:99-152): every row, then every column; the inverse scaled by 1 / (width height).
struct Fft2D {
    int w, h;
    Fft1D rows, cols;
    Fft2D(int width, int height) : w(width), h(height), rows(width), cols(height) {}
    void run(double* re, double* im, bool inverse) const {
        for (int r = 0; r < h; ++r) rows.transform(re, im, (size_t)r * w, 1, inverse);
        for (int c = 0; c < w; ++c) cols.transform(re, im, (size_t)c, (size_t)w, inverse);
    }
    void forward(double* re, double* im) const { run(re, im, false); }
    void inverse(double* re, double* im) const {
        run(re, im, true);
        const double scale = 1.0 / ((double)w * (double)h);
        for (size_t c = 0; c < (size_t)w * h; ++c) {
            re[c] *= scale;
            im[c] *= scale;
        }
    }
};

// Isostasy.Flexure (Isostasy.kt:277-411): the plate's deflection under a load, a low-pass filter
// 1 / (dRho g + D k^4) over a grid mirrored about each pole to twice the map's height, the load's
// mean removed and the zero-frequency term left at zero.
struct Flexure {
    int W, H, rows2;
    double restoring, rigidity, per_cycle_across, per_cycle_down;
    Fft2D fft;
    std::vector<double> re, im;
    explicit Flexure(const cg_erosion_params& p)
        : W(p.width), H(p.height), rows2(p.height * 2), fft(p.width, p.height * 2),
          re((size_t)p.width * p.height * 2), im((size_t)p.width * p.height * 2) {
        const float metres_per_km = 1000.0f;
        restoring = (double)(p.mantle_density - p.deflection_fill_density) * (double)p.gravity;
        const double te = (double)p.elastic_thickness_km * (double)metres_per_km;
        const double e = (double)p.youngs_modulus_gpa * 1e9;
        const double nu = (double)p.poisson_ratio;
        rigidity = e * te * te * te / (12.0 * (1.0 - nu * nu));
        const Scale sc = scale_of(p);
        per_cycle_across = 2.0 * M_PI / ((double)W * sc.cell_width_km(W) * (double)metres_per_km);
        per_cycle_down = 2.0 * M_PI / ((double)rows2 * sc.cell_height_km(H) * (double)metres_per_km);
    }
    // deflectionMetres(load, out): `out` may be `load`.
    void deflection(const float* load, float* out) {
        const size_t cells = (size_t)W * H;
        double sum = 0.0;
        for (size_t c = 0; c < cells; ++c) sum += (double)load[c];
        const double mean = sum / (double)cells;
        for (int r = 0; r < H; ++r)
            for (int c = 0; c < W; ++c) {
                const double v = (double)load[(size_t)r * W + c] - mean;
                re[(size_t)r * W + c] = v;
                re[(size_t)(rows2 - 1 - r) * W + c] = v;
                im[(size_t)r * W + c] = 0.0;
                im[(size_t)(rows2 - 1 - r) * W + c] = 0.0;
            }
        fft.forward(re.data(), im.data());
        for (int r = 0; r < rows2; ++r) {
            const int cycles_down = r <= rows2 / 2 ? r : r - rows2;
            const double kd = (double)cycles_down * per_cycle_down;
            for (int c = 0; c < W; ++c) {
                const int cycles_across = c <= W / 2 ? c : c - W;
                const double ka = (double)cycles_across * per_cycle_across;
                const size_t i = (size_t)r * W + c;
                const double k2 = ka * ka + kd * kd;
                if (k2 == 0.0) {
                    re[i] = 0.0;
                    im[i] = 0.0;
                    continue;
                }
                const double response = 1.0 / (restoring + rigidity * k2 * k2);
                re[i] *= response;
                im[i] *= response;
            }
        }
        fft.inverse(re.data(), im.data());
        for (size_t c = 0; c < cells; ++c) out[c] = (float)re[c];
    }
};

struct StageOut {
    std::vector<float> height;
    Cut cut;
    std::vector<float> filled, area;
    std::vector<int32_t> receivers, order;
    FlatCounts flats;
};

// What BeltErosion.replay hands back (BeltReplay, P/BeltErosion.kt:35-47), erodedMeters aside.
struct BeltBooks {
    int rounds = 0, belt_cells = 0;
    double uplifted = 0.0, cut = 0.0, to_sea = 0.0, to_land = 0.0, shed = 0.0;
};

BeltBooks belt_replay(const cg_erosion_params& p, float* surface, const float* tectonic, const float* wear,
                      const float* onset, double window_myr, const float* uplift, const float* rain,
                      const float* cover, const float* rock, float provisional_sea_level, bool shield_cut,
                      const float* unresolved, bool rebounding, double history_cell_km, float* eroded);

// The belts' window for the stage's replay (ErosionTectonics.window), with IsostasyConfig.enabled and
// TectonicsConfig.historyCellKm.
struct BeltStage {
    const float* tectonic;
    const float* wear;
    const float* onset;
    double window_myr;
    bool rebound;
    double history_cell_km;
};

// ErosionStage.apply (ErosionStage.kt:133-183) with HydraulicErosion.apply (HydraulicErosion.kt:596-1506)
// for profiles P0 and P1: no provisional climate (the given weather is held), no flexure, no
// deposition; P1 adds the outlet notch (ErosionConfig.outletIncision): each round's breach
// before the incision (HydraulicErosion.kt:1002-1028) and the closing breach before the last
// relaxation (HydraulicErosion.kt:1404-1442). P1's routing outputs are the closing pass's, as its
// breach left them.
// run_rounds >= 0 stops after that many rounds (the relaxation keeps the whole stage's share per
// round) and initial = false leaves out the initial sweeps: a bounded sample of a stage.
// refreshed (may be NULL) is the weather the provisional climate gives halfway down when
// params.climate_feed is set (HydraulicErosion.kt:655-661, 809-813): it replaces the given weather
// from round hydraulic_rounds / 2 on. The climate itself is not this path's: the caller solves it.
// belts (may be NULL) is the belts' window: BeltErosion.replay runs on the swept terrain with the
// opening weather before round 0 (HydraulicErosion.kt:680-688), with no sub-grid relief.
int erode_stage(const cg_erosion_params& p, const cg_inputs& in, cg_outputs* out, cg_round_stats* stats,
                bool with_thermal = true, bool initial = true, int run_rounds = -1,
                const Switches* switches = nullptr, Tally* tallies = nullptr,
                LevelRepairs* level_repairs = nullptr, WalkCapture* capture = nullptr,
                const cg_inputs* refreshed = nullptr, const BeltStage* belts = nullptr) {
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
    // The belts' replay on the swept terrain, with the opening weather (HydraulicErosion.kt:680-688).
    if (belts) {
        std::vector<float> ones_b, zeros_b, eroded_b(N);
        if (!in.rainfall_mm) ones_b.assign(N, 1.0f);
        if (!in.vegetation_density) zeros_b.assign(N, 0.0f);
        belt_replay(p, working.data(), belts->tectonic, belts->wear, belts->onset, belts->window_myr,
                    in.uplift_mm_per_year, in.rainfall_mm ? in.rainfall_mm : ones_b.data(),
                    in.vegetation_density ? in.vegetation_density : zeros_b.data(), in.rock_erodibility, p.sea_level,
                    p.shield_cut != 0, nullptr, belts->rebound, belts->history_cell_km, eroded_b.data());
    }
    Rates rates(p);
    const Switches sw = switches ? *switches : switches_of(p);
    double r = sc.cell_height_km(H) / sc.cell_width_km(W);   // cellHeightInCellWidths
    int lattice = smooth_field_lattice_columns(p.world_width_km);
    // What deposition carries (HydraulicErosion.kt:729-789): the load in transit (double), the spoil at
    // rest (laid on the terrain once, at the end), the incision's take per cell, and one set of fan
    // stamps for the whole stage, the mouth ids only ever increasing.
    const DepositionRates dr(p, sw);
    std::vector<float> sediment, settled;
    std::vector<double> load, incised_at;
    std::unique_ptr<FanScratch> scratch;
    std::unique_ptr<SquareScratch> square;
    int mouth_id = 0;
    if (sw.deposition) {
        const int reach = dr.delta_reach_cells < 0 ? 0 : dr.delta_reach_cells;
        sediment.assign(N, 0.0f);
        settled.assign(N, 0.0f);
        load.assign(N, 0.0);
        incised_at.assign(N, 0.0);
        if (sw.delta_outline) scratch.reset(new FanScratch(N, reach, r));
        if (!sw.delta_outline || !sw.delta_lobe) square.reset(new SquareScratch(N, reach));
    }
    auto total_mass = [&](const std::vector<float>& f) {
        double sum = 0.0;
        for (float v : f) sum += (double)v;
        return sum;
    };
    // The plate flexure's state (HydraulicErosion.kt:707-725): the field before the rounds, the bend
    // applied so far, and the uplift so far (which arrives compensated, so is no load).
    std::unique_ptr<Flexure> flexure;
    std::vector<float> reference, deflection, load_pa, uplifted;
    if (sw.flexure) {
        flexure.reset(new Flexure(p));
        reference = working;
        deflection.assign(N, 0.0f);
        load_pa.assign(N, 0.0f);
        if (in.uplift_mm_per_year) uplifted.assign(N, 0.0f);
    }
    std::vector<float> ones(N, 1.0f), zeros(N, 0.0f);
    const float* rain = in.rainfall_mm ? in.rainfall_mm : ones.data();
    const float* veg = in.vegetation_density ? in.vegetation_density : zeros.data();
    const int refresh_at = p.climate_feed && p.hydraulic_rounds > 1 ? p.hydraulic_rounds / 2 : -1;
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
        if (round == refresh_at && refreshed) {   // the sky asked again, halfway down
            rain = refreshed->rainfall_mm ? refreshed->rainfall_mm : ones.data();
            veg = refreshed->vegetation_density ? refreshed->vegetation_density : zeros.data();
        }
        if (in.uplift_mm_per_year) {
            const float* rate = in.uplift_mm_per_year;
            for (size_t c = 0; c < N; ++c) {
                if (rate[c] <= 0.0f) continue;
                float metres = rate[c] * uplift_per_mm;
                working[c] += metres / metres_per_field;
                if (!uplifted.empty()) uplifted[c] += metres;
            }
        }
        if (flexure) {   // HydraulicErosion.kt:856-880: the plate answers the whole load so far
            const float density = p.continental_crust_density, gravity = p.gravity;
            for (size_t c = 0; c < N; ++c) {
                float column = (working[c] - reference[c]) * metres_per_field + deflection[c] -
                               (uplifted.empty() ? 0.0f : uplifted[c]) +
                               (sediment.empty() ? 0.0f : sediment[c] * metres_per_field);
                load_pa[c] = column * density * gravity;
            }
            flexure->deflection(load_pa.data(), load_pa.data());
            for (size_t c = 0; c < N; ++c) {
                const float bend = load_pa[c];
                working[c] += (deflection[c] - bend) / metres_per_field;
                deflection[c] = bend;
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
        float to_relative = 1.0f / land_range;
        Tally t;
        if (sw.deposition) {   // HydraulicErosion.kt:940-945
            std::fill(load.begin(), load.end(), 0.0);
            std::fill(incised_at.begin(), incised_at.end(), 0.0);
            for (size_t c = 0; c < N; ++c) settled[c] = cut.relative[c] + sediment[c] * to_relative;
        }
        const double starting_mass = tallies ? total_mass(working) + (sw.deposition ? total_mass(sediment) : 0.0) : 0.0;
        if (sw.outlet_incision) {
            Spillways notch;
            spillways(W, H, cut.is_land.data(), cut.relative.data(), filled.data(), dirs.data(), rates.pond_depth,
                      notch, nullptr);
            Breached b = breach(rates, W, notch, cut.is_land.data(), cut.relative.data(), filled.data(), dirs.data(),
                                area.data(), land_cells, land_range, working.data(),
                                sw.deposition ? settled.data() : nullptr, sw.deposition ? load.data() : nullptr);
            t.incised += b.moved;
        }
        incise(rates, W, N, order.data(), cut.land_cells, dirs.data(), cut.is_land.data(), filled.data(),
               cut.relative.data(), area.data(), land_cells, land_range, cut.shoreline, erod.data(), working.data(),
               p.receiver_clamp != 0, nullptr, sw.deposition ? incised_at.data() : nullptr);
        if (sw.deposition) {
            DepositionWalk walk(p, sw, dr, rates, dirs.data(), cut.is_land.data(), filled.data(), cut.relative.data(),
                                area.data(), land_cells, land_range, to_relative, cut.shoreline, working.data(),
                                sediment.data(), settled.data(), incised_at.data(), scratch.get(), square.get(),
                                mouth_id, t);
            const bool capturing = capture && round == capture->round;
            if (capturing) {
                WalkCapture& c = *capture;
                c.taken = true;
                c.order = order;
                c.dirs = dirs;
                c.land = cut.is_land;
                c.ground = filled;
                c.relative = cut.relative;
                c.area = area;
                c.surface = working;
                c.sediment = sediment;
                c.settled = settled;
                c.load = load;
                c.incised_at = incised_at;
                c.land_cells = land_cells;
                c.land_range = land_range;
                c.to_relative = to_relative;
                c.shoreline = cut.shoreline;
                c.mouth_id = mouth_id;
            }
            if (level_repairs) run_levels(walk, order.data(), cut.land_cells, load.data(), N, *level_repairs);
            else walk.run(order.data(), cut.land_cells, load.data());
            if (capturing) {
                capture->sediment_after = sediment;
                capture->settled_after = settled;
                capture->load_after = load;
            }
        }
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
        const bool closing = round == p.hydraulic_rounds - 1;
        // The spoil, kept before it becomes terrain (the mouths pass tells fresh ground by it), and
        // settle(): the whole stage's deposition laid on the rock at once (HydraulicErosion.kt:1351-1364).
        std::vector<float> spoil;
        if (closing && sw.delta_lobe) spoil = sw.deposition ? sediment : std::vector<float>(N, 0.0f);
        if (closing && sw.deposition) {
            for (size_t c = 0; c < N; ++c) working[c] += sediment[c];
            std::fill(sediment.begin(), sediment.end(), 0.0f);
        }
        if (closing && sw.outlet_incision) {
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
                Breached b = breach(rates, W, notch, after.is_land.data(), after.relative.data(), filled.data(),
                                    dirs.data(), area.data(), (float)after.land_cells, land_range, working.data());
                t.incised += b.moved;
                t.lost += b.moved;
                order.assign(after.land_cells, 0);
                drainage_order(W, H, after.is_land.data(), dirs.data(), after.land_cells, order.data());
                cut = std::move(after);
            }
        }
        if (closing && sw.delta_lobe) {   // HydraulicErosion.kt:1451-1462
            double removed = open_mouths(p, working.data(), spoil.data(), rates.pond_depth, rain, r, lattice, dr);
            t.incised += removed;
            t.lost += removed;
        }
        // relax = thermalErosion(config, field, accelerator, sweepsPerRound) (ErosionStage.kt:178-180).
        if (with_thermal) thermal_sweep(W, H, working.data(), working.data(), lim, per_round, p.rate, true);
        if (tallies) {
            t.field_drop = starting_mass - total_mass(working) - (sw.deposition ? total_mass(sediment) : 0.0);
            tallies[round] = t;
        }
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

// ---------------------------------------------------------------- the belts' replay (P/BeltErosion.kt)

// Kotlin's Double.toInt(): toward zero, NaN to 0, saturating at the Int range.
int jvm_d2i(double x) {
    if (std::isnan(x)) return 0;
    if (x >= 2147483647.0) return INT32_MAX;
    if (x <= -2147483648.0) return INT32_MIN;
    return (int)x;
}

// GaussianBlur.weights (MA/GaussianBlur.kt:53-65): the continuous Gaussian sampled at cell centres
// out to 4 standard deviations, normalised to one.
std::vector<double> gaussian_taps(double sigma) {
    int radius = std::max(jvm_d2i(std::ceil(4.0 * sigma)), 1);
    std::vector<double> taps(2 * (size_t)radius + 1);
    double total = 0.0;
    for (int off = -radius; off <= radius; ++off) {
        double z = off / sigma;
        double w = std::exp(-0.5 * z * z);
        taps[off + radius] = w;
        total += w;
    }
    for (double& t : taps) t /= total;
    return taps;
}

// GaussianBlur.apply (MA/GaussianBlur.kt:44-47, 67-111): across (x wraps) then down (y clamps), each
// output cell a double sum over the taps in order, rounded to float.
void gaussian_blur(int W, int H, float* data, double sigma_across, double sigma_down) {
    const size_t N = (size_t)W * H;
    std::vector<float> blurred(N);
    if (sigma_across > 0.0) {
        std::vector<double> taps = gaussian_taps(sigma_across);
        const int radius = (int)taps.size() / 2;
        std::vector<double> padded(W + 2 * (size_t)radius);
        for (int row = 0; row < H; ++row) {
            const size_t rs = (size_t)row * W;
            for (size_t slot = 0; slot < padded.size(); ++slot) {
                int col = ((int)slot - radius) % W;
                if (col < 0) col += W;
                padded[slot] = (double)data[rs + col];
            }
            for (int col = 0; col < W; ++col) {
                double sum = 0.0;
                for (size_t t = 0; t < taps.size(); ++t) sum += taps[t] * padded[col + t];
                blurred[rs + col] = (float)sum;
            }
        }
        std::memcpy(data, blurred.data(), N * sizeof(float));
    }
    if (sigma_down > 0.0) {
        std::vector<double> taps = gaussian_taps(sigma_down);
        const int radius = (int)taps.size() / 2;
        std::vector<double> sums(W);
        for (int row = 0; row < H; ++row) {
            std::fill(sums.begin(), sums.end(), 0.0);
            for (size_t t = 0; t < taps.size(); ++t) {
                int src = std::min(std::max(row + (int)t - radius, 0), H - 1);
                const double w = taps[t];
                for (int col = 0; col < W; ++col) sums[col] += w * (double)data[(size_t)src * W + col];
            }
            for (int col = 0; col < W; ++col) blurred[(size_t)row * W + col] = (float)sums[col];
        }
        std::memcpy(data, blurred.data(), N * sizeof(float));
    }
}

const double kCrustKernelSpreadSpacings = 0.6;   // CrustMap.KERNEL_SPREAD_SPACINGS (P/CrustMap.kt:521)
const int kReboundRounds = 10;                   // BeltErosion.REBOUND_ROUNDS

// BeltErosion.replay (P/BeltErosion.kt:96-425), statement by statement. `surface` is the height field,
// changed in place; `eroded` (N) receives the metres each cell lost. rain and cover are required
// here (the entry point fills the defaults); uplift, rock and unresolved may be null.
BeltBooks belt_replay(const cg_erosion_params& p, float* surface, const float* tectonic, const float* wear,
                      const float* onset, double window_myr, const float* uplift, const float* rain,
                      const float* cover, const float* rock, float provisional_sea_level, bool shield_cut,
                      const float* unresolved, bool rebounding, double history_cell_km, float* eroded) {
    BeltBooks books;
    const int W = p.width, H = p.height;
    const size_t N = (size_t)W * H;
    std::fill(eroded, eroded + N, 0.0f);
    const Scale sc = scale_of(p);
    const double round_years = sc.years_per_round;
    const double round_myr = round_years / 1e6;
    const double main_myr = p.hydraulic_rounds * round_myr;
    const int rounds = jvm_d2i((window_myr - main_myr) / round_myr + 1e-9);   // ROUND_ROUNDING
    if (rounds <= 0 || p.hydraulic_rounds <= 0 || p.bedrock_erodibility_per_year <= 0.0f) return books;

    const float freeboard = (p.mantle_density - p.continental_crust_density) / p.mantle_density * 1000.0f;
    const float mpfu = sc.relief_span();   // metersPerFieldUnit

    // The belts, and each one's rise (BeltErosion.kt:127-144).
    std::vector<int> belt;
    std::vector<int> local_of(N, -1);
    for (size_t c = 0; c < N; ++c)
        if (onset[c] >= 0.0f) {
            local_of[c] = (int)belt.size();
            belt.push_back((int)c);
        }
    if (belt.empty()) return books;
    const int B = (int)belt.size();
    std::vector<float> rise_per(B);
    std::vector<int> first_round(B);
    for (int l = 0; l < B; ++l) {
        const int c = belt[l];
        surface[c] = surface[c] - freeboard * (tectonic[c] - wear[c]) / mpfu;
        const double rounds_share =
            uplift ? (double)(uplift[c] * (float)p.hydraulic_rounds) * round_years / 1000.0 : 0.0;
        const double rise_m = (double)(freeboard * tectonic[c]) - rounds_share;
        int f = jvm_d2i(std::ceil((window_myr - (double)onset[c]) / round_myr - 1e-9));
        f = std::min(std::max(f, 0), rounds - 1);
        first_round[l] = f;
        rise_per[l] = (float)(rise_m / (double)(rounds - f) / (double)mpfu);
    }

    // The sea the belts' rivers reach, cut once as the window opens (BeltErosion.kt:147-163).
    Cut opening;
    percentile_cut(W, H, surface, provisional_sea_level, sc, 0.0f, opening);
    const u8* is_land = opening.is_land.data();
    const float shoreline = opening.shoreline;
    const float land_cells = std::max((float)opening.land_cells, 1.0f);
    std::vector<float> weights(N), factor(N);
    double rain_sum = 0.0;
    for (size_t c = 0; c < N; ++c)
        if (is_land[c]) rain_sum += (double)rain[c];
    const float rain_mean = (float)(rain_sum / (double)land_cells);
    for (size_t c = 0; c < N; ++c) weights[c] = rain_mean > 0.0f ? rain[c] / rain_mean : 1.0f;
    double cover_sum = 0.0;
    for (size_t c = 0; c < N; ++c)
        if (is_land[c]) cover_sum += (double)(1.0f - kVegetationShielding * cover[c]);
    const float cover_mean = (float)(cover_sum / (double)land_cells);
    for (size_t c = 0; c < N; ++c) {
        const float cv = (shield_cut && cover_mean > 0.0f) ? (1.0f - kVegetationShielding * cover[c]) / cover_mean : 1.0f;
        factor[c] = cv * (rock ? rock[c] : 1.0f);
    }

    // The water reaching the belts from beyond them, routed once over the opening ground
    // (BeltErosion.kt:166-181).
    const double r = sc.cell_height_km(H) / sc.cell_width_km(W);
    std::vector<double> inflow(B, 0.0);
    {
        std::vector<float> filled0(N), area(N);
        std::vector<int32_t> dirs(N);
        fill_depressions(W, H, is_land, opening.relative.data(), filled0.data());
        flow_directions(W, H, is_land, opening.relative.data(), filled0.data(), p.seed, r,
                        smooth_field_lattice_columns(sc.world_width_km), p.facet_routing != 0, p.flat_potential != 0,
                        dirs.data(), nullptr, nullptr);
        accumulate(W, H, is_land, dirs.data(), opening.land_cells, weights.data(), area.data());
        for (size_t c = 0; c < N; ++c) {
            const int rc = dirs[c];
            if (rc < 0 || local_of[c] >= 0) continue;
            const int l = local_of[rc];
            if (l >= 0) inflow[l] += (double)area[c];
        }
    }

    // The ground just beyond the belts (BeltErosion.kt:184-195).
    std::vector<int> frontier;
    std::vector<u8> on_frontier(N, 0);
    for (int c : belt)
        for_each_neighbour(W, H, c % W, c / W, [&](int n, int, int) {
            if (local_of[n] < 0 && !on_frontier[n]) {
                on_frontier[n] = 1;
                frontier.push_back(n);
            }
        });
    std::sort(frontier.begin(), frontier.end());
    std::vector<int> swept(belt);
    swept.insert(swept.end(), frontier.begin(), frontier.end());

    const Rates rates(p);
    const GroundSteps steps(r);
    const float pond_depth_field = kPondDepthMetres / mpfu;
    const int sweeps_per_round = std::max(sweeps_for(p) / std::max(p.hydraulic_rounds, 1), 1);
    const cg_thermal_limits lim = thermal_limits(p);
    const float courant = rates.courant_coefficient;

    std::vector<double> routing(N);
    for (size_t c = 0; c < N; ++c) routing[c] = (double)surface[c];
    std::vector<float> filled(B, 0.0f), give(B, 0.0f), next(swept.size());
    std::vector<int> receiver(B), donors(B), run_order(B);
    std::vector<double> discharge(B), flux(B);
    std::vector<u8> visited(B);
    const double cell_area = sc.cell_width_km(W) * sc.cell_height_km(H) * 1e6;

    std::vector<float> reference, uplifted_m, rebound_m, loss(N);
    if (rebounding) {
        reference.assign(surface, surface + N);
        uplifted_m.assign(N, 0.0f);
        rebound_m.assign(N, 0.0f);
    }
    const float rebound_share = p.continental_crust_density / p.mantle_density;
    const double crust_spread_km = kCrustKernelSpreadSpacings * history_cell_km;

    // forEachNeighborWithLimit's limit by step (BeltErosion.kt:445-466).
    auto limit_of = [&](int rs, int cs) {
        return (rs != 0 && cs != 0) ? lim.diagonal : (rs != 0 ? lim.north_south : lim.east_west);
    };
    auto at_sea = [&](int c) { return !is_land[c] || surface[c] <= shoreline; };

    for (int round = 0; round < rounds; ++round) {
        // The rock rises where the belt has begun to (BeltErosion.kt:240-248).
        for (int l = 0; l < B; ++l) {
            if (round < first_round[l]) continue;
            const float rise = rise_per[l];
            const int c = belt[l];
            surface[c] = surface[c] + rise;
            if (rebounding) uplifted_m[c] = uplifted_m[c] + rise * mpfu;
            books.uplifted += (double)rise * (double)mpfu * cell_area;
        }
        for (int c : swept) routing[c] = (double)surface[c];

        // Every belt cell's spill level, by a priority flood (BeltErosion.kt:253-284).
        std::fill(visited.begin(), visited.end(), 0);
        std::priority_queue<int64_t, std::vector<int64_t>, std::greater<int64_t>> heap;
        for (int l = 0; l < B; ++l) {
            const int c = belt[l];
            if (at_sea(c)) {
                filled[l] = surface[c];
                visited[l] = 1;
                heap.push(encode(surface[c], l));
                continue;
            }
            bool edge = false;
            for_each_neighbour(W, H, c % W, c / W, [&](int n, int, int) {
                if (local_of[n] < 0) edge = true;
            });
            if (c / W == 0 || c / W == H - 1) edge = true;
            if (edge) {
                filled[l] = surface[c];
                visited[l] = 1;
                heap.push(encode(surface[c], l));
            }
        }
        while (!heap.empty()) {
            const int l = decode_index(heap.top());
            heap.pop();
            const float level = filled[l];
            const int c = belt[l];
            for_each_neighbour(W, H, c % W, c / W, [&](int n, int, int) {
                const int o = local_of[n];
                if (o >= 0 && !visited[o]) {
                    visited[o] = 1;
                    filled[o] = surface[n] <= level ? level + kFlatGradientStep : surface[n];
                    heap.push(encode(filled[o], o));
                }
            });
        }
        for (int l = 0; l < B; ++l) {
            const int c = belt[l];
            if (is_land[c] && surface[c] > shoreline) routing[c] = (double)filled[l];
        }
        // The facet rule over the filled ground (BeltErosion.kt:286-292).
        for (int l = 0; l < B; ++l) {
            const int c = belt[l];
            receiver[l] = at_sea(c) ? -1 : facet_receiver(W, H, routing.data(), c % W, c / W, steps, p.seed);
        }
        // The order the water runs in (BeltErosion.kt:296-311).
        std::fill(donors.begin(), donors.end(), 0);
        for (int l = 0; l < B; ++l) {
            const int d = receiver[l];
            if (d < 0) continue;
            const int dl = local_of[d];
            if (dl >= 0) donors[dl]++;
        }
        int downstream = 0;
        for (int l = 0; l < B; ++l)
            if (donors[l] == 0) run_order[downstream++] = l;
        int walked = 0;
        while (walked < downstream) {
            const int d = receiver[run_order[walked++]];
            if (d < 0) continue;
            const int dl = local_of[d];
            if (dl >= 0 && --donors[dl] == 0) run_order[downstream++] = dl;
        }
        // Water gathered from the top down (BeltErosion.kt:313-323).
        for (int l = 0; l < B; ++l) {
            discharge[l] = (double)weights[belt[l]] + inflow[l];
            flux[l] = 0.0;
        }
        for (int i = 0; i < downstream; ++i) {
            const int l = run_order[i];
            const int d = receiver[l];
            if (d < 0) continue;
            const int dl = local_of[d];
            if (dl >= 0) discharge[dl] += discharge[l];
        }
        // The cut, from the outlets up (BeltErosion.kt:325-351).
        for (int i = downstream - 1; i >= 0; --i) {
            const int l = run_order[i];
            const int c = belt[l];
            const int d = receiver[l];
            if (d < 0) continue;
            if (filled[l] - surface[c] > pond_depth_field) continue;
            const int dl = local_of[d];
            const float own = unresolved ? unresolved[c] : 0.0f;
            float base;
            if (at_sea(d)) base = shoreline + own;
            else if (dl >= 0 && filled[dl] - surface[d] > pond_depth_field) base = filled[dl] + own;
            else base = surface[d] + own - (unresolved ? unresolved[d] : 0.0f);
            const float height = surface[c];
            if (height <= base) continue;
            const double share = discharge[l] / (double)land_cells;
            const double cn = (double)courant * std::sqrt(share) * (double)factor[c] / (double)steps.between(c, d, W);
            const float after = (float)((double)base + (double)(height - base) / (1.0 + cn));
            surface[c] = after;
            const float lost = (height - after) * mpfu;
            eroded[c] = eroded[c] + lost;
            books.cut += (double)lost * cell_area;
            flux[l] += (double)lost * cell_area;
        }
        // The spoil carried down to where it leaves the belts (BeltErosion.kt:354-370).
        for (int i = 0; i < downstream; ++i) {
            const int l = run_order[i];
            const int d = receiver[l];
            if (d < 0) {
                if (at_sea(belt[l])) books.to_sea += flux[l];
                else books.to_land += flux[l];
                continue;
            }
            const int dl = local_of[d];
            if (dl >= 0) flux[dl] += flux[l];
            else if (at_sea(d)) books.to_sea += flux[l];
            else books.to_land += flux[l];
        }

        // The slopes, relaxed by the rounds' own sweeps (BeltErosion.kt:373-408).
        for (int s = 0; s < sweeps_per_round; ++s) {
            for (int l = 0; l < B; ++l) {
                const int c = belt[l], col = c % W, row = c / W;
                const float here = surface[c];
                float excess = 0.0f, steepest = 0.0f;
                for (int rs = -1; rs <= 1; ++rs) {
                    const int nr = row + rs;
                    if (nr < 0 || nr >= H) continue;
                    for (int cs = -1; cs <= 1; ++cs) {
                        if (rs == 0 && cs == 0) continue;
                        const int n = nr * W + (col + cs + W) % W;
                        const float drop = here - surface[n];
                        if (drop > 0.0f) {
                            if (drop > steepest) steepest = drop;
                            const float limit = limit_of(rs, cs);
                            if (drop > limit) excess += drop - limit;
                        }
                    }
                }
                give[l] = excess <= lim.east_west * 1e-3f
                              ? 0.0f
                              : jvm_min(p.rate * excess, steepest * 0.5f) / excess;
            }
            for (size_t k = 0; k < swept.size(); ++k) {
                const int c = swept[k], col = c % W, row = c / W;
                const float here = surface[c];
                const int own = local_of[c];
                float received = 0.0f, given = 0.0f;
                for (int rs = -1; rs <= 1; ++rs) {
                    const int nr = row + rs;
                    if (nr < 0 || nr >= H) continue;
                    for (int cs = -1; cs <= 1; ++cs) {
                        if (rs == 0 && cs == 0) continue;
                        const int n = nr * W + (col + cs + W) % W;
                        const float limit = limit_of(rs, cs);
                        const float incoming = surface[n] - here;
                        const int giver = local_of[n];
                        if (incoming > limit && giver >= 0) received += give[giver] * (incoming - limit);
                        else if (-incoming > limit && own >= 0) given += give[own] * (-incoming - limit);
                    }
                }
                next[k] = here - given + received;
            }
            for (size_t k = 0; k < swept.size(); ++k) {
                const int c = swept[k];
                if (local_of[c] < 0) books.shed += (double)(next[k] - surface[c]) * (double)mpfu * cell_area;
                surface[c] = next[k];
            }
        }

        // The crust answering the rock taken so far (BeltErosion.kt:413-423).
        if (rebounding && ((round + 1) % kReboundRounds == 0 || round == rounds - 1)) {
            for (size_t c = 0; c < N; ++c)
                loss[c] = uplifted_m[c] + rebound_m[c] - (surface[c] - reference[c]) * mpfu;
            gaussian_blur(W, H, loss.data(), crust_spread_km / sc.cell_width_km(W), crust_spread_km / sc.cell_height_km(H));
            for (size_t c = 0; c < N; ++c) {
                const float rebound = rebound_share * loss[c];
                surface[c] = surface[c] + (rebound - rebound_m[c]) / mpfu;
                rebound_m[c] = rebound;
            }
        }
    }
    books.rounds = rounds;
    books.belt_cells = B;
    return books;
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
    p->mantle_density = 3300.0f;
    p->deflection_fill_density = 0.0f;
    p->gravity = 9.81f;
    p->continental_crust_density = 2835.0f;
    p->elastic_thickness_km = 30.0f;
    p->youngs_modulus_gpa = 70.0f;
    p->poisson_ratio = 0.25f;
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

// The stage with climateFeed: `in` carries the opening weather, `refreshed` the weather of the
// halfway refresh (HydraulicErosion.kt:655-661, 809-813).
int32_t or_erode_stage_fed(const cg_erosion_params* p, const cg_inputs* in, const cg_inputs* refreshed,
                           cg_outputs* out) {
    return erode_stage(*p, *in, out, nullptr, true, true, -1, nullptr, nullptr, nullptr, nullptr, refreshed);
}

// HydraulicErosion.apply(config, height, seaLevel) { it }: the rounds alone, with no initial sweeps
// and an identity relaxation, as the reference's incision tests drive it.
int32_t or_hydraulic_apply(const cg_erosion_params* p, const cg_inputs* in, cg_outputs* out,
                           cg_round_stats* stats) {
    return erode_stage(*p, *in, out, stats, false);
}

// The first `rounds` rounds of ErosionStage.apply from heights already swept (no initial sweeps),
// each with its relaxation: a bounded sample of the stage for timing.
// The round tail's switches and the deposition's knobs, for tests that set them one by one
// (ErosionConfig.outletIncision, deposition, deltaLobe, gradedAggradation, deltaOutline, transportCapacity,
// depositionRate, deltaShare, lakeShare, deltaMinCatchmentKm2, deltaReachKm, deltaFreeboardMetres).
struct or_switches {
    int32_t outlet_incision, deposition, delta_lobe, graded_aggradation, delta_outline;
    float transport_capacity, deposition_rate, delta_share, lake_share;
    double delta_min_catchment_km2, delta_reach_km;
    float delta_freeboard_metres;
};

// ErosionStage.apply with explicit switches; tallies (may be NULL) receives per round the incised,
// deposited and lost amounts and the field's drop (RoundMass), 4 doubles a round.
int32_t or_erode_stage_switched(const cg_erosion_params* p, const cg_inputs* in, cg_outputs* out,
                                const or_switches* s, double* tallies, int32_t with_thermal) {
    Switches sw;
    sw.outlet_incision = s->outlet_incision != 0;
    sw.deposition = s->deposition != 0;
    sw.delta_lobe = s->delta_lobe != 0;
    sw.graded_aggradation = s->graded_aggradation != 0;
    sw.delta_outline = s->delta_outline != 0;
    sw.transport_capacity = s->transport_capacity;
    sw.deposition_rate = s->deposition_rate;
    sw.delta_share = s->delta_share;
    sw.lake_share = s->lake_share;
    sw.delta_min_catchment_km2 = s->delta_min_catchment_km2;
    sw.delta_reach_km = s->delta_reach_km;
    sw.delta_freeboard_metres = s->delta_freeboard_metres;
    std::vector<Tally> t(p->hydraulic_rounds > 0 ? p->hydraulic_rounds : 1);
    int st = erode_stage(*p, *in, out, nullptr, with_thermal != 0, true, -1, &sw, tallies ? t.data() : nullptr);
    if (tallies)
        for (int i = 0; i < p->hydraulic_rounds; ++i) {
            tallies[4 * i + 0] = t[i].incised;
            tallies[4 * i + 1] = t[i].deposited;
            tallies[4 * i + 2] = t[i].lost;
            tallies[4 * i + 3] = t[i].field_drop;
        }
    return st;
}

// The stage with the deposition walk run in the device's level order (run_levels); repairs (may be
// NULL) receives the ponded cells replayed and the levels redone over the whole stage.
int32_t or_erode_stage_levels(const cg_erosion_params* p, const cg_inputs* in, cg_outputs* out, int64_t* repairs) {
    LevelRepairs r;
    int st = erode_stage(*p, *in, out, nullptr, true, true, -1, nullptr, nullptr, &r);
    if (repairs) {
        repairs[0] = r.replayed;
        repairs[1] = r.redone;
    }
    return st;
}

// The P2 stage's deposition walk of round `round`, captured: the walk's inputs (N-cell arrays, the
// order holding order_len cells) and, after it, the sediment, settled heights and loads (the load a
// cell passes on is its arriving load). scalars: land_cells, land_range, to_relative, shoreline;
// ints: order_len, the mouth id before the walk. Returns 0 if the round was reached.
int32_t or_capture_walk(const cg_erosion_params* p, const cg_inputs* in, int32_t round, int32_t* order,
                        int32_t* dirs, uint8_t* land, float* ground, float* relative, float* area, float* surface,
                        float* sediment, float* settled, double* load, double* incised_at, float* scalars,
                        int32_t* ints, float* sediment_after, float* settled_after, double* load_after) {
    size_t N = (size_t)p->width * p->height;
    std::vector<float> height(N);
    cg_outputs out{};
    out.height = height.data();
    WalkCapture c;
    c.round = round;
    int st = erode_stage(*p, *in, &out, nullptr, true, true, -1, nullptr, nullptr, nullptr, &c);
    if (st != CG_OK || !c.taken) return 1;
    std::memcpy(order, c.order.data(), c.order.size() * 4);
    std::memcpy(dirs, c.dirs.data(), N * 4);
    std::memcpy(land, c.land.data(), N);
    std::memcpy(ground, c.ground.data(), N * 4);
    std::memcpy(relative, c.relative.data(), N * 4);
    std::memcpy(area, c.area.data(), N * 4);
    std::memcpy(surface, c.surface.data(), N * 4);
    std::memcpy(sediment, c.sediment.data(), N * 4);
    std::memcpy(settled, c.settled.data(), N * 4);
    std::memcpy(load, c.load.data(), N * 8);
    std::memcpy(incised_at, c.incised_at.data(), N * 8);
    scalars[0] = c.land_cells;
    scalars[1] = c.land_range;
    scalars[2] = c.to_relative;
    scalars[3] = c.shoreline;
    ints[0] = (int32_t)c.order.size();
    ints[1] = c.mouth_id;
    std::memcpy(sediment_after, c.sediment_after.data(), N * 4);
    std::memcpy(settled_after, c.settled_after.data(), N * 4);
    std::memcpy(load_after, c.load_after.data(), N * 8);
    return 0;
}

// SeaLevelStage.apply's cut with its enclosure rule and the drowned basins' outlets
// (SeaLevelStage.kt:243-270, enclosedSeaIsLand and postCutOutlet on; the drowned valleys, littoral
// grading and shelf after them are not this path's): is_land, relative, land_cells and the passes run.
int32_t or_sea_level_drained_cut(const cg_erosion_params* p, const float* height, double enclosed_max_share,
                                 int32_t post_cut_outlet, float* shoreline, uint8_t* is_land, float* relative,
                                 int32_t* land_cells, int32_t* passes) {
    const int W = p->width, H = p->height;
    const size_t N = (size_t)W * H;
    const Scale sc = scale_of(*p);
    Cut cut;
    percentile_cut(W, H, height, p->sea_level, sc, 0.0f, cut);
    mark_unreachable_water_as_land(W, H, cut, height, sc, sc.cell_width_km(W) * sc.cell_height_km(H),
                                   enclosed_max_share);
    int run = 0;
    if (post_cut_outlet) drain_drowned_basins(*p, cut, height, enclosed_max_share, &run);
    *shoreline = cut.shoreline;
    std::memcpy(is_land, cut.is_land.data(), N);
    std::memcpy(relative, cut.relative.data(), N * 4);
    *land_cells = cut.land_cells;
    *passes = run;
    return 0;
}

// Isostasy.Flexure(config).deflectionMetres(load, out) (Isostasy.kt:327-372), and its two scalars.
int32_t or_flexure_deflection(const cg_erosion_params* p, const float* load, float* out, double* rigidity,
                              double* restoring) {
    Flexure f(*p);
    f.deflection(load, out);
    if (rigidity) *rigidity = f.rigidity;
    if (restoring) *restoring = f.restoring;
    return 0;
}

int32_t or_stage_rounds(const cg_erosion_params* p, const cg_inputs* in, cg_outputs* out, int32_t rounds) {
    return erode_stage(*p, *in, out, nullptr, true, false, rounds);
}

// BeltErosion.replay (BeltErosion.kt:96-425) on host buffers: `height` is changed in place, `eroded`
// (N) receives the metres each cell lost, counts[2] the rounds and belt cells, books[5] the cubic
// metres uplifted, cut, exported to the sea and to the land, and shed beside. rain and cover may be
// null (all 1, all 0).
int32_t or_belt_replay(const cg_erosion_params* p, float* height, const float* tectonic, const float* wear,
                       const float* onset, double window_myr, const float* uplift, const float* rain,
                       const float* cover, const float* rock, float provisional_sea_level, int32_t shield_cut,
                       const float* unresolved, int32_t rebounding, double history_cell_km, float* eroded,
                       int32_t* counts, double* books) {
    const size_t N = (size_t)p->width * p->height;
    std::vector<float> ones, zeros;
    if (!rain) {
        ones.assign(N, 1.0f);
        rain = ones.data();
    }
    if (!cover) {
        zeros.assign(N, 0.0f);
        cover = zeros.data();
    }
    BeltBooks b = belt_replay(*p, height, tectonic, wear, onset, window_myr, uplift, rain, cover, rock,
                              provisional_sea_level, shield_cut != 0, unresolved, rebounding != 0, history_cell_km,
                              eroded);
    counts[0] = b.rounds;
    counts[1] = b.belt_cells;
    books[0] = b.uplifted;
    books[1] = b.cut;
    books[2] = b.to_sea;
    books[3] = b.to_land;
    books[4] = b.shed;
    return 0;
}

// ErosionStage.apply with the belts' window (the stage above with `belts`).
int32_t or_erode_stage_belts(const cg_erosion_params* p, const cg_inputs* in, const float* tectonic, const float* wear,
                             const float* onset, double window_myr, int32_t rebound, double history_cell_km,
                             cg_outputs* out) {
    BeltStage b{tectonic, wear, onset, window_myr, rebound != 0, history_cell_km};
    return erode_stage(*p, *in, out, nullptr, true, true, -1, nullptr, nullptr, nullptr, nullptr, nullptr, &b);
}

// How far the flats' potentials must move before FlowRouting.facetReceiver's answer can change, per
// cell of `mask`: the relative change delta of the routing surface at the cells of `raised` (each such
// value v moving by up to delta |v|; the other values are the filled field widened, exact) that
// could close the gap between the steepest facet and a facet whose receiver (its draw included) is
// another cell, or carry the winning facet's diagonal share across the cell's Rho8 draw. To first order: a facet
// slope moves by at most 2 delta (the sum of its moving values' |v|) / (its shortest leg), a share by
// share (|d outward| / outward + |d cdrop| / cdrop). Cells outside the mask, with no facet falling, or
// whose deciding values are all exact, get +inf.
void or_facet_flip_delta(int32_t W, int32_t H, const double* rs, const uint8_t* mask, const uint8_t* raised,
                         int64_t seed, double r, double* out) {
    GroundSteps steps(r);
    for (int row = 0; row < H; ++row)
        for (int col = 0; col < W; ++col) {
            const int cell = row * W + col;
            out[cell] = INFINITY;
            if (!mask[cell]) continue;
            const double here = rs[cell];
            const double e_here = raised[cell] ? std::fabs(here) : 0.0;
            struct Facet {
                double slope, moves, share, outward, cdrop, m_out, m_drop;
                int kind, card, diag;
            } f[8];
            int nf = 0, win = -1;
            double best = 0.0;
            for (int side = 0; side < 4; ++side) {
                int ccs = kCardColStep[side], crs = kCardRowStep[side];
                int card = neighbour_at(W, H, col + ccs, row + crs);
                if (card < 0) continue;
                const double e_card = raised[card] ? std::fabs(rs[card]) : 0.0;
                double cdrop = here - rs[card];
                double to_card = (double)steps.of(ccs, crs);
                double on_to_diag = (double)(ccs == 0 ? steps.east_west : steps.north_south);
                for (int turn = -1; turn <= 1; turn += 2) {
                    int dcs = ccs == 0 ? turn : ccs;
                    int drs = crs == 0 ? turn : crs;
                    int diag = neighbour_at(W, H, col + dcs, row + drs);
                    if (diag < 0) continue;
                    const double e_diag = raised[diag] ? std::fabs(rs[diag]) : 0.0;
                    double dfall = here - rs[diag];
                    double dslope = dfall / (double)steps.diagonal;
                    double outward = dfall - cdrop;
                    double cslope = cdrop / to_card;
                    double oslope = outward / on_to_diag;
                    double share_edge =
                        cdrop > 0.0 ? outward * to_card * to_card / (cdrop * on_to_diag * on_to_diag) : 1.0;
                    bool to_cardinal = cdrop > 0.0 && outward <= 0.0;
                    bool to_diagonal = !to_cardinal && share_edge >= 1.0;
                    double fslope = to_cardinal ? cslope
                                                : (to_diagonal ? dslope : std::sqrt(cslope * cslope + oslope * oslope));
                    double share = to_cardinal ? 0.0 : (to_diagonal ? 1.0 : share_edge);
                    const double leg = std::min({to_card, on_to_diag, (double)steps.diagonal});
                    const int kind = share <= 0.0 ? 1 : (share >= 1.0 ? 2 : 3);
                    f[nf] = Facet{fslope, 2.0 * (e_here + e_card + e_diag) / leg, share, outward, cdrop,
                                  e_here + e_diag + e_card, e_here + e_card, kind, card, diag};
                    if (fslope > best) {
                        best = fslope;
                        win = nf;
                    }
                    ++nf;
                }
            }
            if (win < 0) continue;
            const Facet& w = f[win];
            // Each facet's receiver as the rule would take it, the draw included.
            const double draw = sub_grid_draw(col, row, seed);
            auto taken = [&](const Facet& g) {
                return g.kind == 1 ? g.card : (g.kind == 2 ? g.diag : (draw < g.share ? g.diag : g.card));
            };
            double delta = INFINITY;
            for (int i = 0; i < nf; ++i) {
                const Facet& g = f[i];
                if (i == win) continue;
                if (taken(g) == taken(w) || w.moves + g.moves <= 0.0) continue;
                delta = std::min(delta, (w.slope - g.slope) / (w.moves + g.moves));
            }
            // The no-receiver threshold: the winner's slope against zero.
            if (w.moves > 0.0) delta = std::min(delta, w.slope / w.moves);
            if (w.kind == 3 && (w.m_out > 0.0 || w.m_drop > 0.0)) {
                const double d_share = w.share * (2.0 * w.m_out / w.outward + 2.0 * w.m_drop / w.cdrop);
                if (d_share > 0.0) delta = std::min(delta, std::fabs(draw - w.share) / d_share);
            }
            out[cell] = delta;
        }
}

// DeltaFan.growFan driven straight, as DeltaOutlineTest drives it (T:DeltaOutlineTest.kt:556-688): a rim
// at `apex` with the given reach, bearing, hash, grooves and wobble, every cell accepted, its distance
// bent by 1 - surface when `bent` (else 1), every level 0, a budget of 1e9. `sediment` (N, zeroed
// here) receives what the fan laid; returns the volume laid.
double or_grow_fan_fixture(int32_t W, int32_t H, int32_t apex, double r, float reach, float out_x, float out_y,
                           int32_t hash, int32_t grooved, float wobble, const float* surface, int32_t bent,
                           float* sediment) {
    const size_t N = (size_t)W * H;
    std::fill(sediment, sediment + N, 0.0f);
    std::vector<float> settled(N, 0.0f);
    FanScratch scratch(N, (int)reach, r);
    Rim rim(apex, W, r, reach, out_x, out_y, hash, grooved != 0);
    rim.wobble = wobble;
    return grow_fan(
        W, H, 1e9, rim, scratch, 1, surface, sediment, settled.data(), 1.0f, false, nullptr, [](int) { return true; },
        [&](int c) { return bent ? 1.0f - surface[c] : 1.0f; }, [](int, float) { return 0.0f; });
}

int32_t or_fan_hash(int64_t seed, int32_t index) { return fan_hash(seed, index); }

// FlatRouting.stencil (FlatRouting.kt:177-186): the flat Laplacian's east-west, north-south and
// diagonal weights on cells r as tall as they are wide.
void or_flat_stencil(double r, double* weights) {
    Stencil s = stencil_of(r);
    weights[0] = s.ew;
    weights[1] = s.ns;
    weights[2] = s.diag;
}

// GaussianBlur.apply (MA/GaussianBlur.kt:44-111) in place.
void or_gaussian_blur(int32_t W, int32_t H, float* data, double sigma_across, double sigma_down) {
    gaussian_blur(W, H, data, sigma_across, sigma_down);
}

}  // extern "C"
