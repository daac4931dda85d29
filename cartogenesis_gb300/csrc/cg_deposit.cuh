// Profile P2's deposition, the per-cell logic for the device kernels of the deposition walk, built
// for the host too so that tests can run it against the oracle: a cell's own walk and its mouth
// (HydraulicErosion.kt:1068-1349), the floodplain's headroom (HydraulicErosion.kt:2400-2424), the
// outlined lobes and lake fans (DeltaFan.kt: Rim, Scratch, growFan) and the helpers they hash with.
//
// Everything here is the reference's float and double arithmetic in the reference's order. Compiled by
// nvcc with --fmad=false and IEEE division and square root, and by a host compiler with
// -ffp-contract=off, plain operators give the same bits on both.
#pragma once

#include <stdint.h>

#include <cmath>

#include "cg_params.h"

#ifdef __CUDACC__
#define CG_HD __host__ __device__ __forceinline__
#define CG_HDN __host__ __device__
#else
#define CG_HD inline
#define CG_HDN
#endif

namespace cg {
namespace dep {

CG_HD float sqrt_rn(float x) {
#ifdef __CUDA_ARCH__
    return __fsqrt_rn(x);
#else
    return std::sqrt(x);
#endif
}

// ErosionConfig's deposition knobs and the round's constants (HydraulicErosion.kt:285-300, 937-975).
struct Params {
    int W, H;
    int64_t seed;
    double r;                 // cellHeightInCellWidths
    float step_ns, step_diag; // GroundSteps
    float pond_depth;
    float land_cells, land_range, to_relative, shoreline;
    float transport_capacity, deposition_rate, delta_share, lake_share;
    int graded_aggradation;
    int reach_cells;          // deltaReachCells, at least 0
    float delta_top, rim_top, shelf_depth, delta_min_cells;
};

// The round's constants from the configuration and the round's cut (HydraulicErosion.kt:285-300,
// 639, 937-975), with the reference's float steps: host code.
inline Params make_params(const cg_erosion_params& cp, float land_cells, float land_range, float to_relative,
                          float shoreline) {
    const ScaleF s = scale_of(cp);
    const RatesF rates = rates_of(cp);
    Params p;
    p.W = cp.width;
    p.H = cp.height;
    p.seed = cp.seed;
    p.r = rates.cell_height_in_cell_widths;
    p.step_ns = rates.step_ns;
    p.step_diag = rates.step_diag;
    p.pond_depth = rates.pond_depth;
    p.land_cells = land_cells;
    p.land_range = land_range;
    p.to_relative = to_relative;
    p.shoreline = shoreline;
    p.transport_capacity = 20.0f;   // ErosionConfig.transportCapacity
    p.deposition_rate = 0.06f;      // ErosionConfig.depositionRate
    p.delta_share = 0.15f;          // ErosionConfig.deltaShare
    p.lake_share = 0.1f;            // ErosionConfig.lakeShare
    p.graded_aggradation = 1;       // ErosionConfig.gradedAggradation
    int reach = whole_cells_for(cp, 140.625, 1);   // ErosionConfig.deltaReachKm
    p.reach_cells = reach < 0 ? 0 : reach;
    const float delta_freeboard = s.relief_share_of_metres(48.0f);   // ErosionConfig.deltaFreeboardMetres
    p.delta_top = shoreline + delta_freeboard * land_range;
    p.rim_top = shoreline + (p.delta_top - shoreline) * 0.15f;        // LOBE_RIM
    const float shelf_break = s.field_share_of_metres(130.0f);       // SHELF_BREAK_METRES
    p.shelf_depth = shelf_break < 1e-9f ? 1e-9f : shelf_break;
    const double km2 = s.cell_width_km(cp.width) * s.cell_height_km(cp.height);
    p.delta_min_cells = (float)(70000.0 / km2);                     // ErosionConfig.deltaMinCatchmentKm2
    return p;
}

// Entries a fan's heap needs: DeltaFan.Scratch's capacity.
inline int heap_capacity(const Params& p) {
    int reach_rows = (int)std::ceil(p.reach_cells / p.r);
    int c = (2 * p.reach_cells + 1) * (2 * reach_rows + 1);
    return c < 9 ? 9 : c;
}

// The fields a round's walk reads and writes.
struct Fields {
    const int32_t* dirs;
    const uint8_t* land;
    const float* ground;      // the filled surface
    const float* relative;
    const float* area;
    const float* surface;     // the terrain (the walk does not change it)
    float* sediment;
    float* settled;
    const double* incised_at;
};

enum Kind { OFF_MAP = -1, ON = 0, SEA = 1, LAKE = 2 };

CG_HD bool negative_sign(double a) {
#ifdef __CUDA_ARCH__
    return __double_as_longlong(a) < 0;
#else
    return std::signbit(a);
#endif
}

// Math.min(double, double) on the JVM.
CG_HD double jvm_min(double a, double b) {
    if (a != a) return a;
    if (b != b) return b;
    if (a == 0.0 && b == 0.0) return negative_sign(a) ? a : b;
    return a < b ? a : b;
}

CG_HD int shortest_x(int dx, int W) {
    if (dx > W / 2) return dx - W;
    if (dx < -W / 2) return dx + W;
    return dx;
}

// GroundSteps.between / of.
CG_HD float between(const Params& p, int from, int to) {
    const bool same_row = from / p.W == to / p.W;
    const bool same_col = from % p.W == to % p.W;
    return (!same_row && !same_col) ? p.step_diag : (!same_row ? p.step_ns : 1.0f);
}
CG_HD float step_of(const Params& p, int dc, int dr) {
    if (dc != 0 && dr != 0) return p.step_diag;
    if (dr != 0) return p.step_ns;
    return 1.0f;
}

// HydraulicErosion.wobble: Int arithmetic, wrapping.
CG_HD float cell_wobble(int cell) {
    uint32_t bits = (uint32_t)cell * 0x9E3779B9u;
    bits ^= bits >> 15;
    bits *= 0x2c1b3c6du;
    bits ^= bits >> 12;
    return (float)((bits >> 8) & 0xFFFFu) / 65535.0f;
}

// HydraulicErosion.mouthKey.
CG_HD int mouth_key(int apex, int reach_cells, int W) {
    int block = reach_cells < 1 ? 1 : reach_cells;
    return (apex / W / block) * 0x2000 + (apex % W / block);
}

// DeltaFan.hash: Long arithmetic, wrapping.
CG_HD int32_t fan_hash(int64_t seed, int32_t index) {
    uint64_t mixed = (uint64_t)seed * (uint64_t)(-0x61c8864680b583ebLL) +
                     (uint64_t)(int64_t)index * (uint64_t)(-0x7ee3623a03d3c83fLL) + (uint64_t)0x5DE17A11;
    mixed = (mixed ^ (mixed >> 30)) * (uint64_t)(-0x40a7b892e31b1a47LL);
    mixed = (mixed ^ (mixed >> 27)) * (uint64_t)(-0x6b2fb644ecceee15LL);
    mixed = mixed ^ (mixed >> 31);
    return (int32_t)(uint32_t)(mixed >> 17);
}

// DeltaFan.draw.
CG_HD float fan_draw(int32_t hash, int slot) {
    uint32_t mixed = (uint32_t)hash + (uint32_t)slot * 0x9E3779B9u;
    mixed ^= mixed >> 15;
    mixed *= 0x2c1b3c6du;
    mixed ^= mixed >> 12;
    mixed *= 0x297a2d39u;
    mixed ^= mixed >> 15;
    return (float)((mixed >> 8) & 0xFFFFu) / 65535.0f;
}

// Reads and writes of the sediment and settled heights a fan or lobe may share with one laid just
// before it. On the device they go through L2: the earlier one may have run on another SM of the same
// launch and handed over through a flag rather than a grid barrier, and L1 is not coherent. On the host
// they are plain accesses.
CG_HD float ld_l2(const float* p) {
#ifdef __CUDA_ARCH__
    return __ldcg(p);
#else
    return *p;
#endif
}
CG_HD void st_l2(float* p, float v) {
#ifdef __CUDA_ARCH__
    __stcg(p, v);
#else
    *p = v;
#endif
}

// HydraulicErosion.raise: the change the float field actually took, in double.
CG_HD double raise(float* field, int cell, double amount) {
    const float prior = ld_l2(&field[cell]);
    const float now = (float)((double)prior + amount);
    st_l2(&field[cell], now);
    return (double)now - (double)prior;
}

// HydraulicErosion.headroom.
CG_HD float headroom(const Params& p, const Fields& f, int cell, float drop, float grade) {
    float room = 3.402823466e+38f;
    bool fed = false;
    const int col = cell % p.W, row = cell / p.W;
    for (int rs = -1; rs <= 1; ++rs) {
        int nr = row + rs;
        if (nr < 0 || nr >= p.H) continue;
        for (int cs = -1; cs <= 1; ++cs) {
            if (cs == 0 && rs == 0) continue;
            int nc = (col + cs) % p.W;
            if (nc < 0) nc += p.W;
            int n = nr * p.W + nc;
            if (f.dirs[n] != cell) continue;
            fed = true;
            float margin = f.settled[n] - f.settled[cell] - grade * between(p, n, cell);
            if (margin < room) room = margin;
        }
    }
    return fed ? room : drop - grade;
}

CG_HD bool ponded(const Params& p, const Fields& f, int c) { return f.ground[c] - f.relative[c] > p.pond_depth; }

// A cell's own walk (HydraulicErosion.kt:1068-1186) with `carried` arriving; returns where what it
// carries goes. *used_headroom says whether it read its donors' settled heights; the incision's take
// and the floodplain's give are added to *incised and *deposited.
CG_HD int own_walk(const Params& p, const Fields& f, int cell, double& carried, bool* used_headroom,
                   double* incised, double* deposited) {
    const int receiver = f.dirs[cell];
    *used_headroom = false;
    if (receiver < 0) return OFF_MAP;
    const bool to_sea = !f.land[receiver];
    const float drop = f.ground[cell] - (f.land[receiver] ? f.ground[receiver] : 0.0f);
    const bool wet = ponded(p, f, cell);
    const float distance = between(p, cell, receiver);
    const float slope = drop > 0.0f ? drop / distance * (float)p.W : 0.0f;
    const double capacity = (double)(p.transport_capacity * sqrt_rn(f.area[cell] / p.land_cells) * slope);
    const double moved = f.incised_at[cell];
    if (moved > 0.0) {
        f.settled[cell] -= (float)(moved * (double)p.to_relative);
        carried += moved;
        *incised += moved;
    }
    if (!wet && carried > capacity) {
        float grade = 0.0f;
        if (p.graded_aggradation) {
            const double conveyance = (double)(p.transport_capacity * sqrt_rn(f.area[cell] / p.land_cells));
            grade = conveyance > 1e-12 ? (float)(carried / conveyance / (double)p.W) : 0.0f;
        }
        *used_headroom = true;
        const float room = headroom(p, f, cell, drop, grade) * p.land_range;
        const double give = jvm_min(carried - capacity, (double)room) * (double)p.deposition_rate;
        if (give > 0.0) {
            const double laid = raise(f.sediment, cell, give);
            f.settled[cell] += (float)(laid * (double)p.to_relative);
            carried -= laid;
            *deposited += laid;
        }
    }
    if (to_sea) return SEA;
    if (!wet && ponded(p, f, receiver)) return LAKE;
    return ON;
}

// DeltaFan.Rim: a lobe's outline around its apex, its bearing, its wobble and its grooves.
struct Rim {
    int apex, width;
    float reach_cells;
    int apex_column, apex_row;
    float ahead_x, ahead_y;
    float ph2x, ph2y, ph3x, ph3y, ph5x, ph5y, ph7x, ph7y;
    int distributaries, live;
    float groove_x[5], groove_y[5];
    float groove_half_width;
    float row_scale;
    float step_ns, step_diag;
};

CG_HD void rim_phase(int32_t hash, int slot, float& x, float& y) {
    float hx = fan_draw(hash, slot * 2) * 2.0f - 1.0f;
    float hy = fan_draw(hash, slot * 2 + 1) * 2.0f - 1.0f;
    float len = sqrt_rn(hx * hx + hy * hy);
    if (len < 1e-4f) {
        x = 1.0f;
        y = 0.0f;
    } else {
        x = hx / len;
        y = hy / len;
    }
}

constexpr float kSideReachShare = 0.38f;
constexpr float kFanWobble = 0.30f;
constexpr float kWobbleW2 = 1.0f, kWobbleW3 = 0.7f, kWobbleW5 = 0.5f, kWobbleW7 = 0.45f;
constexpr float kDistributarySpread = 1.1f;
constexpr float kLobeRim = 0.15f;
constexpr float kDepthCost = 1.0f;
constexpr float kGrooveKeep = 0.45f;
constexpr float kLakeFanSlope = 1.5f;

CG_HD float wobble_total_inverse() { return 1.0f / (kWobbleW2 + kWobbleW3 + kWobbleW5 + kWobbleW7); }

CG_HD float rim_radius(const Rim& m, float co, float ro, float distance) {
    if (distance <= 0.0f) return m.reach_cells;
    float c1 = co / distance, s1 = ro / distance;
    float ahead = c1 * m.ahead_x + s1 * m.ahead_y;
    float nose = kSideReachShare + (1.0f - kSideReachShare) * (ahead > 0.0f ? ahead : 0.0f);
    float c2 = c1 * c1 - s1 * s1, s2 = 2.0f * c1 * s1;
    float c3 = c2 * c1 - s2 * s1, s3 = s2 * c1 + c2 * s1;
    float c5 = c3 * c2 - s3 * s2, s5 = s3 * c2 + c3 * s2;
    float c7 = c5 * c2 - s5 * s2, s7 = s5 * c2 + c5 * s2;
    float term = (kWobbleW2 * (c2 * m.ph2x - s2 * m.ph2y) + kWobbleW3 * (c3 * m.ph3x - s3 * m.ph3y) +
                  kWobbleW5 * (c5 * m.ph5x - s5 * m.ph5y) + kWobbleW7 * (c7 * m.ph7x - s7 * m.ph7y)) *
                 wobble_total_inverse();
    return m.reach_cells * nose * (1.0f + kFanWobble * term);
}

CG_HD void rim_init(Rim& m, int apex, int width, double r, float step_ns, float step_diag, float reach,
                    float out_x, float out_y, int32_t hash, bool grooved) {
    m.apex = apex;
    m.width = width;
    m.reach_cells = reach;
    m.apex_column = apex % width;
    m.apex_row = apex / width;
    m.row_scale = (float)r;
    m.step_ns = step_ns;
    m.step_diag = step_diag;
    m.ahead_x = m.ahead_y = 0.0f;
    for (int g = 0; g < 5; ++g) m.groove_x[g] = m.groove_y[g] = 0.0f;
    m.groove_half_width = reach * 0.05f > 0.55f ? reach * 0.05f : 0.55f;
    float out_down = out_y * m.row_scale;
    float out_length = sqrt_rn(out_x * out_x + out_down * out_down);
    if (out_length > 0.0f) {
        m.ahead_x = out_x / out_length;
        m.ahead_y = out_down / out_length;
    }
    rim_phase(hash, 1, m.ph2x, m.ph2y);
    rim_phase(hash, 2, m.ph3x, m.ph3y);
    rim_phase(hash, 3, m.ph5x, m.ph5y);
    rim_phase(hash, 4, m.ph7x, m.ph7y);
    m.distributaries = (!grooved || reach < 4.0f || out_length <= 0.0f) ? 0 : 2 + (int)(((uint32_t)hash >> 3) & 3u);
    if (m.distributaries > 0) {
        const int n = m.distributaries;
        float left_x = -m.ahead_y, left_y = m.ahead_x;
        float span = n > 1 ? 2.0f * kDistributarySpread / (float)(n - 1) : 0.0f;
        for (int g = 0; g < n; ++g) {
            float jitter = (fan_draw(hash, 10 + g) - 0.5f) * 0.8f * span;
            float off_axis = n > 1 ? -kDistributarySpread + span * (float)g + jitter : jitter;
            float ray_x = m.ahead_x + left_x * off_axis;
            float ray_y = m.ahead_y + left_y * off_axis;
            float ray_length = sqrt_rn(ray_x * ray_x + ray_y * ray_y);
            if (ray_length < 1e-6f) ray_length = 1e-6f;
            m.groove_x[g] = ray_x / ray_length;
            m.groove_y[g] = ray_y / ray_length;
        }
    }
    m.live = m.distributaries;
}

CG_HD bool rim_grooved(const Rim& m, float co, float ro) {
    for (int g = 0; g < m.live; ++g) {
        if (co * m.groove_x[g] + ro * m.groove_y[g] < 0.0f) continue;
        float across = co * m.groove_y[g] - ro * m.groove_x[g];
        if (across > -m.groove_half_width && across < m.groove_half_width) return true;
    }
    return false;
}

CG_HD float rim_column_offset(const Rim& m, int cell) { return (float)shortest_x(cell % m.width - m.apex_column, m.width); }
CG_HD float rim_row_offset(const Rim& m, int cell) { return (float)(cell / m.width - m.apex_row) * m.row_scale; }

// Rim.pruneGrooves with `open` = a sea cell.
CG_HD void rim_prune(Rim& m, int height, const uint8_t* land) {
    int kept = 0;
    for (int g = 0; g < m.distributaries; ++g) {
        float rx = m.groove_x[g], ry = m.groove_y[g];
        float ray_reach = rim_radius(m, rx, ry, 1.0f);
        bool blocked = false;
        float stride = 1.0f < m.row_scale ? 1.0f : m.row_scale;
        float along = stride;
        while (along <= (float)(int)ray_reach) {
            int row = m.apex_row + (int)(ry * along / m.row_scale);
            if (row < 0 || row >= height) {
                blocked = true;
                break;
            }
            int column = (m.apex_column + (int)(rx * along)) % m.width;
            if (column < 0) column += m.width;
            if (land[row * m.width + column]) {
                blocked = true;
                break;
            }
            along += stride;
        }
        if (blocked) continue;
        if (kept != g) {
            m.groove_x[kept] = m.groove_x[g];
            m.groove_y[kept] = m.groove_y[g];
        }
        kept++;
    }
    m.live = kept;
}

// DeltaFan.Scratch for one fan: a min-heap on (key, cell) with penalties, the admitted list, and the
// stamps (shared by every fan of the stage; ids only increase).
struct Heap {
    int* cells;
    float* keys;
    float* penalties;
    int* admitted;
    int capacity;
    int size;
    int admitted_count;
};

CG_HD bool heap_less(const Heap& h, int a, int b) {
    return h.keys[a] < h.keys[b] || (h.keys[a] == h.keys[b] && h.cells[a] < h.cells[b]);
}
CG_HD void heap_swap(Heap& h, int a, int b) {
    int c = h.cells[a];
    h.cells[a] = h.cells[b];
    h.cells[b] = c;
    float k = h.keys[a];
    h.keys[a] = h.keys[b];
    h.keys[b] = k;
    float q = h.penalties[a];
    h.penalties[a] = h.penalties[b];
    h.penalties[b] = q;
}
CG_HD void heap_push(Heap& h, int cell, float key, float penalty) {
    if (h.size >= h.capacity) return;
    int slot = h.size++;
    h.cells[slot] = cell;
    h.keys[slot] = key;
    h.penalties[slot] = penalty;
    while (slot > 0) {
        int parent = (slot - 1) / 2;
        if (!heap_less(h, slot, parent)) break;
        heap_swap(h, slot, parent);
        slot = parent;
    }
}
CG_HD bool heap_pop(Heap& h, int& cell, float& penalty) {
    if (h.size == 0) return false;
    cell = h.cells[0];
    penalty = h.penalties[0];
    h.size--;
    if (h.size > 0) {
        h.cells[0] = h.cells[h.size];
        h.keys[0] = h.keys[h.size];
        h.penalties[0] = h.penalties[h.size];
        int slot = 0;
        while (true) {
            int left = 2 * slot + 1;
            if (left >= h.size) break;
            int right = left + 1;
            int smaller = left;
            if (right < h.size && heap_less(h, right, left)) smaller = right;
            if (!heap_less(h, smaller, slot)) break;
            heap_swap(h, slot, smaller);
            slot = smaller;
        }
    }
    return true;
}

// A cell a fan laid into: its settled height and sediment before, and what its settled height gained.
struct Touch {
    int cell;
    float settled_before, sediment_before, increment;
};

// A fan's deposit log (may be absent): the touches in laying order, up to `capacity`.
struct TouchLog {
    Touch* touches;
    int capacity;
    int count;
    int overflow;
};

// The mouth of `cell` (HydraulicErosion.kt:1187-1349) with the outlined fans of profile P2: a sea lobe
// or a lake fan grown from the receiver by growFan (DeltaFan.kt), in two halves. The admission grows
// the admitted set best-first over distance bent by depth inside the rim; a lake fan's admission reads
// only fixed fields (land, the lake's depth), a sea lobe's reads the sediment earlier lobes laid. The
// laying then builds the admitted cells nearest first, each up to its level.
CG_HD bool mouth_accepts(const Params& p, const Fields& f, bool sea, int c) {
    return sea ? !f.land[c] : (f.land[c] && ponded(p, f, c));
}

CG_HD double mouth_budget(const Params& p, const Fields& f, int cell, double carried, int kind) {
    if (kind == SEA) return f.area[cell] >= p.delta_min_cells ? carried * (double)p.delta_share : 0.0;
    return carried * (double)p.lake_share;
}

CG_HD void mouth_rim(const Params& p, const Fields& f, int cell, int kind, Rim& m) {
    const int receiver = f.dirs[cell];
    const int W = p.W;
    const float out_x = (float)shortest_x(receiver % W - cell % W, W);
    const float out_y = (float)(receiver / W - cell / W);
    rim_init(m, receiver, W, p.r, p.step_ns, p.step_diag, (float)p.reach_cells, out_x, out_y,
             fan_hash(p.seed, mouth_key(receiver, p.reach_cells, W)), kind == SEA);
    if (kind == SEA) rim_prune(m, p.H, f.land);
}

// The cells a fan has pushed: the stage's stamps (a cell is this fan's when it holds the fan's id;
// ids only increase), for fans that run one at a time.
struct StampVisited {
    int* stamp;
    int id;
    CG_HD bool seen(int n) const { return stamp[n] == id; }
    CG_HD void mark(int n) { stamp[n] = id; }
};

// The same for a fan that runs beside others: its own bits over the box its admission can reach
// (the rim's widest reach, 1.3 reach cells, and the neighbours it reads). A cell outside the box,
// which the rim's bound excludes, sets `outside` and reads as seen.
struct BoxVisited {
    uint32_t* bits;
    int W, apex_col, apex_row, bx, by;
    int* outside;
    CG_HD int index(int n) const {
        int dx = shortest_x(n % W - apex_col, W), dy = n / W - apex_row;
        if (dx < -bx || dx > bx || dy < -by || dy > by) return -1;
        return (dy + by) * (2 * bx + 1) + (dx + bx);
    }
    CG_HD bool seen(int n) const {
        int i = index(n);
        if (i < 0) {
            *outside = 1;
            return true;
        }
        return (bits[i >> 5] >> (i & 31)) & 1u;
    }
    CG_HD void mark(int n) {
        int i = index(n);
        if (i >= 0) bits[i >> 5] |= 1u << (i & 31);
    }
};

// The half sizes of a BoxVisited box, and its words.
CG_HD int box_bx(const Params& p) { return (int)ceilf(1.3f * (float)p.reach_cells) + 2; }
CG_HD int box_by(const Params& p) { return (int)ceil(1.3 * (double)p.reach_cells / p.r) + 2; }
CG_HD int box_words(const Params& p) { return ((2 * box_bx(p) + 1) * (2 * box_by(p) + 1) + 31) / 32; }

// The admission; heap.admitted[0..returned) holds the admitted cells in admission order.
template <class Visited>
CG_HD int admit(const Params& p, const Fields& f, const Rim& m, bool sea, Visited& visited, Heap& heap) {
    const int W = p.W;
    heap.size = 0;
    heap.admitted_count = 0;
    visited.mark(m.apex);
    heap_push(heap, m.apex, 0.0f, 0.0f);
    int cur;
    float penalty;
    while (heap_pop(heap, cur, penalty)) {
        if (heap.admitted_count < heap.capacity) heap.admitted[heap.admitted_count++] = cur;
        const int column = cur % W, row = cur / W;
        for (int sy = -1; sy <= 1; ++sy) {
            int nr = row + sy;
            if (nr < 0 || nr >= p.H) continue;
            for (int sx = -1; sx <= 1; ++sx) {
                if (sx == 0 && sy == 0) continue;
                int nc = (column + sx) % W;
                if (nc < 0) nc += W;
                int n = nr * W + nc;
                if (visited.seen(n) || !mouth_accepts(p, f, sea, n)) continue;
                float co = rim_column_offset(m, n), ro = rim_row_offset(m, n);
                float distance = sqrt_rn(co * co + ro * ro);
                float depth = sea ? p.shoreline - (f.surface[n] + ld_l2(&f.sediment[n]))
                                  : (f.ground[n] - f.relative[n]) * p.land_range;
                float advance = 1.0f + kDepthCost * (depth > 0.0f ? depth : 0.0f) / p.shelf_depth;
                float np = penalty + step_of(p, sx, sy) * (advance - 1.0f);
                if (distance + np > rim_radius(m, co, ro, distance)) continue;
                visited.mark(n);
                heap_push(heap, n, distance + np, np);
            }
        }
    }
    return heap.admitted_count;
}

// The laying over `count` admitted cells (the heap's own arrays order them; `admitted` must not be
// the heap's cells array). Returns what it laid.
CG_HD double lay_admitted(const Params& p, const Fields& f, const Rim& m, bool sea, const int* admitted, int count,
                          double budget, Heap& heap, TouchLog* log) {
    heap.size = 0;
    for (int k = 0; k < count; ++k) {
        int c = admitted[k];
        float co = rim_column_offset(m, c), ro = rim_row_offset(m, c);
        heap_push(heap, c, sqrt_rn(co * co + ro * ro), 0.0f);
    }
    double remaining = budget, laid = 0.0;
    int cur;
    float penalty;
    while (remaining > 0.0 && heap_pop(heap, cur, penalty)) {
        float co = rim_column_offset(m, cur), ro = rim_row_offset(m, cur);
        float distance = sqrt_rn(co * co + ro * ro);
        float fraction = distance / m.reach_cells;
        if (fraction > 1.0f) fraction = 1.0f;
        float level;
        if (sea) {
            level = p.delta_top + (p.rim_top - p.delta_top) * fraction;
            if (rim_grooved(m, co, ro)) level = p.shoreline + (level - p.shoreline) * kGrooveKeep;
        } else {
            float depth = 2.0f * p.pond_depth * (1.0f + kLakeFanSlope * fraction) * (0.9f + 0.35f * cell_wobble(cur));
            level = p.shoreline + (f.ground[cur] - depth) * p.land_range;
        }
        double need = (double)level - (double)f.surface[cur] - (double)ld_l2(&f.sediment[cur]);
        if (need <= 0.0) continue;
        if (sea && need > remaining) break;   // a sea lobe lays whole cells
        if (log) {
            if (log->count < log->capacity)
                log->touches[log->count] = {cur, ld_l2(&f.settled[cur]), ld_l2(&f.sediment[cur]), 0.0f};
            else log->overflow = 1;
        }
        double moved = raise(f.sediment, cur, need < remaining ? need : remaining);
        float increment = (float)(moved * (double)p.to_relative);
        st_l2(&f.settled[cur], ld_l2(&f.settled[cur]) + increment);
        if (log && log->count < log->capacity) log->touches[log->count++].increment = increment;
        remaining -= moved;
        laid += moved;
    }
    return laid;
}

// The whole mouth, its admission's visited cells kept by `make_visited(rim)`. Returns what it laid.
template <class MakeVisited>
CG_HD double mouth_with(const Params& p, const Fields& f, int cell, double carried, int kind, MakeVisited make_visited,
                        Heap& heap, TouchLog* log) {
    const bool sea = kind == SEA;
    const double budget = mouth_budget(p, f, cell, carried, kind);
    Rim m;
    mouth_rim(p, f, cell, kind, m);
    if (budget <= 0.0 || !mouth_accepts(p, f, sea, m.apex)) return 0.0;
    auto visited = make_visited(m);
    const int count = admit(p, f, m, sea, visited, heap);
    return lay_admitted(p, f, m, sea, heap.admitted, count, budget, heap, log);
}

// The whole mouth with the stage's stamps. Returns what it laid.
CG_HD double mouth(const Params& p, const Fields& f, int cell, double carried, int kind, int* stamp, int id,
                   Heap& heap, TouchLog* log) {
    return mouth_with(p, f, cell, carried, kind, [=](const Rim&) { return StampVisited{stamp, id}; }, heap, log);
}

}  // namespace dep
}  // namespace cg
