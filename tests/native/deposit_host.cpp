// The device's deposition logic (cartogenesis_gb300/csrc/cg_deposit.cuh) built for the host, run on a
// round captured from the oracle in the reference's order and in the device's level order, so that
// tests can hold both against the oracle's own walk.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <unordered_map>
#include <vector>

#include "../../cartogenesis_gb300/csrc/cg_deposit.cuh"

using namespace cg::dep;

extern "C" {

// mode 0: the reference's order; mode 1: level by level (own walks, then the level's mouths in rank
// order, with the two repairs); mode 2: mode 1 with each level's mouths in waves of fans whose reaches
// do not overlap; mode 3: mode 1 with every lake fan's admission done first, out of order; mode 4:
// mode 3 with each admission's own visited bits over its box, as fans running side by side keep them;
// mode 5: mode 3 with the lake fans laying in waves of fans whose admitted cells do not meet.
// repairs[3] counts mode 5's laying waves. arriving[] receives each cell's arriving load (the notch's hand-off plus its
// donors'). repairs[0..2]: ponded cells replayed, levels redone, fan waves.
int dep_walk(int mode, const cg_erosion_params* cp, float land_cells, float land_range, float to_relative,
             float shoreline, const int32_t* order, int order_len, const int32_t* dirs, const uint8_t* land,
             const float* ground, const float* relative, const float* area, const float* surface, float* sediment,
             float* settled, const double* load0, const double* incised_at, int first_id, double* arriving,
             long* repairs) {
    const Params p = make_params(*cp, land_cells, land_range, to_relative, shoreline);
    const size_t N = (size_t)p.W * p.H;
    const Fields f{dirs, land, ground, relative, area, surface, sediment, settled, incised_at};
    std::vector<int> stamp(N, 0);
    const int cap = heap_capacity(p);
    std::vector<int> hc(cap), ha(cap);
    std::vector<float> hk(cap), hp(cap);
    Heap heap{hc.data(), hk.data(), hp.data(), ha.data(), cap, 0, 0};
    int id = first_id;
    double incised = 0, deposited = 0;
    repairs[0] = repairs[1] = repairs[2] = repairs[3] = 0;
    if (mode == 0) {
        std::vector<double> load(load0, load0 + N);
        for (int k = 0; k < order_len; ++k) {
            int c = order[k];
            double carried = load[c];
            bool used;
            int kind = own_walk(p, f, c, carried, &used, &incised, &deposited);
            if (kind == SEA) mouth(p, f, c, carried, kind, stamp.data(), ++id, heap, nullptr);
            else if (kind == LAKE) load[dirs[c]] += carried - mouth(p, f, c, carried, kind, stamp.data(), ++id, heap, nullptr);
            else if (kind == ON) load[dirs[c]] += carried;
        }
        std::memcpy(arriving, load.data(), N * 8);
        return 0;
    }
    // Levels.
    std::vector<int> level(N, -1), rank_of(N, -1);
    for (int k = 0; k < order_len; ++k) level[order[k]] = 0, rank_of[order[k]] = k;
    for (int k = 0; k < order_len; ++k) {
        int c = order[k], r = dirs[c];
        if (r >= 0 && land[r]) level[r] = std::max(level[r], level[c] + 1);
    }
    std::vector<int> dstart(N + 1, 0), donors;
    for (int k = 0; k < order_len; ++k) {
        int r = dirs[order[k]];
        if (r >= 0 && land[r]) dstart[r + 1]++;
    }
    for (size_t c = 0; c < N; ++c) dstart[c + 1] += dstart[c];
    donors.resize(dstart[N]);
    {
        std::vector<int> next(dstart.begin(), dstart.end() - 1);
        for (int k = 0; k < order_len; ++k) {
            int c = order[k], r = dirs[c];
            if (r >= 0 && land[r]) donors[next[r]++] = c;
        }
    }
    std::vector<double> handoff(N, 0.0);
    std::vector<char> used(N, 0);
    auto arrive = [&](int c) {
        double v = load0[c];
        for (int k = dstart[c]; k < dstart[c + 1]; ++k) v += handoff[donors[k]];
        return v;
    };
    struct Event {
        int rank, cell, kind;
        double carried;
        std::vector<Touch> touches;
    };
    std::vector<Touch> buffer(cap);
    int lo = 0;
    while (lo < order_len) {
        const int L = level[order[lo]];
        int hi = lo;
        while (hi < order_len && level[order[hi]] == L) ++hi;
        std::vector<float> settled0(hi - lo), sediment0(hi - lo);
        for (int k = lo; k < hi; ++k) settled0[k - lo] = settled[order[k]], sediment0[k - lo] = sediment[order[k]];
        std::vector<Event> events;
        for (int k = lo; k < hi; ++k) {
            int c = order[k];
            double carried = arrive(c);
            bool u;
            int kind = own_walk(p, f, c, carried, &u, &incised, &deposited);
            used[c] = u;
            if (kind == ON) handoff[c] = carried;
            else if (kind == SEA || kind == LAKE) events.push_back({k, c, kind, carried, {}});
        }
        auto run_fan = [&](Event& e) {
            TouchLog log{buffer.data(), cap, 0, 0};
            double laid = mouth(p, f, e.cell, e.carried, e.kind, stamp.data(), ++id, heap, &log);
            if (log.overflow) return false;
            e.touches.assign(buffer.begin(), buffer.begin() + log.count);
            if (e.kind == LAKE) handoff[e.cell] = e.carried - laid;
            return true;
        };
        if (mode == 1) {
            for (Event& e : events)
                if (!run_fan(e)) return 2;
        } else if (mode == 3 || mode == 4 || mode == 5) {
            // Every lake fan's admission first, in reverse rank order (they read only fixed fields),
            // then the mouths in rank order, the lake fans laying over their admitted cells.
            std::vector<std::vector<int>> admitted(events.size());
            std::vector<char> admitted_ok(events.size(), 0);
            for (size_t i = events.size(); i-- > 0;) {
                Event& e = events[i];
                if (e.kind != LAKE) continue;
                const double budget = mouth_budget(p, f, e.cell, e.carried, e.kind);
                Rim m;
                mouth_rim(p, f, e.cell, e.kind, m);
                if (budget <= 0.0 || !mouth_accepts(p, f, false, m.apex)) continue;
                int n;
                if (mode == 3 || mode == 5) {
                    StampVisited v{stamp.data(), ++id};
                    n = admit(p, f, m, false, v, heap);
                } else {
                    std::vector<uint32_t> bits(box_words(p), 0u);
                    int outside = 0;
                    BoxVisited v{bits.data(), p.W, m.apex_column, m.apex_row, box_bx(p), box_by(p), &outside};
                    n = admit(p, f, m, false, v, heap);
                    if (outside) return 3;
                }
                admitted[i].assign(heap.admitted, heap.admitted + n);
                admitted_ok[i] = 1;
            }
            auto lay_lake = [&](size_t i) {
                Event& e = events[i];
                double laid = 0.0;
                if (admitted_ok[i]) {
                    Rim m;
                    mouth_rim(p, f, e.cell, e.kind, m);
                    TouchLog log{buffer.data(), cap, 0, 0};
                    laid = lay_admitted(p, f, m, false, admitted[i].data(), (int)admitted[i].size(),
                                        mouth_budget(p, f, e.cell, e.carried, e.kind), heap, &log);
                    if (log.overflow) return false;
                    e.touches.assign(buffer.begin(), buffer.begin() + log.count);
                }
                handoff[e.cell] = e.carried - laid;
                return true;
            };
            if (mode == 3 || mode == 4) {
                for (size_t i = 0; i < events.size(); ++i) {
                    if (events[i].kind == SEA) {
                        if (!run_fan(events[i])) return 2;
                    } else if (!lay_lake(i)) {
                        return 2;
                    }
                }
            } else {
                // Mode 5: the sea lobes in rank order (they touch only sea cells), and the lake fans'
                // laying in waves: a fan lays once no earlier waiting fan admitted any of its cells; a
                // wave lays in reverse rank order.
                for (size_t i = 0; i < events.size(); ++i)
                    if (events[i].kind == SEA && !run_fan(events[i])) return 2;
                std::vector<int> waiting;
                for (size_t i = 0; i < events.size(); ++i)
                    if (events[i].kind == LAKE) waiting.push_back((int)i);
                std::unordered_map<int, int> claim;
                while (!waiting.empty()) {
                    claim.clear();
                    for (int i : waiting)
                        for (int c : admitted[i]) claim.emplace(c, i);   // the earliest waiting fan keeps a cell
                    std::vector<int> wave, rest;
                    for (int i : waiting) {
                        bool held = true;
                        for (int c : admitted[i]) held = held && claim[c] == i;
                        (held ? wave : rest).push_back(i);
                    }
                    for (auto it = wave.rbegin(); it != wave.rend(); ++it)
                        if (!lay_lake(*it)) return 2;
                    repairs[3]++;
                    waiting.swap(rest);
                }
            }
        } else {
            // Waves: a fan runs once no earlier waiting fan's reach overlaps its own (the rim's widest
            // reach, 1.3 reach cells, plus the neighbours its admission reads); a wave's fans run in
            // reverse rank order, which only disjoint fans can afford.
            const int bx = (int)std::ceil(1.3 * p.reach_cells) + 1;
            const int by = (int)std::ceil(1.3 * p.reach_cells / p.r) + 1;
            auto overlap = [&](int a, int b) {
                int dx = std::abs(a % p.W - b % p.W);
                dx = std::min(dx, p.W - dx);
                int dy = std::abs(a / p.W - b / p.W);
                return dx <= 2 * bx && dy <= 2 * by;
            };
            // Earlier waiting fans are looked up in coarse blocks of the map, one block a reach wide.
            const int sx = 2 * bx + 1, sy = 2 * by + 1;
            const int nbx = (p.W + sx - 1) / sx, nby = (p.H + sy - 1) / sy;
            std::vector<int> waiting(events.size());
            for (size_t i = 0; i < events.size(); ++i) waiting[i] = (int)i;
            while (!waiting.empty()) {
                std::vector<std::vector<int>> block(nbx * nby);
                std::vector<int> wave, rest;
                for (int i : waiting) {
                    const int apex = dirs[events[i].cell];
                    const int ax = (apex % p.W) / sx, ay = (apex / p.W) / sy;
                    bool blocked = false;
                    for (int oy = -1; oy <= 1 && !blocked; ++oy) {
                        const int yy = ay + oy;
                        if (yy < 0 || yy >= nby) continue;
                        for (int ox = -1; ox <= 1 && !blocked; ++ox) {
                            const int xx = ((ax + ox) % nbx + nbx) % nbx;
                            for (int j : block[yy * nbx + xx])
                                if (overlap(apex, dirs[events[j].cell])) {
                                    blocked = true;
                                    break;
                                }
                        }
                    }
                    (blocked ? rest : wave).push_back(i);
                    block[ay * nbx + ax].push_back(i);   // every waiting fan blocks the later ones
                }
                for (auto it = wave.rbegin(); it != wave.rend(); ++it)
                    if (!run_fan(events[*it])) return 2;
                repairs[2]++;
                waiting.swap(rest);
            }
        }
        bool redo = false;
        std::vector<int> replay;
        for (const Event& e : events)
            for (const Touch& t : e.touches) {
                int x = t.cell;
                if (!land[x]) continue;
                if (level[x] == L && rank_of[x] > e.rank) replay.push_back(x);
                int r = dirs[x];
                if (r >= 0 && land[r] && level[r] == L && rank_of[r] > e.rank && used[r]) redo = true;
            }
        if (redo) {
            repairs[1]++;
            for (auto e = events.rbegin(); e != events.rend(); ++e)
                for (auto t = e->touches.rbegin(); t != e->touches.rend(); ++t)
                    settled[t->cell] = t->settled_before, sediment[t->cell] = t->sediment_before;
            for (int k = lo; k < hi; ++k) settled[order[k]] = settled0[k - lo], sediment[order[k]] = sediment0[k - lo];
            for (int k = lo; k < hi; ++k) {
                int c = order[k];
                double carried = arrive(c);
                bool u;
                int kind = own_walk(p, f, c, carried, &u, &incised, &deposited);
                if (kind == ON) handoff[c] = carried;
                else if (kind == SEA) mouth(p, f, c, carried, kind, stamp.data(), ++id, heap, nullptr);
                else if (kind == LAKE) handoff[c] = carried - mouth(p, f, c, carried, kind, stamp.data(), ++id, heap, nullptr);
            }
        } else if (!replay.empty()) {
            std::sort(replay.begin(), replay.end());
            replay.erase(std::unique(replay.begin(), replay.end()), replay.end());
            for (int x : replay) {
                repairs[0]++;
                float v = settled0[rank_of[x] - lo];
                bool own_done = false;
                auto own_op = [&]() {
                    if (incised_at[x] > 0.0) v -= (float)(incised_at[x] * (double)p.to_relative);
                    own_done = true;
                };
                for (const Event& e : events)
                    for (const Touch& t : e.touches)
                        if (t.cell == x) {
                            if (!own_done && e.rank > rank_of[x]) own_op();
                            v += t.increment;
                        }
                if (!own_done) own_op();
                settled[x] = v;
            }
        }
        lo = hi;
    }
    for (size_t c = 0; c < N; ++c) arriving[c] = land[c] ? arrive((int)c) : load0[c];
    return 0;
}

}  // extern "C"
