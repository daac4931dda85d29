"""Pins the oracle (the CPU restatement) to the reference's own known answers.

The reference ships no golden arrays; what it pins are analytic answers and exact invariants.
Each test here ports one of them, with the reference test it follows named in its docstring
(T = worldgen/src/jvmTest/kotlin/com/cartogenesis/worldgen). The fixtures are rebuilt from the
reference tests' own constants.
"""
import math

import numpy as np
import pytest

import oracle
from cartogenesis_gb300 import synthetic

f32 = np.float32


def field_at_altitude(m):
    """WorldScale.fieldAtAltitude in float (M/WorldGenConfig.kt:192)."""
    return f32(f32(m) + f32(10000.0)) / f32(16000.0)


def altitude_at_field(f):
    """WorldScale.altitudeAtField (M/WorldGenConfig.kt:195)."""
    return float(f32(f32(f) * f32(16000.0)) - f32(10000.0))


# ------------------------------------------------------------------ fill (T/DepressionFillTest.kt)

def test_depression_fill_fixture():
    """T/DepressionFillTest.kt:36-106 on its 32x32 grid (:118-171): no sinks, every land cell has a
    receiver, the submerged patch comes up to its spill level, the plateau rim keeps exactly 0.05
    and the pit is raised to it."""
    side = 32
    sea_floor, submerged, plateau, pit_level = f32(-0.1), f32(-0.2), f32(0.05), f32(0.01)
    is_land = np.zeros((side, side), np.uint8)
    elev = np.full((side, side), sea_floor, np.float32)
    is_land[12:20, 12:20] = 1
    elev[12:20, 12:20] = submerged
    is_land[3:8, 3:8] = 1
    elev[3:8, 3:8] = plateau
    elev[5, 5] = pit_level
    filled = oracle.fill_depressions(is_land, elev)
    # WorldGenConfig().cellHeightInCellWidths on the default 512 x 512 grid is 0.5.
    target, _ = oracle.flow_directions(is_land, elev, filled, seed=1, r=0.5, lattice=side // 8)
    sinks = without = 0
    for r in range(side):
        for c in range(side):
            if not is_land[r, c]:
                continue
            lower = False
            for dr in (-1, 0, 1):
                nr = r + dr
                if nr < 0 or nr >= side:
                    continue
                for dc in (-1, 0, 1):
                    if dr == 0 and dc == 0:
                        continue
                    nc = (c + dc) % side
                    s = filled[nr, nc] if is_land[nr, nc] else elev[nr, nc]
                    if s < filled[r, c]:
                        lower = True
            sinks += not lower
            without += target[r, c] < 0
    assert sinks == 0
    assert without == 0
    corner = filled[12, 12]
    assert sea_floor < corner < sea_floor + f32(1e-3)
    assert filled[3, 3] == plateau
    assert abs(float(filled[5, 5]) - float(plateau)) <= 1e-3


# ------------------------------------------------------------------ incise (T/ImplicitIncisionTest.kt)

def _three_cells(outlet_m, middle_m, head_m, courants, lake=False):
    """The 16x16 fixtures of T/ImplicitIncisionTest.kt:355-419 and 422-470: three cells in row 8
    running east into the sea at column 2."""
    p = oracle.default_params(16, 16, 1)
    _, cc, pond = oracle.rates(p)
    n = 256
    row = 8 * 16
    sea, a, b, c = row + 2, row + 3, row + 4, row + 5
    shoreline = field_at_altitude(0.0)
    land_range = f32(6000.0) / f32(16000.0)
    is_land = np.zeros(n, np.uint8)
    dirs = np.full(n, -1, np.int32)
    surface = np.full(n, field_at_altitude(-1.0), np.float32)
    for cell, metres, rec in ((a, outlet_m, sea), (b, middle_m, a), (c, head_m, b)):
        is_land[cell] = 1
        dirs[cell] = rec
        surface[cell] = field_at_altitude(metres)
    relative = ((surface - shoreline) / land_range).astype(np.float32)
    ground = relative.copy()
    if lake:
        ground[b] = relative[a]
        assert ground[b] - relative[b] > pond
    discharge = np.zeros(n, np.float32)
    for cell, courant in zip((a, b, c), courants):
        discharge[cell] = f32((courant / float(cc)) ** 2)
    before = surface.copy()
    oracle.incise(p, np.array([c, b, a], np.int32), dirs, is_land, ground, relative, discharge, f32(1.0),
                  land_range, shoreline, np.ones(n, np.float32), surface)
    return p, cc, before, surface, (a, b, c), discharge


def test_incise_cell_below_receiver_cut_once_receiver_is():
    """T/ImplicitIncisionTest.kt:355-419: the middle cell, 10 m below its receiver, is cut by
    exactly F/(1+F) of its drop to the receiver's new height, within 0.01 m."""
    _, cc, before, after, (mouth, below, _), discharge = _three_cells(100.0, 90.0, 300.0, (9.0, 1.0, 1.0))
    mouth_after = altitude_at_field(after[mouth])
    below_before = altitude_at_field(before[below])
    below_after = altitude_at_field(after[below])
    courant = float(f32(f32(cc * np.sqrt(f32(discharge[below] / f32(1.0)))) * f32(1.0)) / f32(1.0))
    expected = mouth_after + (below_before - mouth_after) / (1.0 + courant)
    assert before[below] < before[mouth]
    assert mouth_after < below_before
    assert abs(below_after - expected) <= 0.01


@pytest.mark.parametrize("outlet_courant,bed,want", [
    (9.0, 70.0, (10.0, 16.0, 26.4)),
    (0.25, 50.0, (80.0, 50.0, 84.0)),
])
def test_incise_lake_falls_with_its_outlet(outlet_courant, bed, want):
    """T/ImplicitIncisionTest.kt:422-496: the draining lake (outlet 10.0, bed 16.0, inflow 26.4 m)
    and the standing lake (80.0, 50.0, 84.0 m), each within 0.01 m."""
    _, _, _, after, cells, _ = _three_cells(100.0, bed, 120.0, (outlet_courant, 9.0, 9.0), lake=True)
    for cell, w in zip(cells, want):
        assert abs(altitude_at_field(after[cell]) - w) <= 0.01, (cell, altitude_at_field(after[cell]), w)


@pytest.mark.parametrize("erodibility", [1e-7, 1e-6, 5e-5])
def test_incise_plane_round_matches_recursion(erodibility):
    """T/ImplicitIncisionTest.kt:510-632: one production round (cut, fill, facet routing, flats,
    accumulation, drainage order, implicit incision) on a 128x128 plane falling west at 1 m/km
    leaves every cell of the middle row where the recursion (z + F z_r')/(1 + F) puts it, and
    removes F/(1+F) of each drop, within 0.01 m."""
    side = 128
    land_cols = side // 4
    p = oracle.default_params(side, side, 7, sea_level=float(f32(1.0 - land_cols / side)), hydraulic_rounds=1,
                              bedrock_erodibility_per_year=erodibility, lowstand_metres=0.0)
    first = (side - land_cols) // 2
    crest = first + land_cols - 1
    cell_w_km = 40075.0 / side
    cell_w_m = cell_w_km * 1000.0
    fall = 1.0 / 1000.0 * cell_w_m
    ground = np.empty((side, side), np.float32)
    for row in range(side):
        for col in range(side):
            up = col - first + 1
            if 1 <= up <= land_cols:
                ground[row, col] = field_at_altitude(f32(up * fall))
            else:
                ground[row, col] = field_at_altitude(f32(-1.0) - f32(row * side + col) * f32(0.01))
    shoreline, _, _, land_count = oracle.percentile_cut(ground, float(p.sea_level))
    shore_m = altitude_at_field(shoreline)
    out = oracle.erode_stage(p, ground, thermal=False)["height"]
    row = side // 2
    land_area = (1.0 - float(p.sea_level)) * 40075.0 ** 2 * 0.5
    cell_area = land_area / land_count * 1e6
    years = 336476.4
    failures = []
    receiver_after = shore_m
    smalls = larges = 0
    for idx, col in enumerate(range(first, crest + 1)):
        catchment = 1 if col == crest else crest - col
        F = erodibility * years * math.sqrt(catchment * cell_area) / cell_w_m
        smalls += F < 0.1
        larges += F > 10.0
        before = altitude_at_field(ground[row, col])
        after = altitude_at_field(out[row, col])
        grade = shore_m if col == crest else receiver_after
        base_after = shore_m if (col == crest or idx == 0) else altitude_at_field(out[row, col - 1])
        predicted = (before + F * grade) / (1.0 + F)
        receiver_after = predicted
        removed = before - after
        law = F / (1.0 + F) * (before - base_after)
        if abs(removed - law) > 0.01 or abs(after - predicted) > 0.01:
            failures.append((col, before, after, predicted, F))
    assert not failures, failures[:5]
    if erodibility == 1e-7:
        assert smalls > 0
    if erodibility == 5e-5:
        assert larges > 0


# ------------------------------------------------------------------ thermal (T/ErosionSkipTest, ThermalAspectTest)

def test_thermal_skip_is_bit_identical():
    """T/ErosionSkipTest.kt:28-49: the sweeps with and without the settled-tile skip are
    bit-identical (on a seeded synthetic world at 256 rows in place of the reference's plates)."""
    W, H = 512, 256
    h, up, _ = synthetic.world(W, H, seed=234475)
    h = np.clip(h + up / 3.0 * 0.05, 0, None).astype(np.float32)
    p = oracle.default_params(W, H, 234475)
    lim, sweeps = oracle.thermal_limits(p)
    assert sweeps == 24
    a = oracle.thermal_sweep(h, lim, sweeps, skip=True)
    b = oracle.thermal_sweep(h, lim, sweeps, skip=False)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert not np.array_equal(a, h)


@pytest.mark.parametrize("width", [256, 512])
def test_thermal_aspect_settles_at_critical_slope(width):
    """T/ThermalAspectTest.kt:33-76: a 6,000 m mesa (radius 1,200 km) on a 9,000 m plain of a
    12,000 km planet, 1,500 sweeps: the steepest settled fall per step kind lies within
    [0.75, 1.01] x 60 m/km."""
    H = 256
    planet = 12000.0
    p = oracle.default_params(width, H, 1, world_width_km=planet)
    lim, _ = oracle.thermal_limits(p)
    cw = planet / width
    ch = planet * 0.5 / H
    cols = np.arange(width)[None, :]
    rows = np.arange(H)[:, None]
    on_top = np.sqrt(((cols - width // 2) * cw) ** 2 + ((rows - H // 2) * ch) ** 2) < 1200.0
    mesa = (np.where(on_top, 9000.0 + 6000.0, 9000.0).astype(np.float32) / f32(16000.0)).astype(np.float32)
    s = oracle.thermal_sweep(mesa, lim, 1500).astype(np.float64) * 16000.0
    inner = s[1:-1, 1:-1]
    ew = np.abs(s[1:-1, 2:] - inner).max() / cw
    ns = np.abs(s[2:, 1:-1] - inner).max() / ch
    dg = np.abs(s[2:, 2:] - inner).max() / math.sqrt(cw * cw + ch * ch)
    for fall in (ew, ns, dg):
        assert 60.0 * 0.75 <= fall <= 60.0 * 1.01, (ew, ns, dg)


# ------------------------------------------------------------------ routing (T/RoutingGroundTest.kt)

@pytest.mark.parametrize("row_scale", [0.5, 1.0])
def test_routing_planes_run_down_their_bearing(row_scale):
    """T/RoutingGroundTest.kt:36-79: on 256x256 planes at twelve bearings the mean routed step
    points down the plane on the ground within 2 degrees (interior cells, margin 16)."""
    side, margin = 256, 16
    cols = np.arange(side)[None, :].astype(np.float64)
    rows = np.arange(side)[:, None].astype(np.float64)
    land = np.ones((side, side), np.uint8)
    worst = 0.0
    for deg in (0.0, 10.0, 26.565, 30.0, 45.0, 60.0, 75.0, 90.0, 120.0, 135.0, 200.0, 300.0):
        fall = deg * math.pi / 180.0
        plane = (0.5 - 1e-3 * (cols * math.cos(fall) + rows * row_scale * math.sin(fall))).astype(np.float32)
        rec, _ = oracle.flow_directions(land, plane, plane, 7, row_scale, 8, by_facet=True, over_potential=False)
        inner = rec[margin:side - margin, margin:side - margin]
        cc = np.broadcast_to(np.arange(margin, side - margin)[None, :], inner.shape)
        rr = np.broadcast_to(np.arange(margin, side - margin)[:, None], inner.shape)
        ok = inner >= 0
        east = float(((inner % side) - cc)[ok].sum())
        south = float((((inner // side) - rr) * row_scale)[ok].sum())
        routed = math.degrees(math.atan2(south, east))
        err = (routed - deg + 180.0) % 360.0 - 180.0
        worst = max(worst, abs(err))
    assert worst <= 2.0


# ------------------------------------------------------------------ flats and the forest (T/FlatCourseTest.kt)

def test_flats_keep_a_lower_neighbour_and_the_network_is_a_forest():
    """T/FlatCourseTest.kt:82-174 on a synthetic world: every flat lays its potential (flatsKept
    == 0), every land cell has a receiver strictly lower on the routing surface, and the drainage
    order reaches every land cell (no cycle)."""
    W, H = 256, 128
    h, up, _ = synthetic.world(W, H, seed=42)
    shoreline, is_land, rel, land = oracle.percentile_cut(h, 0.70)
    filled = oracle.fill_depressions(is_land, rel)
    rec, surf, counts = oracle.flow_directions(is_land, rel, filled, 42, 0.5, 214, want_surface=True)
    assert counts[0] > 0 and counts[1] == 0
    lr = np.flatnonzero(is_land.ravel())
    r = rec.ravel()[lr]
    # Land on the polar rows is an outlet of the fill and may drain off the map (-1).
    interior = (lr >= W) & (lr < W * (H - 1))
    assert (r[interior] >= 0).all()
    has = r >= 0
    assert (surf.ravel()[r[has]] < surf.ravel()[lr[has]]).all()
    r = np.where(has, r, 0)
    order = oracle.drainage_order(is_land, rec, land)
    assert sorted(order.tolist()) == lr.tolist()
    pos = np.empty(W * H, np.int64)
    pos[order] = np.arange(land)
    to_land = has & (is_land.ravel()[r] == 1)
    assert (pos[lr[to_land]] < pos[r[to_land]]).all()


def test_accumulate_sums_weights_down_the_forest():
    """FlowRouting.accumulate (P/FlowRouting.kt:485-511): on integer weights the float sums are
    exact, so each mouth's area is its catchment's cell count and the land total is conserved."""
    W, H = 128, 64
    h, _, _ = synthetic.world(W, H, seed=9)
    _, is_land, rel, land = oracle.percentile_cut(h, 0.70)
    filled = oracle.fill_depressions(is_land, rel)
    rec, _ = oracle.flow_directions(is_land, rel, filled, 9, 0.5, 214)
    area = oracle.accumulate(is_land, rec, land, np.ones((H, W), np.float32))
    flat_rec = rec.ravel()
    il = is_land.ravel().astype(bool)
    mouths = [c for c in np.flatnonzero(il) if flat_rec[c] < 0 or not il[flat_rec[c]]]
    assert abs(sum(float(area.ravel()[m]) for m in mouths) - land) < 1e-3


def test_one_round_asks_what_the_stream_power_law_and_the_clock_say():
    """T:ErosionUnitsTest.kt:163-247: a 32-column plane falling due west at 1 m/km into a deep sea on a
    128 x 128 map a quarter land, one round, no climate, deposition, notch, flexure or relaxation. The
    law's rate the pass spends on a cell k cells below the crest, F times the drop to its receiver as
    the pass found it, is K T sqrt(k A) S to a thousandth, with F from 0.24 at one cell to 1.3 at
    thirty. F is read back from the cut: after = base + (h - base) / (1 + F), the base the receiver's
    height after the pass."""
    import math
    W = H = 128
    land_cols = W // 4
    p = oracle.default_params(W, H, seed=7, sea_level=np.float32(1.0 - land_cols / W), hydraulic_rounds=1,
                              climate_feed=0, profile=0, lowstand_metres=0.0)
    f32 = np.float32
    span = f32(6000.0) + f32(10000.0)

    def field_at(m):   # WorldScale.fieldAtAltitude
        return f32((f32(m) + f32(10000.0)) / span)

    fall = f32(1.0 * 40075.0 / W)
    first = (W - land_cols) // 2
    g = np.empty((H, W), np.float32)
    for r in range(H):
        for c in range(W):
            up = c - first + 1
            g[r, c] = (field_at(f32(up) * fall) if 1 <= up <= land_cols
                       else field_at(f32(-4000.0) - f32(r * W + c) * f32(0.01)))
    _, _, _, n = oracle.percentile_cut(g, p.sea_level, 0.0)
    assert 0 <= n - land_cols * H <= 1   # SEA_CELLS_READ_AS_LAND
    out = oracle.erode_stage(p, g, thermal=False, want=("receivers",))
    after, rec = out["height"].ravel(), out["receivers"].ravel()
    crest = first + land_cols - 1
    cell_area = (1.0 - float(p.sea_level)) * 40075.0 ** 2 * 0.5 / n * 1e6
    worst, fs = 0.0, []
    for k in range(1, 31):
        law = float(p.bedrock_erodibility_per_year) * p.years_per_hydraulic_round * math.sqrt(k * cell_area) * 1e-3
        for row in (H // 4, H // 2, 3 * H // 4):
            c = row * W + crest - k
            r = rec[c]
            assert r == c - 1   # due west
            h0, a, b, b0 = float(g.ravel()[c]), float(after[c]), float(after[r]), float(g.ravel()[r])
            F = (h0 - b) / (a - b) - 1.0
            worst = max(worst, abs(F * (h0 - b0) * float(span) / law - 1.0))
            fs.append(F)
    assert worst <= 1e-3, worst
    assert abs(min(fs) - 0.24) < 0.01 and abs(max(fs) - 1.3) < 0.01


STEADY_SIDE = 64


def _steady_state(uplift_mm, zone_of, rock_of, rain_of):
    """ImplicitIncisionTest.steadyState (T:ImplicitIncisionTest.kt:640-752): a 64 x 64 island lifted
    every round and cut by the routing and the incision (no thermal pass, deposition or notch) until
    no land cell moves by more than 1e-3 of a round's uplift, the routing taken afresh for 1000 rounds
    and then held. Returns (rounds, {zone: (channel cells, concavity, median steepness in m)})."""
    import math
    f32 = np.float32
    side = STEADY_SIDE
    p = oracle.default_params(side, side, seed=11, climate_feed=0, profile=0)
    N = side * side
    span = f32(16000.0)
    land_range, sea_half = f32(6000.0) / span, f32(10000.0) / span
    shoreline = f32((f32(0.0) + f32(10000.0)) / span)   # WorldScale.fieldAtAltitude(0)
    cell = np.arange(N)
    row, col = cell // side, cell % side
    land = ((row >= 2) & (row < side - 2) & (col >= 3) & (col < side - 3)).astype(np.uint8)
    n = int(land.sum())
    zones = np.array([zone_of(r) for r in row])
    erod = np.array([rock_of(z) for z in zones], np.float32)
    rain = np.array([rain_of(z) for z in zones], np.float32)
    rain_sum = 0.0
    for c in range(N):   # the stage's sequential double sum over the land
        if land[c]:
            rain_sum += float(rain[c])
    weight = (rain / f32(rain_sum / n)).astype(np.float32)
    up = f32(f32(uplift_mm / 1000.0 * p.years_per_hydraulic_round) / span)
    rough = ((cell.astype(np.int64) * 2654435761) >> 7) % 1000
    metres = (f32(1.0) + (f32(5.0) * rough.astype(np.float32)) / f32(1000.0)).astype(np.float32)
    surface = np.where(land == 1, ((metres + f32(10000.0)) / span).astype(np.float32),
                       f32((f32(-100.0) + f32(10000.0)) / span)).astype(np.float32)
    lm = land.reshape(side, side)
    r = 0.5   # cellHeightInCellWidths of a square grid
    rounds = 0
    while True:
        rounds += 1
        assert rounds <= 20000, "no balance in 20000 rounds"
        prev = surface.copy()
        surface[land == 1] = (surface[land == 1] + up).astype(np.float32)
        rel = np.where(land == 1, (surface - shoreline) / land_range,
                       (surface - shoreline) / sea_half).astype(np.float32).reshape(side, side)
        filled = oracle.fill_depressions(lm, rel)
        if rounds <= 1000:
            rec, _ = oracle.flow_directions(lm, rel, filled, 11, r, 214)
            disc = oracle.accumulate(lm, rec, n, weight.reshape(side, side))
            order = oracle.drainage_order(lm, rec, n)
        oracle.incise(p, order, rec, land, filled, rel, disc, f32(n), land_range, shoreline, erod, surface)
        if rounds > 1000 and np.abs(surface[land == 1] - prev[land == 1]).max() < f32(1e-3) * up:
            break
    upstream = oracle.accumulate(lm, rec, n, np.ones((side, side), np.float32)).ravel()
    land_area = (1.0 - float(f32(0.71))) * 40075.0 ** 2 * 0.5 * 1e6
    cell_m = 40075.0 / side * 1000.0
    step_ns, step_diag = float(f32(r)), float(f32(math.sqrt(1.0 + r * r)))
    recf = rec.ravel()
    out = {}
    for z in sorted(set(zones)):
        in_zone = oracle.accumulate(lm, rec, n, (zones == z).astype(np.float32).reshape(side, side)).ravel()
        la, ls, steep = [], [], []
        for c in range(N):
            if not land[c] or zones[c] != z or upstream[c] < 4 or in_zone[c] != upstream[c]:
                continue
            d = recf[c]
            if d < 0:
                continue
            fall = float(f32(surface[c] - (surface[d] if land[d] else shoreline))) * 16000.0
            if fall <= 0.0:
                continue
            same_row, same_col = c // side == d // side, c % side == d % side
            step = step_diag if not same_row and not same_col else (step_ns if not same_row else 1.0)
            slope = fall / (step * cell_m)
            area = float(upstream[c]) / n * land_area
            la.append(math.log(area))
            ls.append(math.log(slope))
            steep.append(slope * math.sqrt(area))
        la, ls = np.array(la), np.array(ls)
        theta = -np.sum((la - la.mean()) * (ls - ls.mean())) / np.sum((la - la.mean()) ** 2)
        steep.sort()
        out[z] = (len(la), float(theta), steep[len(steep) // 2])
    return rounds, out


def test_at_balance_the_profiles_are_the_laws_across_rock_and_uplift():
    """T:ImplicitIncisionTest.kt:763-820: under uniform uplift the concavity at balance is m / n = 0.5
    and the steepness U / (K e) in each of two rocks (e 0.5 and 2), and doubles with the uplift, each
    to a hundredth."""
    rock = {"hard": 0.5, "soft": 2.0}
    res = {}
    for uplift in (0.1, 0.2):
        _, out = _steady_state(uplift, lambda r: "hard" if r < STEADY_SIDE // 2 else "soft", rock.get, lambda z: 1.0)
        res[uplift] = out
        for z, e in rock.items():
            cells, theta, steep = out[z]
            assert cells > 50
            assert abs(theta - 0.5) <= 0.01, (uplift, z, theta)
            assert abs(steep / (uplift / 1000.0 / (1e-6 * e)) - 1.0) <= 0.01, (uplift, z, steep)
    for z in rock:
        assert abs(res[0.2][z][2] / res[0.1][z][2] / 2.0 - 1.0) <= 0.01
    assert abs(res[0.1]["hard"][2] / res[0.1]["soft"][2] / 4.0 - 1.0) <= 0.01


def test_at_balance_the_steepness_falls_as_the_square_root_of_the_rain():
    """T:ImplicitIncisionTest.kt:822-857: a wet zone with four times the dry zone's rain, one rock: the
    concavity stays 0.5 in both and the wet steepness is half the dry, each to a hundredth."""
    _, out = _steady_state(0.1, lambda r: "wet" if r < STEADY_SIDE // 2 else "dry", lambda z: 1.0,
                           lambda z: 4.0 if z == "wet" else 1.0)
    for z in ("wet", "dry"):
        assert abs(out[z][1] - 0.5) <= 0.01, (z, out[z])
    assert abs(out["wet"][2] / out["dry"][2] / 0.5 - 1.0) <= 0.01, out


def _knickpoint(southward, rounds, share):
    """ImplicitIncisionTest.knickpoint (T:ImplicitIncisionTest.kt:870-935): a 40-cell-width profile
    into the sea along a row or down a column of a 128 x 128 grid, a break in slope (60 m a cell width
    below, 20 above) 12 cell widths from the sea, the same F = 2 along a row on both bearings, the sea
    lowered each round with the lower reach, cut by the incision for `rounds` rounds of `share` of the
    clock. Returns (sharp-break distance, steepest-change point, smear) in cell widths."""
    f32 = np.float32
    lower, upper, knick, length, courant_ew = 60.0, 20.0, 12.0, 40, 2.0
    span = f32(16000.0)

    def field_at(m):
        return f32((f32(m) + f32(10000.0)) / span)

    side = 128
    p = oracle.default_params(side, side, seed=3)
    p.years_per_hydraulic_round = p.years_per_hydraulic_round * share
    courant = oracle.rates(p)[1]
    step = float(f32(0.5)) if southward else 1.0
    cells = int(length / step)
    N = side * side
    start = 20 * side + 64 if southward else 64 * side + 4
    stride = side if southward else 1
    prof = [start + (i + 1) * stride for i in range(cells)]
    land = np.zeros(N, np.uint8)
    dirs = np.full(N, -1, np.int32)
    for i, c in enumerate(prof):
        land[c] = 1
        dirs[c] = start if i == 0 else prof[i - 1]
    surface = np.full(N, field_at(0.0), np.float32)
    for i, c in enumerate(prof):
        g = (i + 1) * step
        m = 1000.0 + lower * g if g <= knick else 1000.0 + lower * knick + upper * (g - knick)
        surface[c] = field_at(f32(m))
    root = courant_ew / (float(courant) / share)
    disc = np.full(N, f32(root * root), np.float32)
    erod = np.ones(N, np.float32)
    order = np.array(prof[::-1], np.int32)
    land_half = f32(6000.0) / span
    sea = 1000.0
    for _ in range(rounds):
        sea -= courant_ew * share * lower
        rel = ((surface - field_at(0.0)) / land_half).astype(np.float32)
        oracle.incise(p, order, dirs, land, rel, rel, disc, f32(1.0), land_half, field_at(f32(sea)), erod, surface)
    h = np.array([float(f32(surface[c] * span - f32(10000.0))) for c in prof])   # altitudeAtField
    sharp = ((h[-1] - sea) - upper * cells * step) / (lower - upper)
    slopes = np.array([(h[i] - (sea if i == 0 else h[i - 1])) / step for i in range(cells)])
    mids = (np.arange(cells) + 0.5) * step

    def crossing(s):
        level = upper + (lower - upper) * s
        for i in range(1, cells):
            if slopes[i - 1] >= level > slopes[i]:
                a = (slopes[i - 1] - level) / (slopes[i - 1] - slopes[i])
                return mids[i - 1] + a * (mids[i] - mids[i - 1])
        return float("nan")

    return sharp, crossing(0.5), crossing(0.1) - crossing(0.9)


def test_a_knickpoint_retreats_as_far_north_south_as_east_west_and_in_two_half_rounds():
    """T:ImplicitIncisionTest.kt:937-996: the break, read as a sharp break of equal relief, retreats the
    law's F = 2 cell widths a round along a row, to 1e-3, and as far down a column and in two half
    rounds; read as the steepest-change point, the four retreats agree to a cell width."""
    start, ns_start = _knickpoint(False, 0, 1.0), _knickpoint(True, 0, 1.0)
    ew, ns = _knickpoint(False, 1, 1.0), _knickpoint(True, 1, 1.0)
    ewh, nsh = _knickpoint(False, 2, 0.5), _knickpoint(True, 2, 0.5)
    retreat = ew[0] - start[0]
    assert retreat > 0.0 and abs(retreat - 2.0) <= 1e-3, retreat
    for other in (ns[0] - ns_start[0], ewh[0] - start[0], nsh[0] - ns_start[0]):
        assert abs(other - retreat) <= 1e-3, (other, retreat)
    mid = ew[1] - start[1]
    for other in (ns[1] - ns_start[1], ewh[1] - start[1], nsh[1] - ns_start[1]):
        assert abs(other - mid) <= 1.0, (other, mid)


def _facet_share(fall, rs):
    """RoutingGroundTest.facetShare (T:RoutingGroundTest.kt:214-228): the share of a plane's steps the
    facet rule sends to the diagonal, and whether that facet's cardinal is a column step."""
    import math
    off = math.atan2(abs(math.sin(fall)), abs(math.cos(fall)))
    if off <= math.atan2(rs, 1.0):
        return math.tan(off) / rs, False
    return rs * math.tan(math.pi / 2 - off), True


@pytest.mark.parametrize("rs,want", [(0.5, (44.87, 15.31, 39.82)), (1.0, (27.94, 27.94, 44.13))])
def test_the_facet_rule_takes_each_bearing_as_often_as_its_geometry_says(rs, want):
    """T:RoutingGroundTest.kt:84-213: on 128 x 128 planes at 360 bearings and three seeds, the facet
    rule's Rho8 draws take a column, a row and a diagonal as often as the facets' geometry says (44.87,
    15.31 and 39.82% on cells half as tall as wide; 27.94, 27.94 and 44.13% on square ones), each
    within four standard errors, and each plane's mean step points down it within 4.5."""
    import math
    side, margin, bearings, seeds = 128, 16, 360, (7, 42, 1234)
    taken, expected = np.zeros(3), np.zeros(3)
    per = np.zeros((len(seeds), 3, side * side))
    worst = 0.0
    land = np.ones((side, side), np.uint8)
    cols = np.arange(side)[None, :].astype(np.float64)
    rows = np.arange(side)[:, None].astype(np.float64)
    inner = np.zeros((side, side), bool)
    inner[margin:side - margin, margin:side - margin] = True
    index = np.arange(side * side).reshape(side, side)[inner]
    for si, seed in enumerate(seeds):
        for i in range(bearings):
            deg = (i + 0.5) * 360.0 / bearings
            fall = math.radians(deg)
            plane = (0.5 - 1e-3 * (cols * math.cos(fall) + rows * rs * math.sin(fall))).astype(np.float32)
            rec, _ = oracle.flow_directions(land, plane, plane, seed, rs, 8)
            share, colwise = _facet_share(fall, rs)
            t = rec[inner]
            ok = t >= 0
            t, c = t[ok], index[ok]
            dc, dr = (t % side) - (c % side), (t // side) - (c // side)
            way = np.where(dc == 0, 0, np.where(dr == 0, 1, 2))
            for k in range(3):
                taken[k] += (way == k).sum()
            np.add.at(per[si], (way, c), 1.0)
            per[si, 2, c] -= share
            per[si, 0 if colwise else 1, c] -= 1 - share
            expected[2] += len(t) * share
            expected[0 if colwise else 1] += len(t) * (1 - share)
            x, y = dc.astype(np.float64), dr * rs
            mx, my = x.mean(), y.mean()
            err = (math.degrees(math.atan2(my, mx)) - deg + 180.0) % 360.0 - 180.0
            ax, ay = -math.sin(fall), math.cos(fall)
            var = (ax * ax * ((x * x).mean() - mx * mx) + ay * ay * ((y * y).mean() - my * my)
                   + 2 * ax * ay * ((x * y).mean() - mx * my))
            sigma = math.sqrt(max(var, 0.0) / len(t)) / math.hypot(mx, my) * 180.0 / math.pi
            worst = max(worst, abs(err) / sigma if sigma > 0 else (0.0 if abs(err) < 1e-9 else math.inf))
    cells = taken.sum()
    for k in range(3):
        assert abs(100.0 * expected[k] / cells - want[k]) < 0.01
        assert abs(taken[k] - expected[k]) <= 4.0 * math.sqrt((per[:, k, :] ** 2).sum()), k
    assert worst <= 4.5, worst


@pytest.mark.parametrize("aspect", [0.25, 0.5, 1.0, 2.0])
def test_the_potential_across_a_flat_is_round_on_the_ground(aspect):
    """T:RoutingGroundTest.kt:239-300: a flat of radius 50 cell widths, one flat-gradient step of fill
    over its floor, its outlet one lower cell at the centre and a rim far above: laid (one flat, none
    kept), and at 10, 20, 30 and 40 cell widths from the outlet the north-south quarters' mean
    potential is the east-west quarters' within a tenth, on cells a quarter to twice as tall as wide."""
    import math
    columns = 128
    rows = int(math.ceil(128 / aspect))
    cc, cr = columns // 2, rows // 2
    across = (np.arange(columns)[None, :] - cc).astype(np.float64)
    down = (np.arange(rows)[:, None] - cr) * aspect
    dist = np.sqrt(across ** 2 + down ** 2)
    ground = np.where(dist <= 50.0, np.float32(0.0), np.float32(10.0)).astype(np.float32)
    filled = np.where(dist <= 50.0, np.float32(1e-3), np.float32(10.0)).astype(np.float32)
    ground[cr, cc] = filled[cr, cc] = np.float32(-1.0)
    land = np.ones((rows, columns), np.uint8)
    _, surf, counts = oracle.flow_directions(land, ground, filled, 1, aspect, 8, want_surface=True)
    assert counts[0] == 1 and counts[1] == 0, counts   # one flat, laid
    floor = surf[cr, cc + 1]
    for radius in (10.0, 20.0, 30.0, 40.0):
        ring = np.abs(dist - radius) <= 0.75 * max(1.0, aspect)
        ew = ring & (np.abs(across) > np.abs(down))
        ns = ring & ~(np.abs(across) > np.abs(down))
        ratio = (surf[ns] - floor).mean() / (surf[ew] - floor).mean()
        assert abs(ratio - 1.0) <= 0.10, (aspect, radius, ratio)


def test_the_flats_weights_are_positive_and_isotropic_on_cells_of_every_shape():
    """T:RoutingGroundTest.kt:313-332: for r = 2^k, k from -8 to 8, every weight of the flat Laplacian
    is positive and e + 2d = r^2 (n + 2d) to 1e-9."""
    for k in range(-8, 9):
        r = 2.0 ** k
        ew, ns, d = oracle.flat_stencil(r)
        assert ew > 0 and ns > 0 and d > 0, (r, ew, ns, d)
        a, b = ew + 2.0 * d, r * r * (ns + 2.0 * d)
        assert abs(a - b) <= 1e-9 * a, (r, a, b)


def test_the_sea_covers_the_share_of_the_planet_the_slider_asks_for():
    """T:SeaShareTest.kt:26-58: ground falling from the equator to both poles on a 512 x 256 map, half
    the planet asked for: the percentile cut drowns half the planet's area (the ground poleward of 30
    degrees) to 1e-3, where a cut by the map's cells would drown 0.29 of it."""
    import math
    cols, rows = 512, 256
    lat = 90.0 - (np.arange(rows) + 0.5) * 180.0 / rows
    h = (-np.abs(lat)[:, None] + np.arange(cols)[None, :] * 1e-4).astype(np.float32)
    shoreline, _, _, _ = oracle.percentile_cut(h, 0.5, 0.0)
    weight = np.cos(np.radians(lat))[:, None] * np.ones((1, cols))

    def share(mask):
        return float((weight * mask).sum() / weight.sum())

    drowned = share(h < np.float32(shoreline))
    by_cells = np.sort(h.ravel())[int(h.size * 0.5)]
    assert abs(drowned - 0.5) <= 1e-3, drowned
    assert abs(share(h < by_cells) - 0.5) > 0.1
