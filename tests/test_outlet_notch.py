"""The outlet notch of profile P1: HydraulicErosion.breach (P/HydraulicErosion.kt:1931-2171) and the
closing breach (P/HydraulicErosion.kt:1404-1442).

The oracle is pinned to the reference's own case of a basin whose margin shelves
(T/OutletIncisionTest.kt:282-387, constants :740-761), rebuilt from that test's constants, and to
the notch's exact invariants; the GPU (cg_breach, and the stage with profile P1) is then held to the
oracle bit for bit. P = worldgen/src/commonMain/kotlin/com/cartogenesis/worldgen/pipeline,
T = worldgen/src/jvmTest/kotlin/com/cartogenesis/worldgen.
"""
import numpy as np
import pytest

import oracle
from cartogenesis_gb300 import synthetic

f32 = np.float32
LATTICE = 214   # FlowRouting.smoothFieldLatticeColumns of the 40075 km world

# T/OutletIncisionTest.kt:740-761
SHELF_GRID = 128
SHELF_SEA_COLUMNS = 4
SHELF_SEA_DEPTH_METRES = f32(600)
SHELF_LIP_ROW = 64
SHELF_LIP_COLUMN = 24
SHELF_LIP_METRES = f32(600)
SHELF_BASIN_ROWS = range(50, 79)
SHELF_MARGIN_COLUMNS = range(25, 33)
SHELF_CORE_COLUMNS = range(33, 51)
SHELF_MARGIN_NEAR_RIM_METRES = f32(18)
SHELF_MARGIN_SHELVING_METRES = f32(2)
SHELF_CORE_DEPTH_METRES = f32(30)
SHELF_WALL_METRES = f32(300)
OUTFLOW_POWER_METRES = f32(10)


def bits(a):
    return a.view(np.uint32)


def shelf_land():
    col = np.arange(SHELF_GRID * SHELF_GRID) % SHELF_GRID
    return (col >= SHELF_SEA_COLUMNS).astype(np.uint8).reshape(SHELF_GRID, SHELF_GRID)


def shelved_basin(fall_per_cell):
    """The test's terrain in metres, over highestLandMetres, with the Kotlin float steps."""
    land = shelf_land()
    out = np.empty((SHELF_GRID, SHELF_GRID), np.float32)
    first, last = SHELF_MARGIN_COLUMNS[0], SHELF_MARGIN_COLUMNS[-1]
    for row in range(SHELF_GRID):
        for col in range(SHELF_GRID):
            if not land[row, col]:
                m = -SHELF_SEA_DEPTH_METRES
            elif row == SHELF_LIP_ROW and col == SHELF_LIP_COLUMN:
                m = SHELF_LIP_METRES
            elif row == SHELF_LIP_ROW and col < SHELF_LIP_COLUMN:
                m = f32(SHELF_LIP_METRES - f32(fall_per_cell * f32(SHELF_LIP_COLUMN - col)))
            elif row in SHELF_BASIN_ROWS and col in SHELF_MARGIN_COLUMNS:
                m = f32(f32(SHELF_LIP_METRES - SHELF_MARGIN_NEAR_RIM_METRES) -
                        f32(f32(SHELF_MARGIN_SHELVING_METRES * f32(col - first)) / f32(last - first)))
            elif row in SHELF_BASIN_ROWS and col in SHELF_CORE_COLUMNS:
                m = f32(SHELF_LIP_METRES - SHELF_CORE_DEPTH_METRES)
            else:
                m = f32(f32(SHELF_LIP_METRES + SHELF_WALL_METRES) + f32(col))
            out[row, col] = f32(m / f32(6000))
    return out


def route(relative, seed=7):
    land = shelf_land()
    filled = oracle.fill_depressions(land, relative)
    # WorldGenConfig(seed, 128, 128).cellHeightInCellWidths = 0.5
    flow, _ = oracle.flow_directions(land, relative, filled, seed, 0.5, LATTICE)
    area = oracle.accumulate(land, flow, int(land.sum()), np.ones_like(relative))
    return filled, flow, area


def shelf_case():
    params = oracle.default_params(SHELF_GRID, SHELF_GRID, 7)
    rel_inc, _, _ = oracle.outlet_rates(params)
    land = shelf_land()
    land_cells = f32(land.sum())
    lip = SHELF_LIP_ROW * SHELF_GRID + SHELF_LIP_COLUMN
    _, _, area1 = route(shelved_basin(f32(1)))
    power_per_slope = f32(f32(f32(rel_inc) * f32(1.125)) * np.sqrt(f32(area1.ravel()[lip] / land_cells)))
    fall_per_cell = f32(OUTFLOW_POWER_METRES / f32(power_per_slope * f32(SHELF_GRID)))
    relative = shelved_basin(fall_per_cell)
    filled, flow, area = route(relative)
    power_metres = f32(f32(f32(f32(rel_inc) * f32(1.125)) * np.sqrt(f32(area.ravel()[lip] / land_cells))) *
                       fall_per_cell * f32(SHELF_GRID))
    land_half = f32(f32(6000) / f32(16000))
    shoreline = f32(f32(10000) / f32(16000))
    surface = (shoreline + relative * land_half).astype(np.float32)
    return dict(params=params, land=land, relative=relative, filled=filled, flow=flow, area=area,
                land_cells=float(land_cells), land_half=float(land_half), surface=surface, lip=lip,
                power_metres=float(power_metres))


def test_outlet_rates():
    """HydraulicErosion.Rates (P/HydraulicErosion.kt:246-247, 281-282, 303)."""
    for W, H, reach in ((8192, 4096, 307), (512, 256, 19), (128, 128, 5)):
        p = oracle.default_params(W, H, 1)
        rel_inc, notch, got_reach = oracle.outlet_rates(p)
        inc, _, _ = oracle.rates(p)
        assert rel_inc == f32(f32(f32(inc) * f32(16000)) / f32(6000))
        assert notch == f32(f32(f32(0.0025) * f32(40075.0 / W)) / f32(6000))
        assert got_reach == reach


def test_shelved_basin_notch_lowers_the_lip():
    """T/OutletIncisionTest.kt:282-387: a lake whose margin shelves, the old reading's exit inside the
    margin; one notch lowers the lip by at least half the outflow's power."""
    c = shelf_case()
    assert 0.5 * OUTFLOW_POWER_METRES <= c["power_metres"] <= 1.5 * OUTFLOW_POWER_METRES
    land, rel, fil, flow = c["land"].ravel(), c["relative"].ravel(), c["filled"].ravel(), c["flow"].ravel()
    pond = oracle.rates(c["params"])[2]
    old_spill, old_level = -1, np.float32(np.finfo(np.float32).max)
    for cell in range(land.size):
        if not land[cell] or f32(fil[cell] - rel[cell]) <= pond:
            continue
        r = flow[cell]
        if r < 0 or not land[r] or f32(fil[r] - rel[r]) > pond:
            continue
        if fil[r] < old_level:
            old_level, old_spill = fil[r], r
    assert old_spill >= 0 and old_spill % SHELF_GRID in SHELF_MARGIN_COLUMNS
    relative, ground, surface = c["relative"].copy(), c["filled"].copy(), c["surface"].copy()
    before = relative.ravel()[c["lip"]]
    cells, moved = oracle.breach(c["params"], c["land"], relative, ground, c["flow"], c["area"], c["land_cells"],
                                 c["land_half"], surface)
    lowered = float(before - relative.ravel()[c["lip"]]) * 6000.0
    assert lowered >= 0.5 * OUTFLOW_POWER_METRES, lowered
    assert cells > 0 and moved > 0.0


def routed_world(W, H, seed, sea_level=0.70):
    """One round's routing of a synthetic world, as the rounds route it (unit rain)."""
    h, _, _ = synthetic.world(W, H, seed)
    p = oracle.default_params(W, H, seed, sea_level=sea_level)
    shoreline, land, rel, n = oracle.percentile_cut(h, sea_level)
    filled = oracle.fill_depressions(land, rel)
    flow, _ = oracle.flow_directions(land, rel, filled, seed, 0.5 * W / H, LATTICE)
    area = oracle.accumulate(land, flow, n, np.ones((H, W), np.float32))
    land_half = f32(f32(6000) / f32(16000))
    return dict(params=p, land=land, relative=rel, filled=filled, flow=flow, area=area, land_cells=float(n),
                land_half=float(land_half), surface=h.copy())


def test_breach_cuts_only_down_from_its_lips():
    """The notch's exact invariants: it only lowers; every cell it touches lies on a basin's channel
    below the lip or on its margin; the relative field falls by the amount the surface did, in the
    land's units; dry ground falls with it and a pond's surface does not; nothing is cut below the
    shoreline."""
    c = routed_world(256, 128, 11)
    rel, fil, sur = c["relative"].copy(), c["filled"].copy(), c["surface"].copy()
    cells, moved = oracle.breach(c["params"], c["land"], rel, fil, c["flow"], c["area"], c["land_cells"],
                                 c["land_half"], sur)
    assert cells > 0
    changed = np.flatnonzero(sur.ravel() != c["surface"].ravel())
    assert 0 < changed.size <= cells   # a cell on two basins' channels is cut by each
    assert np.all(sur.ravel()[changed] < c["surface"].ravel()[changed])
    assert np.array_equal(np.flatnonzero(rel.ravel() != c["relative"].ravel()), changed)
    pond = oracle.rates(c["params"])[2]
    was_ponded = (c["filled"] - c["relative"]).ravel() > pond
    fil_changed = np.flatnonzero(fil.ravel() != c["filled"].ravel())
    assert np.array_equal(fil_changed, changed[~was_ponded[changed]])
    assert np.all(rel.ravel()[changed] >= -1e-6)
    removed = (c["surface"].ravel()[changed].astype(np.float64) - sur.ravel()[changed].astype(np.float64))
    assert abs(removed.sum() - moved) <= 1e-9 * max(1.0, moved)
    # Every touched cell is downstream of some basin's lip (on its channel) or upstream of it (margin).
    sw = oracle.spillways(c["land"], c["relative"], c["filled"], c["flow"], pond)
    flow = c["flow"].ravel()
    reach = oracle.outlet_rates(c["params"])[2]
    allowed = set()
    for spill, entry in zip(sw["spill"], sw["entry"]):
        if spill < 0:
            continue
        cell, steps = spill, 0
        while cell >= 0 and c["land"].ravel()[cell] and steps <= 2 * reach + 2:
            allowed.add(int(cell))
            cell, steps = flow[cell], steps + 1
        cell, steps = entry, 0
        while cell >= 0 and cell != spill and steps <= 2 * reach + 2:
            allowed.add(int(cell))
            cell, steps = flow[cell], steps + 1
    assert set(changed.tolist()) <= allowed


def long_margin_case(W=2048, H=1024, seed=7):
    """The shelved basin again, stretched so that one notch cuts a long channel margin: a 30 m deep
    core behind a margin shelving gently from 1 m to 1.5 m below the lip over 46 columns, drained
    through a lip at column 24 and a channel falling 2 m a cell to the sea. Its margin walk from the
    entry to the lip is longer than a warp's 32 cells."""
    row = np.arange(H)[:, None].repeat(W, 1)
    col = np.arange(W)[None, :].repeat(H, 0)
    land = (col >= 4).astype(np.uint8)
    lip_r, lip_c, margin_last, core_last = H // 2, 24, 70, 120
    m = (f32(900) + col.astype(f32)).astype(f32)
    basin = np.abs(row - lip_r) <= 14
    m = np.where(basin & (col >= 25) & (col <= margin_last),
                 f32(599) - f32(0.5) * (col - 25).astype(f32) / f32(margin_last - 25), m)
    m = np.where(basin & (col > margin_last) & (col <= core_last), f32(570), m)
    m = np.where((row == lip_r) & (col < lip_c), f32(600) - f32(2) * (lip_c - col).astype(f32), m)
    m = np.where((row == lip_r) & (col == lip_c), f32(600), m)
    rel = (np.where(land == 0, f32(-600), m).astype(f32) / f32(6000)).astype(f32)
    filled = oracle.fill_depressions(land, rel)
    flow, _ = oracle.flow_directions(land, rel, filled, seed, 0.5 * W / H, LATTICE)
    area = oracle.accumulate(land, flow, int(land.sum()), np.ones((H, W), np.float32))
    land_half = f32(f32(6000) / f32(16000))
    surface = (f32(f32(10000) / f32(16000)) + rel * land_half).astype(np.float32)
    return dict(params=oracle.default_params(W, H, seed), land=land, relative=rel, filled=filled, flow=flow,
                area=area, land_cells=float(land.sum()), land_half=float(land_half), surface=surface)


def test_long_margin_case_poses_the_question():
    """One basin, its entry far up the margin (more than 32 cells of margin walk to the lip, within the
    reach), and a notch that cuts more cells than one warp's chunk."""
    c = long_margin_case()
    pond = oracle.rates(c["params"])[2]
    sw = oracle.spillways(c["land"], c["relative"], c["filled"], c["flow"], pond)
    assert sw["count"] == 1
    flow = c["flow"].ravel()
    cell, steps = sw["entry"][0], 0
    while cell >= 0 and cell != sw["spill"][0]:
        cell, steps = flow[cell], steps + 1
    assert cell == sw["spill"][0] and 32 < steps <= oracle.outlet_rates(c["params"])[2]
    rel, fil, sur = c["relative"].copy(), c["filled"].copy(), c["surface"].copy()
    cells, _ = oracle.breach(c["params"], c["land"], rel, fil, c["flow"], c["area"], c["land_cells"],
                             c["land_half"], sur)
    assert cells > 64


def test_p1_stage_adds_the_notch():
    """Profile P1 runs the notch in every round and the closing breach: it differs from P0, and its
    routing outputs are the closing pass's, a valid drainage of the final field's own cut."""
    W, H, seed = 128, 64, 3
    h, up, rk = synthetic.world(W, H, seed)
    p0 = oracle.erode_stage(oracle.default_params(W, H, seed, sea_level=0.70), h, up, rk)
    p1 = oracle.erode_stage(oracle.default_params(W, H, seed, sea_level=0.70, profile=1), h, up, rk)
    assert not np.array_equal(bits(p0["height"]), bits(p1["height"]))
    land = p1["is_land"].ravel().astype(bool)
    rec = p1["receivers"].ravel()
    assert np.all(rec[~land] == -1)
    assert np.all((rec[land] >= 0) | (rec[land] == -1))
    assert np.all(p1["filled"].ravel()[land] >= p1["relative"].ravel()[land])
    assert p1["order"].ravel()[:land.sum()].min() >= 0


# ------------------------------------------------------------------ GPU parity

@pytest.mark.gpu
def test_gpu_breach_shelf_matches_oracle():
    from cartogenesis_gb300 import ErosionConfig, HydraulicErosion
    c = shelf_case()
    want = [c["relative"].copy(), c["filled"].copy(), c["surface"].copy()]
    cells_want, _ = oracle.breach(c["params"], c["land"], *want[:2], c["flow"], c["area"], c["land_cells"],
                                  c["land_half"], want[2])
    got = [c["relative"].copy(), c["filled"].copy(), c["surface"].copy()]
    cells = HydraulicErosion.breach(ErosionConfig(SHELF_GRID, SHELF_GRID, 7), c["land"], got[0], got[1], c["flow"],
                                    c["area"], c["land_cells"], c["land_half"], got[2])
    assert cells == cells_want
    for g, w in zip(got, want):
        assert np.array_equal(bits(g), bits(w))


@pytest.mark.gpu
def test_gpu_breach_long_margin_matches_oracle():
    """A notch whose margin spans several warp chunks (the warp-parallel cut)."""
    from cartogenesis_gb300 import ErosionConfig, HydraulicErosion
    c = long_margin_case()
    want = [c["relative"].copy(), c["filled"].copy(), c["surface"].copy()]
    cells_want, _ = oracle.breach(c["params"], c["land"], *want[:2], c["flow"], c["area"], c["land_cells"],
                                  c["land_half"], want[2])
    got = [c["relative"].copy(), c["filled"].copy(), c["surface"].copy()]
    cells = HydraulicErosion.breach(ErosionConfig(2048, 1024, 7), c["land"], got[0], got[1], c["flow"], c["area"],
                                    c["land_cells"], c["land_half"], got[2])
    assert cells == cells_want
    for g, w in zip(got, want):
        assert np.array_equal(bits(g), bits(w))


@pytest.mark.gpu
@pytest.mark.parametrize("W,H,seed", [(256, 128, 11), (1024, 512, 4), (2048, 1024, 1)])
def test_gpu_breach_world_matches_oracle(W, H, seed):
    """Many basins, channels shared between them: the waves must give the sequential result."""
    from cartogenesis_gb300 import ErosionConfig, HydraulicErosion
    c = routed_world(W, H, seed)
    want = [c["relative"].copy(), c["filled"].copy(), c["surface"].copy()]
    cells_want, _ = oracle.breach(c["params"], c["land"], *want[:2], c["flow"], c["area"], c["land_cells"],
                                  c["land_half"], want[2])
    got = [c["relative"].copy(), c["filled"].copy(), c["surface"].copy()]
    cells = HydraulicErosion.breach(ErosionConfig(W, H, seed, sea_level=0.70), c["land"], got[0], got[1],
                                    c["flow"], c["area"], c["land_cells"], c["land_half"], got[2])
    assert cells == cells_want and cells > 0
    for g, w in zip(got, want):
        d = np.flatnonzero(bits(g) != bits(w))
        assert d.size == 0, f"{d.size} cells differ, first {d[:6]}"


@pytest.mark.gpu
@pytest.mark.parametrize("W,H,seed", [(64, 32, 5), (256, 128, 42), (512, 256, 1)])
def test_gpu_stage_p1_matches_oracle(W, H, seed):
    from cartogenesis_gb300 import ErosionConfig, ErosionStage
    from test_gpu_stage import compare
    h, up, rk = synthetic.world(W, H, seed)
    got = ErosionStage.apply(ErosionConfig(W, H, seed, sea_level=0.70, profile=1), h, up, rk)
    want = oracle.erode_stage(oracle.default_params(W, H, seed, sea_level=0.70, profile=1), h, up, rk)
    compare(got, want)


@pytest.mark.gpu
def test_gpu_stage_p1_2048x1024_with_weather():
    from cartogenesis_gb300 import ErosionConfig, ErosionStage
    W, H, seed = 2048, 1024, 2
    h, up, rk = synthetic.world(W, H, seed)
    rng = np.random.default_rng(seed)
    rain = rng.uniform(60.0, 2500.0, (H, W)).astype(np.float32)
    keys = ("receivers", "area", "filled", "relative", "is_land")
    got = ErosionStage.apply(ErosionConfig(W, H, seed, sea_level=0.70, profile=1), h, up, rk, rain, want=keys)
    want = oracle.erode_stage(oracle.default_params(W, H, seed, sea_level=0.70, profile=1), h, up, rk, rain,
                              want=keys)
    assert np.array_equal(bits(got.height), bits(want["height"]))
    assert np.array_equal(got.receivers, want["receivers"])
    for k in ("area", "filled", "relative"):
        assert np.array_equal(bits(getattr(got, k)), bits(want[k])), k


@pytest.mark.gpu
def test_gpu_stage_p1_bench_world_8192x4096():
    """The benchmark workload with the outlet notch: 8192 x 4096 cells, 12 rounds and the closing
    breach, every routing output of the closing pass bit for bit (the oracle takes a few minutes)."""
    from cartogenesis_gb300 import ErosionConfig, ErosionStage
    from test_gpu_stage import compare
    W, H, seed = 8192, 4096, 1
    h, up, rk = synthetic.world(W, H, seed, uplift="ridges")
    keys = ("receivers", "area", "filled", "relative", "is_land", "basin_of_cell", "donors")
    got = ErosionStage.apply(ErosionConfig(W, H, seed, sea_level=0.70, profile=1), h, up, rk, want=keys)
    want = oracle.erode_stage(oracle.default_params(W, H, seed, sea_level=0.70, profile=1), h, up, rk, want=keys)
    compare(got, want, order=False)



@pytest.mark.gpu
def test_gpu_breach_without_basins_changes_nothing():
    """A plane falling to the sea has no basin: the notch's early return leaves every array as it was."""
    from cartogenesis_gb300 import ErosionConfig, HydraulicErosion
    W, H = 64, 32
    col = np.arange(W)[None, :].repeat(H, 0)
    land = (col >= 8).astype(np.uint8)
    rel = np.where(land == 1, (col - 7).astype(np.float32) * f32(0.01), f32(-0.5)).astype(np.float32)
    filled = oracle.fill_depressions(land, rel)
    flow, _ = oracle.flow_directions(land, rel, filled, 1, 0.5 * W / H, LATTICE)
    area = oracle.accumulate(land, flow, int(land.sum()), np.ones((H, W), np.float32))
    surface = (f32(0.625) + rel * f32(0.375)).astype(np.float32)
    got = [rel.copy(), filled.copy(), surface.copy()]
    cells = HydraulicErosion.breach(ErosionConfig(W, H, 1), land, got[0], got[1], flow, area, float(land.sum()),
                                    0.375, got[2])
    assert cells == 0
    for g, w in zip(got, (rel, filled, surface)):
        assert np.array_equal(bits(g), bits(w))
