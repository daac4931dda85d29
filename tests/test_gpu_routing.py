"""Each routing function of the round on the GPU against the oracle, on the same inputs.

Integer outputs (masks, receivers, orders, donor counts, basin labels and outlets) must be
identical; float fields must be identical bit for bit (the REF32 mode reproduces the reference's
float arithmetic). The one documented exception is the flats' potential surface, an intermediate
the receivers are read from: its conjugate-gradient dot products are block reductions where the
reference sums sequentially, so it may differ in its last bits (tolerance 1e-12 relative, written
below); the receivers read from it must still be identical.
"""
import numpy as np
import pytest

import oracle
from cartogenesis_gb300 import FlowRouting, SeaLevelStage, synthetic

pytestmark = pytest.mark.gpu

SIZES = [(64, 32, 11), (128, 64, 3), (256, 128, 42), (512, 256, 7)]
SURFACE_RTOL = 1e-12


def bits(a):
    return a.view(np.uint32) if a.dtype == np.float32 else a.view(np.uint64)


def world_cut(W, H, seed, sea_level=0.70, lowstand=0.0):
    h, up, rk = synthetic.world(W, H, seed)
    return h, oracle.percentile_cut(h, sea_level, lowstand)


@pytest.mark.parametrize("W,H,seed", SIZES + [(2048, 1024, 1)])
@pytest.mark.parametrize("sea_level,lowstand", [(0.70, 0.0), (0.71, 0.0075), (0.30, 0.0025)])
def test_percentile_cut(W, H, seed, sea_level, lowstand):
    h, _, _ = synthetic.world(W, H, seed)
    s0, l0, r0, n0 = oracle.percentile_cut(h, sea_level, lowstand)
    s1, l1, r1, n1 = SeaLevelStage.percentile_cut(h, sea_level, lowstand)
    assert np.float32(s0).view(np.uint32) == np.float32(s1).view(np.uint32)
    assert n0 == n1
    assert np.array_equal(l0, l1)
    assert np.array_equal(bits(r0), bits(r1))


def test_percentile_cut_sea_level_sweep():
    """Nineteen sea levels on one 2048 x 1024 world: each moves the bracket to another bin and the
    walk to another cell, so an error in the exact per-bin sums or in the bracket's sum would show
    as a different shoreline in some of them."""
    h, _, _ = synthetic.world(2048, 1024, 23)
    for sea_level in np.linspace(0.05, 0.95, 19):
        s0, l0, r0, n0 = oracle.percentile_cut(h, float(sea_level))
        s1, l1, r1, n1 = SeaLevelStage.percentile_cut(h, float(sea_level))
        assert np.float32(s0).view(np.uint32) == np.float32(s1).view(np.uint32), sea_level
        assert n0 == n1, sea_level


def test_percentile_cut_edges():
    """A flat field (the answer is its height), a field of two levels with ties in the bracket,
    and sea levels 0 and 1."""
    for h in (np.full((16, 32), 0.4, np.float32),
              np.where(np.arange(16 * 32).reshape(16, 32) % 3 == 0, 0.2, 0.7).astype(np.float32)):
        for sl in (0.0, 0.5, 1.0):
            s0, l0, r0, n0 = oracle.percentile_cut(h, sl)
            s1, l1, r1, n1 = SeaLevelStage.percentile_cut(h, sl)
            assert (s0, n0) == (s1, n1) and np.array_equal(l0, l1) and np.array_equal(bits(r0), bits(r1))


@pytest.mark.parametrize("W,H,seed", SIZES + [(2048, 1024, 1)])
def test_fill_depressions(W, H, seed):
    _, (s, land, rel, n) = world_cut(W, H, seed)
    want = oracle.fill_depressions(land, rel)
    got, ties, unresolved = FlowRouting.fill_depressions(land, rel, with_ties=True)
    diff = np.flatnonzero(bits(got) != bits(want))
    assert diff.size == 0, f"{diff.size} cells differ (ties {ties}, unresolved {unresolved}): {diff[:8]}"
    assert unresolved == 0


def test_fill_depression_fixture():
    """T/DepressionFillTest.kt's 32x32 grid: the device fill equals the oracle's bit for bit."""
    land = np.zeros((32, 32), np.uint8)
    elev = np.full((32, 32), np.float32(-0.1), np.float32)
    land[12:20, 12:20] = 1
    elev[12:20, 12:20] = np.float32(-0.2)
    land[3:8, 3:8] = 1
    elev[3:8, 3:8] = np.float32(0.05)
    elev[5, 5] = np.float32(0.01)
    assert np.array_equal(bits(FlowRouting.fill_depressions(land, elev)), bits(oracle.fill_depressions(land, elev)))


def test_fill_flat_plateaus_with_ties():
    """Tie-heavy ground: broad exactly-flat basins and terraces whose heights share a quantised key."""
    rng = np.random.default_rng(4)
    W, H = 128, 64
    g = np.round(rng.uniform(0.0, 0.02, (H, W)) * 2000) / 2000
    g = g.astype(np.float32)
    g[10:30, 20:60] = np.float32(0.001)
    g[40:50, 70:120] = np.float32(0.0105)
    land = np.ones((H, W), np.uint8)
    land[:, :4] = 0
    rel = np.where(land == 1, g, np.float32(-0.05)).astype(np.float32)
    want = oracle.fill_depressions(land, rel)
    got, ties, unresolved = FlowRouting.fill_depressions(land, rel, with_ties=True)
    assert unresolved == 0
    assert np.array_equal(bits(got), bits(want)), np.flatnonzero(bits(got) != bits(want))[:8]


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_fill_key_plateaus(seed):
    """Ground whose neighbouring heights share a quantised heap key (steps of 1e-7, below the key's
    2.4e-7 quantum at 4): within-level ties everywhere, which the fill resolves by replaying levels."""
    rng = np.random.default_rng(seed)
    W, H = 256, 128
    g = (np.float32(0.3) + np.float32(1e-7) * rng.integers(0, 6, (H, W)).astype(np.float32)).astype(np.float32)
    g[20:40, 30:90] -= np.float32(2e-6)       # a shallow pit in the plateau
    land = np.ones((H, W), np.uint8)
    land[:, 0:3] = 0
    rel = np.where(land == 1, g, np.float32(0.29)).astype(np.float32)
    want = oracle.fill_depressions(land, rel)
    got, ties, unresolved = FlowRouting.fill_depressions(land, rel, with_ties=True)
    assert unresolved == 0
    diff = np.flatnonzero(bits(got) != bits(want))
    assert diff.size == 0, f"{diff.size} cells differ (ties {ties}): {diff[:8]}"


def test_fill_key_level_larger_than_any_fixed_cap():
    """A coastal plain of 512K cells whose heights all lie within one quantum of the heap key (steps
    of 1e-7 around 0.3): the key level holds more than 2^18 cells, and the flood raises a staircase of
    thousands of levels across the plain, each with ties only its own pops can order. The fill must
    give the oracle's bits, whatever the level's size (or, past its repairs' guard, answer
    CG_INEXACT rather than a wrong result with CG_OK)."""
    rng = np.random.default_rng(9)
    W, H = 2048, 256
    g = (np.float32(0.3) + np.float32(1e-7) * rng.integers(0, 4, (H, W)).astype(np.float32)).astype(np.float32)
    land = np.ones((H, W), np.uint8)
    land[:, 0:2] = 0
    rel = np.where(land == 1, g, np.float32(0.29)).astype(np.float32)
    q = (rel[land == 1] + np.float32(4.0)).astype(np.float32).view(np.int32)
    assert np.bincount(q - q.min()).max() > (1 << 18)   # one key level alone is over 2^18 cells
    want = oracle.fill_depressions(land, rel)
    got, ties, unresolved = FlowRouting.fill_depressions(land, rel, with_ties=True)
    assert unresolved == 0
    diff = np.flatnonzero(bits(got) != bits(want))
    assert diff.size == 0, f"{diff.size} cells differ (ties {ties}): {diff[:8]}"


def test_fill_bench_world_8192x4096():
    """The bench world's first cut (8192 x 4096, 33.5M cells), where the index rule alone left a few
    within-level ties open: the device fill equals the oracle's bit for bit."""
    h, up, rk = synthetic.world(8192, 4096, 1, uplift="ridges")
    s, land, rel, n = oracle.percentile_cut(h, 0.70, np.float32(120.0) / np.float32(16000.0))
    want = oracle.fill_depressions(land, rel)
    got, ties, unresolved = FlowRouting.fill_depressions(land, rel, with_ties=True)
    assert unresolved == 0
    assert np.array_equal(bits(got), bits(want))


@pytest.mark.parametrize("W,H,seed", SIZES + [(2048, 1024, 1)])
@pytest.mark.parametrize("by_facet,over_potential", [(True, True), (True, False), (False, False)])
@pytest.mark.parametrize("r", [0.5, 1.0])
def test_flow_directions(W, H, seed, by_facet, over_potential, r):
    """r = 1.0 is the square-cell case of a 2:1 world (both legs one cell width)."""
    _, (s, land, rel, n) = world_cut(W, H, seed)
    filled = oracle.fill_depressions(land, rel)
    want, wsurf, wc = oracle.flow_directions(land, rel, filled, seed, r, 214, by_facet, over_potential,
                                             want_surface=True)
    got, gsurf, gc = FlowRouting.flow_directions(land, rel, filled, seed, r, 214, by_facet, over_potential,
                                                 want_surface=True)
    assert list(wc) == list(gc)
    np.testing.assert_allclose(gsurf, wsurf, rtol=SURFACE_RTOL, atol=0)
    diff = np.flatnonzero(got != want)
    assert diff.size == 0, f"{diff.size} receivers differ: {diff[:8]}"


@pytest.mark.parametrize("r", [1.0, 0.5, 1.75])
@pytest.mark.parametrize("step", [1.0 / 64, 1.0 / 1024])
def test_flow_directions_quantised_ties(r, step):
    """Heights on a coarse lattice, so facets tie on slope, cardinals on drop and shares sit on 1:
    the facet rule's comparisons and early outs must pick the reference's receiver at every tie."""
    W, H, seed = 256, 128, 17
    h, up, rk = synthetic.world(W, H, seed)
    s, land, rel, n = oracle.percentile_cut(h, 0.55)
    rel = (np.round(rel / step) * step).astype(np.float32)
    filled = oracle.fill_depressions(land, rel)
    for over_potential in (False, True):
        want, wc = oracle.flow_directions(land, rel, filled, seed, r, 214, True, over_potential)
        got, gc = FlowRouting.flow_directions(land, rel, filled, seed, r, 214, True, over_potential)
        assert list(wc) == list(gc)
        diff = np.flatnonzero(got != want)
        assert diff.size == 0, f"{diff.size} receivers differ: {diff[:8]}"


def carved_pits(W, H, seed):
    """Land everywhere but the polar rows, on the synthetic relief, with pits carved into it: round
    pits of about 600 to 9000 cells, one across the x-wrap seam, and a two-column trench (column runs
    several hundred cells long), so that the fill leaves flats for every flat solver (a CTA, a
    cluster of CTAs, and the global-memory one the cluster hands long runs to)."""
    h, _, _ = synthetic.world(W, H, seed)
    rel = ((h - h.min()) / (h.max() - h.min()) + 0.05).astype(np.float32)
    land = np.ones((H, W), np.uint8)
    land[:4] = 0
    land[-4:] = 0
    yy, xx = np.mgrid[0:H, 0:W]
    rng = np.random.default_rng(seed)
    for cx, cy, rad in [(W // 5, H // 3, 14), (W // 2, H // 2, 30), (3 * W // 4, H // 3, 54),
                        (W // 3, 2 * H // 3, 22), (0, H // 2, 18)]:
        dx = np.minimum(np.abs(xx - cx), W - np.abs(xx - cx))
        d2 = dx ** 2 + (yy - cy) ** 2
        pit = d2 <= rad * rad
        ring = (d2 <= (rad + 2) ** 2) & ~pit
        rel[pit] = float(rel[ring].min()) - 0.01 - 0.001 * rng.random(int(pit.sum())).astype(np.float32)
    trench = (xx >= 7 * W // 8) & (xx <= 7 * W // 8 + 1) & (yy > H // 8) & (yy < 7 * H // 8)
    ring = (xx >= 7 * W // 8 - 1) & (xx <= 7 * W // 8 + 2) & (yy >= H // 8) & (yy <= 7 * H // 8) & ~trench
    rel[trench] = float(rel[ring].min()) - 0.01
    return land, rel.astype(np.float32)


@pytest.mark.parametrize("r", [1.0, 0.5])
def test_flow_directions_large_flats(r):
    W, H, seed = 1024, 512, 5
    land, rel = carved_pits(W, H, seed)
    filled = oracle.fill_depressions(land, rel)
    want, wsurf, wc = oracle.flow_directions(land, rel, filled, seed, r, 214, True, True, want_surface=True)
    got, gsurf, gc = FlowRouting.flow_directions(land, rel, filled, seed, r, 214, True, True, want_surface=True)
    assert list(wc) == list(gc)
    np.testing.assert_allclose(gsurf, wsurf, rtol=SURFACE_RTOL, atol=0)
    diff = np.flatnonzero(got != want)
    assert diff.size == 0, f"{diff.size} receivers differ: {diff[:8]}"


@pytest.mark.parametrize("W,H,seed", SIZES + [(2048, 1024, 1)])
def test_drainage_order_accumulate_spillways(W, H, seed):
    _, (s, land, rel, n) = world_cut(W, H, seed)
    filled = oracle.fill_depressions(land, rel)
    rec, _ = oracle.flow_directions(land, rel, filled, seed, 0.5, 214)
    assert np.array_equal(FlowRouting.drainage_order(land, rec, n), oracle.drainage_order(land, rec, n))
    # Uneven weights make the float sums order-sensitive.
    w = np.random.default_rng(seed).uniform(0.3, 3.0, (H, W)).astype(np.float32)
    a_want = oracle.accumulate(land, rec, n, w)
    a_got = FlowRouting.accumulate(land, rec, n, w)
    assert np.array_equal(bits(a_got), bits(a_want))
    pond = np.float32(24.0) / np.float32(6000.0)
    sw_want = oracle.spillways(land, rel, filled, rec, pond)
    sw_got = FlowRouting.spillways(land, rel, filled, rec, pond)
    assert sw_got["count"] == sw_want["count"]
    if W >= 512:
        assert sw_want["count"] > 0   # the larger worlds hold basins deeper than the pond depth
    assert np.array_equal(sw_got["labels"], sw_want["labels"])
    for k in ("spill", "entry", "cells"):
        assert np.array_equal(sw_got[k], sw_want[k]), k
    for k in ("level", "floor"):
        assert np.array_equal(bits(sw_got[k]), bits(sw_want[k])), k
    for k in ("largest", "largest_cells", "largest_depth", "deepest"):
        assert sw_got[k] == sw_want[k], k


@pytest.mark.parametrize("W,H,seed", [(128, 64, 3), (512, 256, 7), (256, 256, 5)])
def test_route_cut_is_the_downstream_stages_routing(W, H, seed):
    # cg_route_cut: fillDepressions, flowDirections, accumulate and drainageOrder of one cut in one call,
    # as DrownedValleys.kt:411-421, RiverStage.kt:228-240 and GlaciationStage.kt:371-385 run them.
    from cartogenesis_gb300 import ErosionConfig
    _, (s, land, rel, n) = world_cut(W, H, seed)
    cfg = ErosionConfig(W, H, seed)
    r = (cfg.params.world_width_km * 0.5 / H) / (cfg.params.world_width_km / W)
    filled_w = oracle.fill_depressions(land, rel)
    rec_w, _ = oracle.flow_directions(land, rel, filled_w, seed, r, 214)
    filled, rec, area, order = FlowRouting.route_cut(cfg, land, rel, n)
    assert np.array_equal(bits(filled), bits(filled_w))
    assert np.array_equal(rec, rec_w)
    assert np.array_equal(bits(area), bits(oracle.accumulate(land, rec_w, n, np.ones((H, W), np.float32))))
    assert np.array_equal(order, oracle.drainage_order(land, rec_w, n))
    w = np.random.default_rng(seed).uniform(0.3, 3.0, (H, W)).astype(np.float32)
    _, _, area_w, _ = FlowRouting.route_cut(cfg, land, rel, n, weights=w)
    assert np.array_equal(bits(area_w), bits(oracle.accumulate(land, rec_w, n, w)))
