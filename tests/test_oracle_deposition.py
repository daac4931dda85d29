"""The oracle's restatement of profile P2's deposition (the walk, the outlined sea lobes and lake fans,
settle, the closing mouths pass), pinned to the reference's DepositionTest
(T/DepositionTest.kt, T = worldgen/src/jvmTest/kotlin/com/cartogenesis/worldgen): every round's mass
budget closes, and deposition switched off is deposition absent, whatever its knobs say, while
deposition running with every rate at zero leaves the rock bit-identical. The GPU's P2 stage is held
to this restatement bit for bit by tests/test_gpu_deposition.py.
"""
import numpy as np
import pytest

import oracle
from cartogenesis_gb300 import synthetic


def bits(a):
    return a.view(np.uint32)


@pytest.mark.parametrize("W,H,seed,knobs", [
    (256, 128, 42, {}), (512, 256, 7, {}),
    (256, 128, 42, {"delta_outline": 0}),                    # square lobes and lake fans
    (256, 128, 42, {"delta_outline": 0, "delta_lobe": 0}),   # the flat slab, no mouths pass
])
def test_every_round_conserves_mass(W, H, seed, knobs):
    """T/DepositionTest.kt:44-94: incised = deposited + lost, and the field fell by what was lost,
    each within 1% in every round, and every round deposited something."""
    h, up, rk = synthetic.world(W, H, seed)
    p = oracle.default_params(W, H, seed, sea_level=0.70, profile=2)
    _, tallies = oracle.erode_stage_switched(p, h, up, rk, oracle.Switches(2, **knobs))
    assert tallies.shape == (12, 4)
    for incised, deposited, lost, drop in tallies:
        assert abs(incised - (deposited + lost)) / max(incised, 1e-12) < 0.01
        assert abs(drop - lost) / max(lost, 1e-12) < 0.01
        assert deposited > 0.0


def test_deposition_off_is_deposition_absent():
    """T/DepositionTest.kt:165-214: with deposition off no knob beside it leaks into the world, and with
    deposition running but every rate that lays spoil at zero the rock is bit-identical to the rock
    with the machinery off."""
    W, H, seed = 256, 128, 42
    h, up, rk = synthetic.world(W, H, seed)
    p = oracle.default_params(W, H, seed, sea_level=0.70)
    off, _ = oracle.erode_stage_switched(p, h, up, rk, oracle.Switches(2, deposition=0))
    fiddled, _ = oracle.erode_stage_switched(
        p, h, up, rk, oracle.Switches(2, deposition=0, transport_capacity=0.1, deposition_rate=1.0, delta_share=1.0,
                                      delta_min_catchment_km2=0.0, lake_share=1.0, delta_reach_km=469.0,
                                      delta_freeboard_metres=3000.0))
    silent, _ = oracle.erode_stage_switched(
        p, h, up, rk, oracle.Switches(2, delta_share=0.0, deposition_rate=0.0, lake_share=0.0))
    on, tallies = oracle.erode_stage_switched(p, h, up, rk, oracle.Switches(2))
    assert np.array_equal(bits(fiddled), bits(off))
    assert np.array_equal(bits(silent), bits(off))
    assert not np.array_equal(bits(on), bits(off))
    assert tallies[:, 1].sum() > 0.0


def test_profiles_nest():
    """The profile switches: P2 through the ABI's profile field is the switched stage with the reference
    defaults, and the mouths pass (deltaLobe) is the only difference between P1 and P2 with deposition
    off."""
    W, H, seed = 128, 64, 3
    h, up, rk = synthetic.world(W, H, seed)
    p2 = oracle.default_params(W, H, seed, sea_level=0.70, profile=2)
    via_profile = oracle.erode_stage(p2, h, up, rk, want=())["height"]
    switched, _ = oracle.erode_stage_switched(p2, h, up, rk, oracle.Switches(2))
    assert np.array_equal(bits(via_profile), bits(switched))
    p1 = oracle.default_params(W, H, seed, sea_level=0.70, profile=1)
    plain_p1 = oracle.erode_stage(p1, h, up, rk, want=())["height"]
    switched_p1, _ = oracle.erode_stage_switched(p1, h, up, rk, oracle.Switches(1))
    assert np.array_equal(bits(plain_p1), bits(switched_p1))


def test_fan_shapes_differ():
    """The outlined fans, the square lobes and the flat slab lay different spoil: each shape reaches
    the terrain."""
    W, H, seed = 256, 128, 42
    h, up, rk = synthetic.world(W, H, seed)
    p = oracle.default_params(W, H, seed, sea_level=0.70)
    outs = [oracle.erode_stage_switched(p, h, up, rk, oracle.Switches(2, **k))[0]
            for k in ({}, {"delta_outline": 0}, {"delta_outline": 0, "delta_lobe": 0})]
    for i in range(3):
        for j in range(i + 1, 3):
            assert not np.array_equal(bits(outs[i]), bits(outs[j]))



@pytest.mark.parametrize("W,H,seed,uplift,replays,redos", [
    (512, 256, 7, "bands", 1, 0),
    (2048, 1024, 1, "ridges", 1, 1),
])
def test_level_schedule_reproduces_the_walk(W, H, seed, uplift, replays, redos):
    """The deposition walk in the order a device runs it (level by level, each level's own walks at
    once, then its mouths in rank order, with the two repairs for fans that reach into their own level)
    gives the reference order's bits over the whole P2 stage; the worlds are chosen so that the repairs
    happen (at least the given counts)."""
    h, up, rk = synthetic.world(W, H, seed, uplift=uplift)
    p = oracle.default_params(W, H, seed, sea_level=0.70, profile=2)
    walk = oracle.erode_stage(p, h, up, rk, want=())["height"]
    levels, (replayed, redone) = oracle.erode_stage_levels(p, h, up, rk)
    assert np.array_equal(bits(levels), bits(walk))
    assert replayed >= replays and redone >= redos


@pytest.mark.parametrize("r", [1.0, 0.5])
def test_a_lobe_reaches_as_far_north_as_east_on_the_ground(r):
    """T:DeltaOutlineTest.kt:546-597: a directionless lobe of 40 cell widths, no wobble, grown on open flat
    water at the centre of a 256 x 256 grid reaches as far east-west as north-south on the ground, to a
    cell width (the project's 2:1 grids have square cells; half-height cells are read too)."""
    W = H = 256
    apex = (H // 2) * W + W // 2
    sed, laid = oracle.grow_fan_fixture(np.full((H, W), -1.0, np.float32), apex, r, 40.0, 0.0, 0.0,
                                        oracle.fan_hash(42, 1), grooved=False, wobble=0.0)
    assert laid > 0
    rows, cols = np.nonzero(sed > 0)
    east_west = np.abs(cols[rows == H // 2] - W // 2).max()
    north_south = (np.abs(rows[cols == W // 2] - H // 2) * r).max()
    assert abs(east_west - north_south) <= 1.0, (east_west, north_south)


def test_a_fan_reaches_further_over_a_shelf_than_into_deep_water():
    """T:DeltaOutlineTest.kt:599-688: a lobe of 24 cells aimed east from the edge between a 0.2-deep shelf
    and 6-deep water, over 24 mouths: with the depth term (the distance bent by 1 - surface) it
    reaches on average at least 1.5 times as far over the shelf as into the deep water; without it,
    not."""
    W = H = 96
    ax, ay = 32, 48
    surface = np.where(np.arange(H)[:, None] < ay, np.float32(-0.2), np.float32(-6.0)) * np.ones((1, W), np.float32)
    ratios = {True: [], False: []}
    for trial in range(24):
        h = oracle.fan_hash(9001, trial)
        for bent in (True, False):
            sed, _ = oracle.grow_fan_fixture(surface, ay * W + ax, 1.0, 24.0, 1.0, 0.0, h, grooved=False,
                                             wobble=0.30, bent=bent)
            rows, cols = np.nonzero(sed > 0)
            dx, dy = (cols - ax).astype(np.float64), (rows - ay).astype(np.float64)
            rr = np.sqrt(dx * dx + dy * dy)
            shelf = rr[dy < 0].max() if (dy < 0).any() else 0.0
            deep = rr[dy > 0].max() if (dy > 0).any() else 0.0
            ratios[bent].append(shelf / max(deep, 1e-9))
    assert np.mean(ratios[False]) < 1.5
    assert np.mean(ratios[True]) >= 1.5, np.mean(ratios[True])


def _rim_shape(w, h, apex, mask, bins=32):
    """DeltaOutlineTest.rimOf (T:DeltaOutlineTest.kt:454-532): per angle bin the farthest cell laid;
    the rim's max / min radius, its RMS departure from a fitted a0 + a1 cos + b1 sin over the mean, and
    its RMS difference from its reflection about the fitted axis (snapped to a half bin) over the mean."""
    import math
    ax, ay = apex % w, apex // w
    radius = np.full(bins, -1.0)
    for c in np.flatnonzero(mask.ravel()):
        dx = c % w - ax
        dx = dx - w if dx > w // 2 else (dx + w if dx < -(w // 2) else dx)
        dy = c // w - ay
        r = math.hypot(dx, dy)
        if r <= 0:
            continue
        a = math.atan2(dy, dx) / (2 * math.pi)
        a = a + 1.0 if a < 0 else a
        b = min(max(int(a * bins), 0), bins - 1)
        radius[b] = max(radius[b], r)
    filled = [b for b in range(bins) if radius[b] > 0]
    if len(filled) < bins // 4:
        return None
    pos = radius[radius > 0]
    ratio = pos.max() / pos.min()
    t = np.array([2 * math.pi * (b + 0.5) / bins for b in filled])
    A = np.stack([np.ones_like(t), np.cos(t), np.sin(t)], axis=1)
    fit = np.linalg.solve(A.T @ A, A.T @ radius[filled])
    mean = radius[filled].mean()
    residual = math.sqrt(((radius[filled] - A @ fit) ** 2).mean()) / mean
    k = math.floor(math.atan2(fit[2], fit[1]) / (math.pi / bins) + 0.5)   # Math.round
    asq, pairs = 0.0, 0
    for b in filled:
        m = (k - b - 1) % bins
        if radius[m] <= 0:
            continue
        asq += (radius[b] - radius[m]) ** 2
        pairs += 1
    asymmetry = 0.0 if pairs < bins // 4 else math.sqrt(asq / pairs) / mean
    return ratio, residual, asymmetry


def test_a_lobe_is_not_a_disc_and_not_a_cosine():
    """T:DeltaOutlineTest.kt:286-383: over 24 mouths on open water, a lobe of 24 cells with its wobble has
    a rim whose radius varies by at least 1.5 and differs by at least 6% from its reflection about its
    own axis; the compass-drawn controls (a half-disc with no direction, a cosine lobe with no wobble)
    fail those bars."""
    W = H = 128
    apex = 64 * W + 64
    shapes = {"shaped": (1.0, 0.0, 0.30), "cosine lobe": (1.0, 0.0, 0.0), "half-disc": (0.0, 0.0, 0.0)}
    worst = {}
    for trial in range(24):
        h = oracle.fan_hash(4242, trial)
        for name, (ox, oy, wob) in shapes.items():
            sed, _ = oracle.grow_fan_fixture(np.full((H, W), -1.0, np.float32), apex, 1.0, 24.0, ox, oy, h,
                                             grooved=False, wobble=wob)
            shape = _rim_shape(W, H, apex, sed > 0)
            if shape is None:
                continue
            pick = min if name == "shaped" else max
            worst[name] = tuple(pick(a, b) for a, b in zip(worst.get(name, shape), shape))
    assert worst["half-disc"][0] < 1.5
    assert worst["cosine lobe"][2] < 0.06 and worst["half-disc"][2] < 0.06
    assert worst["shaped"][0] >= 1.5, worst
    assert worst["shaped"][2] >= 0.06, worst
