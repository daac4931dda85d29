"""The whole erosion stage on the GPU (cg_erode_stage: initial sweeps, 12 hydraulic rounds, relax
sweeps) against the oracle on the same seeded worlds, bit for bit: heights, receivers, donor
counts, drainage order, accumulation, the fill, lake labels and outlets after the last round."""
import numpy as np
import pytest

import oracle
from cartogenesis_gb300 import CgError, ErosionConfig, ErosionStage, synthetic

pytestmark = pytest.mark.gpu


def bits(a):
    return a.view(np.uint32) if a.dtype == np.float32 else a


def compare(got, want, order=True):
    for k in ("receivers", "donors", "order", "is_land", "basin_of_cell"):
        if k == "order" and not order:
            continue
        d = np.flatnonzero(getattr(got, k) != want[k])
        assert d.size == 0, f"{k}: {d.size} cells differ, first {d[:6]}"
    for k in ("height", "area", "filled", "relative"):
        d = np.flatnonzero(bits(getattr(got, k)) != bits(want[k]))
        assert d.size == 0, f"{k}: {d.size} cells differ, first {d[:6]}"
    gb, wb = got.basins, want["basins"]
    assert gb["count"] == wb["count"]
    for k in ("spill", "entry", "cells"):
        assert np.array_equal(gb[k], wb[k]), k
    for k in ("level", "floor"):
        assert np.array_equal(bits(gb[k]), bits(wb[k])), k


@pytest.mark.parametrize("W,H,seed", [(64, 32, 5), (128, 64, 3), (256, 128, 42), (512, 256, 1)])
def test_stage_matches_oracle(W, H, seed):
    h, up, rk = synthetic.world(W, H, seed)
    cfg = ErosionConfig(W, H, seed, sea_level=0.70)
    got = ErosionStage.apply(cfg, h, up, rk)
    want = oracle.erode_stage(oracle.default_params(W, H, seed, sea_level=0.70), h, up, rk)
    compare(got, want)
    assert all(s["fill_unresolved"] == 0 for s in got.stats)
    assert [s["land_cells"] for s in got.stats] == [s["land_cells"] for s in want["stats"]]
    assert [s["flats"] for s in got.stats] == [s["flats"] for s in want["stats"]]


def test_stage_with_weather_and_switches():
    """Rainfall and cover given (climate-fed weights), facet routing off, the clamp off, two rounds."""
    W, H, seed = 128, 64, 9
    h, up, rk = synthetic.world(W, H, seed)
    rng = np.random.default_rng(seed)
    rain = rng.uniform(60.0, 2500.0, (H, W)).astype(np.float32)
    veg = rng.uniform(0.0, 1.0, (H, W)).astype(np.float32)
    for over in ({"facet_routing": 0, "hydraulic_rounds": 2}, {"receiver_clamp": 0, "hydraulic_rounds": 3},
                 {"flat_potential": 0, "shield_cut": 0, "hydraulic_rounds": 2}):
        cfg = ErosionConfig(W, H, seed, sea_level=0.65, **over)
        got = ErosionStage.apply(cfg, h, up, rk, rain, veg)
        want = oracle.erode_stage(oracle.default_params(W, H, seed, sea_level=0.65, **over), h, up, rk, rain, veg)
        compare(got, want)


def test_stage_2048x1024_heights_and_receivers():
    """The benchmark grid: 2048 x 1024 cells, 12 rounds, 96 + 12 x 8 sweeps."""
    W, H, seed = 2048, 1024, 1
    h, up, rk = synthetic.world(W, H, seed)
    cfg = ErosionConfig(W, H, seed, sea_level=0.70)
    got = ErosionStage.apply(cfg, h, up, rk, want=("receivers", "area", "is_land", "donors"))
    want = oracle.erode_stage(oracle.default_params(W, H, seed, sea_level=0.70), h, up, rk,
                              want=("receivers", "area", "is_land", "donors"))
    assert np.array_equal(bits(got.height), bits(want["height"]))
    assert np.array_equal(got.receivers, want["receivers"])
    assert np.array_equal(got.donors, want["donors"])
    assert np.array_equal(bits(got.area), bits(want["area"]))


def test_stage_bench_world_8192x4096():
    """The benchmark workload itself: 8192 x 4096 cells, 12 rounds, the ridge-uplift world, every
    output of the last round bit for bit (the oracle takes about three minutes on 16 cores)."""
    W, H, seed = 8192, 4096, 1
    h, up, rk = synthetic.world(W, H, seed, uplift="ridges")
    keys = ("receivers", "area", "filled", "relative", "is_land", "basin_of_cell", "donors")
    got = ErosionStage.apply(ErosionConfig(W, H, seed, sea_level=0.70), h, up, rk, want=keys)
    want = oracle.erode_stage(oracle.default_params(W, H, seed, sea_level=0.70), h, up, rk, want=keys)
    compare(got, want, order=False)
    assert all(s["fill_unresolved"] == 0 for s in got.stats)
    assert [s["flats"] for s in got.stats] == [s["flats"] for s in want["stats"]]
    assert [s["flats_kept"] for s in got.stats] == [s["flats_kept"] for s in want["stats"]]


def test_stage_rejects_bad_arguments():
    h = np.zeros((32, 48), np.float32)
    with pytest.raises(CgError):
        ErosionStage.apply(ErosionConfig(48, 32, 1), h)
    with pytest.raises(CgError):
        ErosionStage.apply(ErosionConfig(64, 32, 1, profile=4), np.zeros((32, 64), np.float32))
    with pytest.raises(CgError):
        ErosionStage.apply(ErosionConfig(64, 32, 1, mode=1), np.zeros((32, 64), np.float32))


def test_stage_disabled_and_no_rounds_are_copies_or_sweeps():
    W, H = 64, 32
    h, _, _ = synthetic.world(W, H, 2)
    got = ErosionStage.apply(ErosionConfig(W, H, 2, enabled=0), h, want=())
    assert np.array_equal(got.height, h)
    got = ErosionStage.apply(ErosionConfig(W, H, 2, hydraulic_rounds=0), h, want=())
    want = oracle.erode_stage(oracle.default_params(W, H, 2, hydraulic_rounds=0), h, want=())
    assert np.array_equal(bits(got.height), bits(want["height"]))
