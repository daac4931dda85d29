"""The stage round by round on a resident world (cg_stage_begin, cg_erode_rounds, cg_stage_height,
cg_stage_finish): any split of the rounds gives cg_erode_stage's bits, and with climate_feed the
weather the caller solves on the swept terrain and again halfway down (HydraulicErosion.kt:655-661,
809-813) gives the oracle's stage with the same refresh, bit for bit."""
import numpy as np
import pytest

import oracle
from cartogenesis_gb300 import CgError, ErosionConfig, ErosionStage, StageRounds, synthetic

pytestmark = pytest.mark.gpu


def bits(a):
    return a.view(np.uint32)


@pytest.mark.parametrize("profile", [0, 1])
@pytest.mark.parametrize("splits", [(5,), (1, 2, 11), (6,)])
def test_split_rounds_match_the_whole_stage(profile, splits):
    W, H, seed = 256, 128, 5
    h, up, rk = synthetic.world(W, H, seed)
    cfg = ErosionConfig(W, H, seed, sea_level=0.70, profile=profile)
    whole = ErosionStage.apply(cfg, h, up, rk, want=("receivers", "area"))
    run = StageRounds(cfg, h, up, rk)
    for end in list(splits) + [cfg.params.hydraulic_rounds]:
        run.rounds(end)
    got = run.finish(want=("receivers", "area"))
    assert np.array_equal(bits(got.height), bits(whole.height))
    assert np.array_equal(got.receivers, whole.receivers)
    assert np.array_equal(bits(got.area), bits(whole.area))


def weather_of(field):
    """A stand-in for the provisional climate: rain and cover as fixed functions of the terrain."""
    f = field.astype(np.float32)
    rain = (np.float32(300.0) + np.float32(1500.0) * np.abs(np.sin(np.float32(40.0) * f))).astype(np.float32)
    veg = np.clip(np.float32(1.5) - np.float32(2.0) * f, 0, 1).astype(np.float32)
    return rain, veg


@pytest.mark.parametrize("W,H,seed,profile", [(256, 128, 7, 0), (512, 256, 3, 1)])
def test_climate_feed_matches_the_oracle(W, H, seed, profile):
    h, up, rk = synthetic.world(W, H, seed)
    cfg = ErosionConfig(W, H, seed, sea_level=0.70, profile=profile, climate_feed=1)
    seen = {}

    def provisional_weather(field, round_):
        seen[round_] = field.copy()
        return weather_of(field)

    got = StageRounds.apply_fed(cfg, h, provisional_weather, up, rk, want=("receivers",))
    assert sorted(seen) == [0, cfg.params.hydraulic_rounds // 2]
    p = oracle.default_params(W, H, seed, sea_level=0.70, profile=profile)
    p.climate_feed = 1
    lim, sweeps = oracle.thermal_limits(p)
    assert np.array_equal(bits(seen[0]), bits(oracle.thermal_sweep(h, lim, sweeps, p.rate)))
    ra, va = weather_of(seen[0])
    rb, vb = weather_of(seen[cfg.params.hydraulic_rounds // 2])
    want = oracle.erode_stage(p, h, up, rk, ra, va, want=("receivers",), refreshed=(rb, vb))
    assert np.array_equal(bits(got.height), bits(want["height"]))
    assert np.array_equal(got.receivers, want["receivers"])


def test_round_calls_are_checked():
    W, H = 128, 64
    h, up, rk = synthetic.world(W, H, 2)
    cfg = ErosionConfig(W, H, 2, sea_level=0.70, climate_feed=1)
    with pytest.raises(CgError, match="climate_feed"):
        ErosionStage.apply(cfg, h, up, rk)
    run = StageRounds(cfg, h, up, rk)
    with pytest.raises(CgError, match="needs the caller's weather"):
        run.rounds(3)
    rain, veg = weather_of(run.height())
    with pytest.raises(CgError, match="may not run across"):
        run.rounds(12, rain, veg)
    run.rounds(6, rain, veg)
    with pytest.raises(CgError, match="still to run"):
        run.finish()
    cfg2 = ErosionConfig(W, H, 2, sea_level=0.70)
    run2 = StageRounds(cfg2, h, up, rk)
    run2.next_round = 3   # out of order
    with pytest.raises(CgError, match="run in order"):
        run2.rounds(4)
