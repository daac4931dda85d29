"""Profile P2 on the GPU: the deposition walk with its sea lobes and lake fans, settle and the closing
mouths pass (HydraulicErosion.kt:1068-1349, 1351-1364, 1804-1892; DeltaFan.kt), against the oracle's
whole stage, bit for bit (REF32): every output the stage hands back."""
import numpy as np
import pytest

import oracle
from cartogenesis_gb300 import ErosionConfig, ErosionStage, StageRounds, synthetic

pytestmark = pytest.mark.gpu

WANT = ("receivers", "area", "filled", "relative", "is_land")


def check(W, H, seed, uplift="bands", weather=False, rounds=12):
    h, up, rk = synthetic.world(W, H, seed, uplift=uplift)
    rain = veg = None
    if weather:
        rng = np.random.default_rng(seed)
        rain = rng.uniform(150.0, 2500.0, (H, W)).astype(np.float32)
        veg = rng.uniform(0.0, 1.0, (H, W)).astype(np.float32)
    cfg = ErosionConfig(W, H, seed, sea_level=0.70, profile=2, hydraulic_rounds=rounds)
    got = ErosionStage.apply(cfg, h, up, rk, rain, veg, want=WANT)
    p = oracle.default_params(W, H, seed, sea_level=0.70, profile=2, hydraulic_rounds=rounds)
    want = oracle.erode_stage(p, h, up, rk, rain, veg, want=WANT)
    diff = np.flatnonzero(got.height.view(np.uint32) != want["height"].view(np.uint32))
    assert diff.size == 0, f"{diff.size} heights differ, first {diff[:8]}"
    for k in WANT:
        a, b = getattr(got, k), want[k]
        if a.dtype == np.float32:
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), k
        else:
            assert np.array_equal(a, b), k
    return got


@pytest.mark.parametrize("W,H,seed", [(128, 64, 3), (256, 128, 42), (512, 256, 7), (512, 256, 8)])
def test_p2_stage_matches_the_oracle(W, H, seed):
    check(W, H, seed)


def test_p2_stage_with_weather_2048x1024():
    """BASELINE's config-1 shape with rain and cover: lake fans by the thousand a round."""
    check(2048, 1024, 1, uplift="ridges", weather=True)


def test_p2_round_by_round_matches_the_whole_stage():
    """The sediment carried between rounds stays on the context between round-range calls."""
    W, H, seed = 256, 128, 11
    h, up, rk = synthetic.world(W, H, seed)
    cfg = ErosionConfig(W, H, seed, sea_level=0.70, profile=2)
    whole = ErosionStage.apply(cfg, h, up, rk, want=("receivers",))
    run = StageRounds(cfg, h, up, rk)
    run.rounds(4)
    run.rounds(12)
    got = run.finish(want=("receivers",))
    assert np.array_equal(got.height.view(np.uint32), whole.height.view(np.uint32))
    assert np.array_equal(got.receivers, whole.receivers)
