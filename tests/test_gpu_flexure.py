"""Profile P3 on the GPU: the plate flexure (Isostasy.Flexure over Fft2D, Isostasy.kt:277-411,
math/Fft.kt; HydraulicErosion.kt:707-725, 856-884) against the oracle, bit for bit (REF32): the
deflection of a load on its own, and the whole stage with the bend at the top of every round."""
import math

import numpy as np
import pytest

import oracle
from cartogenesis_gb300 import CgError, ErosionConfig, ErosionStage, Isostasy, StageRounds, synthetic

pytestmark = pytest.mark.gpu


def loads(W, H, seed):
    """A load like a round's: broad relief in pascals with sharp edges, and a mean far from zero."""
    rng = np.random.default_rng(seed)
    h, _, _ = synthetic.world(W, H, seed)
    metres = (h - np.float32(0.5)) * np.float32(16000.0)
    metres += rng.normal(0.0, 30.0, (H, W)).astype(np.float32)
    return (metres * np.float32(2835.0) * np.float32(9.81)).astype(np.float32)


@pytest.mark.parametrize("W,H", [(8, 4), (64, 32), (128, 128), (256, 128), (1024, 512), (2048, 1024), (16, 256)])
def test_deflection_matches_the_oracle(W, H):
    load = loads(W, H, W + H)
    cfg = ErosionConfig(W, H, 1)
    fx = Isostasy.Flexure(cfg)
    got = fx.deflection_metres(load)
    want, rigidity, restoring = oracle.flexure_deflection(oracle.default_params(W, H, 1), load)
    diff = np.flatnonzero(got.view(np.uint32) != want.view(np.uint32))
    assert diff.size == 0, f"{diff.size} of {W * H} deflections differ, first {diff[:8]}"
    assert fx.rigidity == rigidity and fx.restoring == restoring


def test_deflection_at_the_largest_lines():
    """Lines of 8192 (the widest a CTA holds): 8192 x 64 and 64 x 4096."""
    for W, H in ((8192, 64), (64, 4096)):
        load = loads(W, H, 5)
        got = Isostasy.Flexure(ErosionConfig(W, H, 1)).deflection_metres(load)
        want, _, _ = oracle.flexure_deflection(oracle.default_params(W, H, 1), load)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (W, H)


def test_broad_load_sinks_to_airy_on_the_device():
    """IsostasyTest's Airy limit (T/IsostasyTest.kt:219-290): a 33-cell square kilometre-high load sinks
    to within 5% of rho_c / (rho_m - rho_fill) of its height; a one-cell load is held up."""
    W = H = 256
    cfg = ErosionConfig(W, H, 1)
    p = cfg.params
    pascals = np.float32(np.float32(1000.0) * np.float32(p.continental_crust_density) * np.float32(p.gravity))
    airy = 1000.0 * p.continental_crust_density / (p.mantle_density - p.deflection_fill_density)
    fx = Isostasy.Flexure(cfg)

    def centre(half):
        load = np.zeros((H, W), np.float32)
        rows = np.abs(np.arange(H) - H // 2) <= half
        cols = np.abs(np.arange(W) - W // 2) <= half
        load[np.ix_(rows, cols)] = pascals
        return float(fx.deflection_metres(load)[H // 2, W // 2])

    assert centre(16) == pytest.approx(airy, rel=0.05)
    assert centre(0) < airy * 0.5
    alpha_km = math.sqrt(math.sqrt(4.0 * fx.rigidity / fx.restoring)) / 1000.0
    assert 50.0 <= alpha_km <= 200.0


def test_flexure_refuses_lines_past_a_cta():
    with pytest.raises(CgError):
        Isostasy.Flexure(ErosionConfig(16384, 16, 1)).deflection_metres(np.zeros((16, 16384), np.float32))
    with pytest.raises(CgError):
        ErosionStage.apply(ErosionConfig(64, 8192, 1, profile=3), np.zeros((8192, 64), np.float32))


WANT = ("receivers", "area", "filled", "relative", "is_land")


def check_stage(W, H, seed, uplift="bands", weather=False):
    h, up, rk = synthetic.world(W, H, seed, uplift=uplift)
    rain = veg = None
    if weather:
        rng = np.random.default_rng(seed)
        rain = rng.uniform(150.0, 2500.0, (H, W)).astype(np.float32)
        veg = rng.uniform(0.0, 1.0, (H, W)).astype(np.float32)
    cfg = ErosionConfig(W, H, seed, sea_level=0.70, profile=3)
    got = ErosionStage.apply(cfg, h, up, rk, rain, veg, want=WANT)
    want = oracle.erode_stage(oracle.default_params(W, H, seed, sea_level=0.70, profile=3), h, up, rk, rain, veg,
                              want=WANT)
    diff = np.flatnonzero(got.height.view(np.uint32) != want["height"].view(np.uint32))
    assert diff.size == 0, f"{diff.size} heights differ, first {diff[:8]}"
    for k in WANT:
        a, b = getattr(got, k), want[k]
        assert np.array_equal(a.view(np.uint32) if a.dtype == np.float32 else a,
                              b.view(np.uint32) if b.dtype == np.float32 else b), k
    return got


@pytest.mark.parametrize("W,H,seed", [(128, 64, 3), (256, 128, 42), (512, 256, 7)])
def test_p3_stage_matches_the_oracle(W, H, seed):
    got = check_stage(W, H, seed)
    assert all(s["ms_flexure"] > 0.0 for s in got.stats)


def test_p3_stage_without_uplift_and_with_weather():
    """No uplift record (0 subtracted, as the reference subtracts it) and the weather's weights."""
    W, H, seed = 256, 128, 5
    h, _, rk = synthetic.world(W, H, seed)
    cfg = ErosionConfig(W, H, seed, sea_level=0.70, profile=3)
    got = ErosionStage.apply(cfg, h, None, rk)
    want = oracle.erode_stage(oracle.default_params(W, H, seed, sea_level=0.70, profile=3), h, None, rk)
    assert np.array_equal(got.height.view(np.uint32), want["height"].view(np.uint32))
    check_stage(256, 128, 9, weather=True)


def test_p3_round_by_round_matches_the_whole_stage():
    """The reference field, the bend and the uplift record stay on the context between round calls."""
    W, H, seed = 256, 128, 13
    h, up, rk = synthetic.world(W, H, seed)
    cfg = ErosionConfig(W, H, seed, sea_level=0.70, profile=3)
    whole = ErosionStage.apply(cfg, h, up, rk, want=("receivers",))
    run = StageRounds(cfg, h, up, rk)
    run.rounds(5)
    run.rounds(12)
    got = run.finish(want=("receivers",))
    assert np.array_equal(got.height.view(np.uint32), whole.height.view(np.uint32))
