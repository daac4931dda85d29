"""The oracle's restatement of the belts' replay (BeltErosion.replay, P/BeltErosion.kt:96-425) and of
GaussianBlur (MA/GaussianBlur.kt), on the CPU.

The reference's own guards for the replay (T:BeltReplayTest.kt) read it on seed 42's plate stage, which
cannot run here; the same two properties are asked of seeded synthetic belts (synthetic.belt_window):
the sediment books close, and the eroded depth converges as the step halves. The rest pins the
replay's arithmetic where it can be worked by hand: its round count, its do-nothing cases, the
lowering and rise it starts from, and the blur's taps.
"""
import numpy as np
import pytest

import oracle
from cartogenesis_gb300 import synthetic

SEED = 5


def world(W, H, seed=SEED):
    h, up, rk = synthetic.world(W, H, seed)
    t, w, o, win = synthetic.belt_window(W, H, seed)
    return h, up, rk, t, w, o, win


def test_the_replays_sediment_books_close():
    # T:BeltReplayTest.kt:34-53: what the rivers cut leaves the belts at their outlets, to a part in a
    # million (CLOSING_TOLERANCE), under an even rain of 1000 mm and no cover.
    W, H = 256, 128
    h, up, rk, t, w, o, win = world(W, H)
    p = oracle.default_params(W, H, seed=SEED)
    rain = np.full((H, W), 1000.0, np.float32)
    _, eroded, b = oracle.belt_replay(p, h, t, w, o, win, uplift=up, rock=rk, rain=rain, cover=np.zeros((H, W)),
                                      shield_cut=False)
    assert b["rounds"] > 0 and b["cut_cubic_meters"] > 0.0
    exported = b["exported_to_sea_cubic_meters"] + b["exported_to_land_cubic_meters"]
    assert abs(b["cut_cubic_meters"] - exported) / b["cut_cubic_meters"] <= 1e-6
    assert b["belt_cells"] == int((o >= 0).sum())
    assert (eroded[o < 0] == 0).all() and eroded.max() > 0


def test_the_replay_converges_as_its_step_halves():
    # T:BeltReplayTest.kt:64-90: the rounds' years halved and their count doubled; the change from the
    # half to the quarter step is at most 0.75 of the change before (CONVERGENCE_RATIO) and under a tenth
    # of the mean eroded depth (CONVERGED_SHARE).
    W, H = 256, 128
    h, up, rk, t, w, o, win = world(W, H)
    rain = np.full((H, W), 1000.0, np.float32)
    eroded = []
    for split in (1, 2, 4):
        p = oracle.default_params(W, H, seed=SEED)
        p.years_per_hydraulic_round /= split
        p.hydraulic_rounds *= split
        _, e, b = oracle.belt_replay(p, h, t, w, o, win, uplift=up, rock=rk, rain=rain, shield_cut=False)
        assert b["rounds"] > 0
        eroded.append(e.astype(np.float64))
    mean = eroded[2].mean()
    coarse = np.abs(eroded[0] - eroded[1]).mean()
    fine = np.abs(eroded[1] - eroded[2]).mean()
    assert fine <= 0.75 * coarse, (fine, coarse)
    assert fine <= 0.1 * mean, (fine, mean)


def test_round_count_and_the_cases_that_do_nothing():
    W, H = 128, 64
    h, up, rk, t, w, o, win = world(W, H)
    p = oracle.default_params(W, H, seed=SEED)
    # ((windowMyr - mainMyr) / roundMyr + 1e-9).toInt() (BeltErosion.kt:117): 40 Myr less twelve rounds
    # of 336476.4 years is 106.88 rounds.
    round_myr = p.years_per_hydraulic_round / 1e6
    assert oracle.belt_replay(p, h, t, w, o, win)[2]["rounds"] == int((win - 12 * round_myr) / round_myr + 1e-9) == 106
    # A window no longer than the rounds' own span, no belt, or no erodibility: BeltReplay.NOTHING and the
    # surface untouched (BeltErosion.kt:118, 129).
    for args, params in (((t, w, o, 12 * round_myr), p),
                         ((t, w, np.full_like(o, -1.0), win), p),
                         ((t, w, o, win), oracle.default_params(W, H, seed=SEED, bedrock_erodibility_per_year=0.0))):
        h2, e2, b2 = oracle.belt_replay(params, h, *args, uplift=up)
        assert b2["rounds"] == 0 and b2["belt_cells"] == 0
        assert np.array_equal(h2, h) and not e2.any()


def test_one_round_window_lowers_raises_and_cuts_as_the_reference_does():
    # A window one round longer than the rounds: one replayed round, every belt cell's first round 0.
    # The lowering and the rise are worked here in the reference's float and double steps
    # (BeltErosion.kt:132-144, 240-248); with rivers and slopes off (erodibility so small that nothing
    # is cut, and a critical fall no slope reaches) the replay is the lowering plus the rise.
    W, H = 128, 64
    h, up, rk, t, w, o, _ = world(W, H)
    p = oracle.default_params(W, H, seed=SEED, bedrock_erodibility_per_year=1e-30, critical_fall_metres_per_km=1e9)
    round_myr = p.years_per_hydraulic_round / 1e6
    win = 13.5 * round_myr
    h2, e2, b = oracle.belt_replay(p, h, t, w, o, win, uplift=up, rebound=False)
    assert b["rounds"] == 1
    f32 = np.float32
    freeboard = (f32(3300.0) - f32(2835.0)) / f32(3300.0) * f32(1000.0)
    mpfu = f32(6000.0) + f32(10000.0)
    belt = o >= 0
    expect = h.copy()
    lowered = h[belt] - freeboard * (t[belt] - w[belt]) / mpfu
    share = (up[belt] * f32(12)).astype(np.float64) * p.years_per_hydraulic_round / 1000.0
    rise_m = (freeboard * t[belt]).astype(np.float64) - share
    rise = (rise_m / 1.0 / np.float64(mpfu)).astype(np.float32)
    expect[belt] = (lowered + rise).astype(np.float32)
    assert np.array_equal(h2, expect)
    up_books = np.float64(0.0)
    area = (40075.0 / W) * (40075.0 * 0.5 / H) * 1e6
    for r in rise:
        up_books += np.float64(r) * np.float64(mpfu) * area
    assert b["uplifted_cubic_meters"] == up_books
    assert b["cut_cubic_meters"] == 0.0 and b["shed_beside_cubic_meters"] == 0.0


def test_rebound_lifts_the_most_cut_ground():
    # The crust answers the rock taken (BeltErosion.kt:413-423): with the rebound on, the belt's most
    # eroded cells stand higher than with it off.
    W, H = 256, 128
    h, up, rk, t, w, o, win = world(W, H)
    p = oracle.default_params(W, H, seed=SEED)
    on, e_on, _ = oracle.belt_replay(p, h, t, w, o, win, uplift=up, rock=rk, rebound=True)
    off, e_off, _ = oracle.belt_replay(p, h, t, w, o, win, uplift=up, rock=rk, rebound=False)
    deep = e_off >= np.quantile(e_off[o >= 0], 0.95)
    deep &= o >= 0
    assert deep.sum() > 10
    assert (on[deep] - off[deep]).mean() > 0.0


@pytest.mark.parametrize("sigma", [0.6, 2.5, 9.7])
def test_gaussian_blur_keeps_a_constant_and_spreads_a_point_evenly(sigma):
    # GaussianBlur.kt:18-20: the taps are normalised, so a constant field is left constant; the kernel
    # is symmetric and, away from the poles (which clamp), sums to one.
    W, H = 64, 128
    c = np.full((H, W), 0.4375, np.float32)
    assert np.array_equal(oracle.gaussian_blur(c, sigma, sigma / 2), c)
    d = np.zeros((H, W), np.float32)
    d[64, 10] = 1.0
    b = oracle.gaussian_blur(d, sigma, sigma)
    assert abs(b.astype(np.float64).sum() - 1.0) < 1e-5
    assert np.allclose(b[64, 10 - 3], b[64, 10 + 3], rtol=0, atol=1e-7)
    assert np.allclose(b[64 - 3, 10], b[64 + 3, 10], rtol=0, atol=1e-7)
    # Zero spread leaves an axis alone.
    assert np.array_equal(oracle.gaussian_blur(d, 0.0, 0.0), d)


@pytest.mark.parametrize("profile", [0, 2, 3])
def test_stage_with_the_window_is_sweeps_then_replay_then_rounds(profile):
    # HydraulicErosion.kt:680-688: the replay runs on the swept terrain before round 0, with the stage's
    # uplift, rock, sea level and shield_cut and the opening weather; the rounds (the flexure's field
    # before them included) start from the replayed terrain.
    W, H = 128, 64
    h, up, rk, t, w, o, win = world(W, H)
    p = oracle.default_params(W, H, seed=SEED, profile=profile)
    whole = oracle.erode_stage_belts(p, h, (t, w, o, win), uplift=up, rock=rk)["height"]
    swept = oracle.thermal_sweep(h, oracle.thermal_limits(p)[0], oracle.thermal_limits(p)[1])
    replayed, _, books = oracle.belt_replay(p, swept, t, w, o, win, uplift=up, rock=rk)
    assert books["rounds"] == 106
    parts = oracle.stage_rounds(p, replayed, up, rk, rounds=p.hydraulic_rounds)
    assert np.array_equal(whole.view(np.uint32), parts.view(np.uint32))
    plain = oracle.erode_stage(p, h, up, rk, want=())["height"]
    assert not np.array_equal(whole, plain)


@pytest.mark.parametrize("W,H", [(512, 512), (512, 256)])
def test_a_point_spreads_as_far_on_the_ground_whichever_way_it_goes(W, H):
    # T:GaussianBlurTest.kt:26-58: a point blurred by 93.75 km, handed over as that many columns and
    # rows, keeps its mass to 1e-5, spreads 93.75 km each way on the ground to a hundredth, and does not
    # lean along a diagonal.
    spread_km = 93.75
    cw, ch = 40075.0 / W, 40075.0 * 0.5 / H
    f = np.zeros((H, W), np.float32)
    f[H // 2, W // 2] = 1.0
    b = oracle.gaussian_blur(f, spread_km / cw, spread_km / ch).astype(np.float64)
    east = (np.arange(W) - W // 2) * cw
    south = (np.arange(H) - H // 2) * ch
    total = b.sum()
    ew = (b * east[None, :] ** 2).sum()
    ns = (b * south[:, None] ** 2).sum()
    across = (b * east[None, :] * south[:, None]).sum()
    assert abs(total - 1.0) < 1e-5
    assert abs(np.sqrt(ew / total) / spread_km - 1.0) < 0.01
    assert abs(np.sqrt(ns / total) / spread_km - 1.0) < 0.01
    assert abs(across / np.sqrt(ew * ns)) < 0.01


def test_a_constant_stays_that_constant():
    # T:GaussianBlurTest.kt:60-66.
    f = np.full((64, 64), 0.625, np.float32)
    assert np.abs(oracle.gaussian_blur(f, 3.0, 6.0) - np.float32(0.625)).max() < 1e-6
