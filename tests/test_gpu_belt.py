"""The belts' replay on the GPU (BeltErosion.replay, P/BeltErosion.kt:96-425) and its two building blocks,
GaussianBlur.apply (MA/GaussianBlur.kt:44-111) and the sequential double sum over double terms that
keeps the replay's books, against the oracle and numpy's running sum, bit for bit (REF32)."""
import numpy as np
import pytest

import oracle
from cartogenesis_gb300 import BeltErosion, BeltWindow, ErosionConfig, GaussianBlur, synthetic
from cartogenesis_gb300.api import sequential_sum_f64

pytestmark = pytest.mark.gpu


def same(a, b):
    return np.float64(a).view(np.uint64) == np.float64(b).view(np.uint64) or (a != a and b != b)


rng = np.random.default_rng(11)
N = 1 << 20
F64_CASES = {
    "normal": rng.normal(0.0, 1e12, N),
    "positive": rng.uniform(0.0, 1e15, N),
    "mixed_scales": rng.normal(0.0, 1.0, N) * 10.0 ** rng.integers(-30, 31, N),
    "running_total_first": np.concatenate([[3.141592653589793e17], rng.uniform(0.0, 1e9, N)]),
    "ties": np.concatenate([[2.0 ** 60], np.full(N // 2, 2.0 ** 7), np.full(N // 2, 3 * 2.0 ** 7)]),
    "ties_negative": np.concatenate([[-(2.0 ** 60)], np.tile([2.0 ** 7, -(2.0 ** 7), 5 * 2.0 ** 7], N // 3)]),
    "mostly_zero": np.where(rng.random(N) < 0.9, 0.0, rng.uniform(0.0, 1e10, N)),
    "signed_zeros": np.where(rng.random(N) < 0.5, -0.0, 0.0),
    "cancelling": np.tile([1e16, 1.0, -1e16, 3.0], N // 4),
    "spikes": np.where(rng.random(N) < 1e-4, 1e300, rng.normal(0.0, 1.0, N)),
    "denormal": rng.normal(0.0, 1.0, N) * 1e-310,
    "infinite": np.concatenate([rng.normal(0.0, 1.0, 1000), [np.inf], rng.normal(0.0, 1.0, 1000)]),
}


@pytest.mark.parametrize("name", sorted(F64_CASES))
def test_sequential_sum_f64_is_the_running_sum(name):
    x = np.asarray(F64_CASES[name], np.float64)
    want = float(np.cumsum(x)[-1])
    got = sequential_sum_f64(x)
    assert same(got, want), (name, got, want)


def test_sequential_sum_f64_short_and_empty():
    assert sequential_sum_f64(np.zeros(0)) == 0.0
    for n in (1, 2, 1023, 1025, 8191, 8193):
        x = rng.normal(0.0, 1e3, n)
        assert same(sequential_sum_f64(x), float(np.cumsum(x)[-1])), n


@pytest.mark.parametrize("W,H,sa,sd", [(64, 32, 0.6, 0.3), (256, 128, 2.5, 5.0), (512, 256, 9.8, 9.8),
                                       (64, 32, 20.0, 20.0), (128, 64, 0.0, 3.0), (128, 64, 4.0, -1.0)])
def test_gaussian_blur_matches_the_oracle(W, H, sa, sd):
    f = (rng.normal(0.0, 100.0, (H, W)) + rng.uniform(-1e3, 1e3)).astype(np.float32)
    want = oracle.gaussian_blur(f, sa, sd)
    got = GaussianBlur.apply(f.copy(), sa, sd)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (W, H, sa, sd)


BOOKS = ("uplifted_cubic_meters", "cut_cubic_meters", "exported_to_sea_cubic_meters",
         "exported_to_land_cubic_meters", "shed_beside_cubic_meters")


def run_both(W, H, seed, params=None, rain=None, cover=None, unresolved=None, shield_cut=True, rebound=True,
             uplift=True, rock=True, window_myr=40.0, sea=None):
    h, up, rk = synthetic.world(W, H, seed)
    t, w, o, win = synthetic.belt_window(W, H, seed, window_myr=window_myr)
    up = up if uplift else None
    rk = rk if rock else None
    params = params or {}
    cfg = ErosionConfig(W, H, seed, **params)
    surface = h.copy()
    got = BeltErosion.replay(cfg, surface, BeltWindow(t, w, o, win), up, rain, cover, rk, sea, shield_cut,
                             unresolved, rebound)
    want_h, want_e, want = oracle.belt_replay(oracle.default_params(W, H, seed, **params), h, t, w, o, win, uplift=up,
                                              rain=rain, cover=cover, rock=rk, provisional_sea_level=sea,
                                              shield_cut=shield_cut, unresolved=unresolved, rebound=rebound)
    return surface, got, want_h, want_e, want, o


def check(surface, got, want_h, want_e, want):
    assert got.rounds == want["rounds"] and got.belt_cells == want["belt_cells"]
    dh = np.flatnonzero(surface.view(np.uint32) != want_h.view(np.uint32))
    assert dh.size == 0, f"{dh.size} heights differ, first {dh[:8]}"
    de = np.flatnonzero(got.eroded_meters.view(np.uint32) != want_e.view(np.uint32))
    assert de.size == 0, f"{de.size} eroded depths differ, first {de[:8]}"
    for k in BOOKS:
        assert same(getattr(got, k), want[k]), (k, getattr(got, k), want[k])


@pytest.mark.parametrize("W,H,seed", [(128, 64, 3), (256, 128, 5), (512, 256, 7), (128, 128, 2)])
def test_replay_matches_the_oracle(W, H, seed):
    surface, got, want_h, want_e, want, o = run_both(W, H, seed)
    assert got.rounds == 106 and got.belt_cells > 0
    check(surface, got, want_h, want_e, want)


def test_replay_with_weather_cover_relief_and_no_rebound():
    W, H, seed = 256, 128, 9
    r = np.random.default_rng(seed)
    rain = r.uniform(100.0, 2500.0, (H, W)).astype(np.float32)
    cover = r.uniform(0.0, 1.0, (H, W)).astype(np.float32)
    unresolved = (r.uniform(0.0, 200.0, (H, W)) / 16000.0).astype(np.float32)
    check(*run_both(W, H, seed, rain=rain, cover=cover, unresolved=unresolved, rebound=False)[:5])


def test_replay_with_slopes_that_shed_beside_the_belts():
    # A critical fall of 2 m/km leaves most belt slopes above it, so the sweeps give every round and
    # the frontier takes what the belts shed; a 30 Myr window; no uplift or rock factors.
    W, H, seed = 256, 128, 4
    surface, got, want_h, want_e, want, o = run_both(W, H, seed, params={"critical_fall_metres_per_km": 2.0},
                                                     uplift=False, rock=False, window_myr=30.0, shield_cut=False)
    assert want["shed_beside_cubic_meters"] != 0.0
    check(surface, got, want_h, want_e, want)


def test_replay_does_nothing_where_the_reference_does_nothing():
    W, H, seed = 128, 64, 3
    h, up, rk = synthetic.world(W, H, seed)
    t, w, o, _ = synthetic.belt_window(W, H, seed)
    cfg = ErosionConfig(W, H, seed)
    for onset, window in ((o, 4.0), (np.full_like(o, -1.0), 40.0)):
        surface = h.copy()
        got = BeltErosion.replay(cfg, surface, BeltWindow(t, w, onset, window), up)
        assert got.rounds == 0 and got.belt_cells == 0 and not got.eroded_meters.any()
        assert np.array_equal(surface, h)


def test_books_close_on_the_device():
    # T:BeltReplayTest.kt:34-53 on the device: the rivers' cut leaves the belts to a part in a million.
    W, H, seed = 512, 256, 13
    h, up, rk = synthetic.world(W, H, seed)
    t, w, o, win = synthetic.belt_window(W, H, seed)
    rain = np.full((H, W), 1000.0, np.float32)
    got = BeltErosion.replay(ErosionConfig(W, H, seed), h.copy(), BeltWindow(t, w, o, win), up, rain,
                             np.zeros((H, W), np.float32), rk, None, False)
    exported = got.exported_to_sea_cubic_meters + got.exported_to_land_cubic_meters
    assert got.cut_cubic_meters > 0.0
    assert abs(got.cut_cubic_meters - exported) / got.cut_cubic_meters <= 1e-6


@pytest.mark.parametrize("W,H,seed,profile", [(256, 128, 5, 0), (128, 64, 3, 2), (128, 64, 7, 3)])
def test_stage_with_the_window_matches_the_oracle(W, H, seed, profile):
    # ErosionStage.apply with ErosionTectonics.window: the initial sweeps, the replay on the resident
    # swept terrain (cg_stage_replay_belts), then the rounds, bit-identical to the oracle's stage; the
    # replay's books are the standalone replay's on the same swept terrain.
    from cartogenesis_gb300 import StageRounds
    h, up, rk = synthetic.world(W, H, seed)
    t, w, o, win = synthetic.belt_window(W, H, seed)
    cfg = ErosionConfig(W, H, seed, profile=profile)
    run = StageRounds(cfg, h, up, rk)
    swept = run.height()
    rep = run.replay_belts(BeltWindow(t, w, o, win))
    run.rounds(cfg.params.hydraulic_rounds)
    got = run.finish(want=("receivers",))
    want = oracle.erode_stage_belts(oracle.default_params(W, H, seed, profile=profile), h, (t, w, o, win), uplift=up,
                                    rock=rk)
    assert np.array_equal(got.height.view(np.uint32), want["height"].view(np.uint32))
    assert np.array_equal(got.receivers, want["receivers"])
    alone = BeltErosion.replay(ErosionConfig(W, H, seed, profile=profile), swept.copy(), BeltWindow(t, w, o, win), up,
                               None, None, rk)
    assert rep.rounds == alone.rounds == 106
    for k in BOOKS:
        assert same(getattr(rep, k), getattr(alone, k)), k
    assert np.array_equal(rep.eroded_meters.view(np.uint32), alone.eroded_meters.view(np.uint32))


def test_replay_matches_the_oracle_at_2048x1024():
    # 158,795 belt cells, 106 rounds, with the rebound's blur at a spread of 2.5 cells; the books close.
    W, H, seed = 2048, 1024, 21
    surface, got, want_h, want_e, want, o = run_both(W, H, seed)
    assert got.belt_cells > 100000
    check(surface, got, want_h, want_e, want)
    exported = got.exported_to_sea_cubic_meters + got.exported_to_land_cubic_meters
    assert abs(got.cut_cubic_meters - exported) / got.cut_cubic_meters <= 1e-6
