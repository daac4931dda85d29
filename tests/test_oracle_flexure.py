"""The oracle's restatement of the plate flexure (Isostasy.Flexure over Fft2D; Isostasy.kt:277-411,
math/Fft.kt), pinned by the reference's own IsostasyTest (T/IsostasyTest.kt:219-362, rebuilt from its
constants): a broad load sinks to Airy's answer, a narrow one is held up, the bend carries no mean,
the flexural parameter is a continent's, and a load on one pole does not bend the other."""
import math

import numpy as np
import pytest

import oracle

KM_PER_METRE = 1e-3


def params(W, H):
    return oracle.default_params(W, H, 1)


def test_broad_load_sinks_to_airy_and_a_narrow_one_is_held_up():
    W = H = 256
    p = params(W, H)
    load_metres = np.float32(1000.0)
    pascals = np.float32(load_metres * np.float32(p.continental_crust_density) * np.float32(p.gravity))
    airy = float(load_metres * np.float32(p.continental_crust_density) /
                 (np.float32(p.mantle_density) - np.float32(p.deflection_fill_density)))

    def deflection_under(half):
        load = np.zeros((H, W), np.float32)
        rows = np.abs(np.arange(H) - H // 2) <= half
        cols = np.abs(np.arange(W) - W // 2) <= half
        load[np.ix_(rows, cols)] = pascals
        out, rigidity, restoring = oracle.flexure_deflection(p, load)
        assert abs(float(out.astype(np.float64).mean())) <= 1e-6   # no mean: the datum is not the plate's
        return float(out[H // 2, W // 2]), rigidity, restoring

    broad, rigidity, restoring = deflection_under(16)
    narrow, _, _ = deflection_under(0)
    alpha_km = math.sqrt(math.sqrt(4.0 * rigidity / restoring)) * KM_PER_METRE
    assert 50.0 <= alpha_km <= 200.0
    assert broad == pytest.approx(airy, abs=airy * 0.05)
    assert narrow < airy * 0.5


def test_a_load_on_one_pole_does_not_bend_the_other():
    H = 512
    W = 2 * H
    p = params(W, H)
    load = np.zeros((H, W), np.float32)
    load[0, :] = np.float32(np.float32(1000.0) * np.float32(p.continental_crust_density) * np.float32(p.gravity))
    out, _, _ = oracle.flexure_deflection(p, load)
    middle = float(out[H // 2, 0])
    near = float(out[1, 0]) - middle
    far = float(out[H - 1, 0]) - middle
    assert abs(near) > 10.0                 # MIN_STRIPE_DEFLECTION_METRES
    assert abs(far) / abs(near) < 1e-6      # FAR_POLE_SHARE_OF_NEAR_ROW


def test_fft_round_trip():
    """Fft2D.inverse(forward(f)) is f to rounding (the transform and its 1 / (w h))."""
    p = params(64, 32)
    rng = np.random.default_rng(1)
    load = rng.standard_normal((32, 64)).astype(np.float32) * np.float32(1e6)
    # A flexure with no stiffness and unit restoring force is the identity less the mean.
    p.elastic_thickness_km = 0.0
    p.mantle_density = 1.0
    p.deflection_fill_density = 0.0
    p.gravity = 1.0
    out, _, _ = oracle.flexure_deflection(p, load)
    want = load.astype(np.float64) - load.astype(np.float64).mean()
    assert np.allclose(out, want, rtol=1e-5, atol=1e-3 * np.abs(want).max())


def test_stripped_ground_rebounds_in_the_stage():
    """IsostasyTest's `a stripped range rebounds and its foreland sinks` (T/IsostasyTest.kt:790-850) in
    the form this stage can show without the plate history: the same world with the flexure on
    (profile P3) and off (P2). The first round's load is nothing, so its bend is nothing (the
    reference says so: HydraulicErosion.kt:853-854); after twelve rounds the ground the rounds cut
    most stands higher with the flexure on, since a loss is a negative load and the plate answers it
    upward, by a good share of what was cut (on cells of 156 km the plate answers almost locally, so
    the share approaches Airy's 2835 / 3300 for a loss as broad as a cell)."""
    from cartogenesis_gb300 import synthetic
    W, H, seed = 256, 128, 4
    h, up, rk = synthetic.world(W, H, seed)

    def heights(profile, rounds):
        p = oracle.default_params(W, H, seed, sea_level=0.70, profile=profile, hydraulic_rounds=rounds)
        return oracle.erode_stage(p, h, up, rk)["height"].astype(np.float64)

    one2, one3 = heights(2, 1), heights(3, 1)
    assert np.abs(one3 - one2).max() * 16000.0 < 1e-3   # no bend after the first round
    p2, p3 = heights(2, 12), heights(3, 12)
    cut = (h.astype(np.float64) - p2) * 16000.0
    stripped = cut > np.quantile(cut, 0.99)             # the most eroded cells
    rebound = float(((p3 - p2) * 16000.0)[stripped].mean())
    assert rebound > 0.1 * float(cut[stripped].mean()), (rebound, float(cut[stripped].mean()))
