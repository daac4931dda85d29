"""cg_erode_batch: worlds of different planet sizes, grid shapes, seeds and profiles in one call, each
bit-identical to the same world run alone (and to the oracle)."""
import numpy as np
import pytest

import oracle
from cartogenesis_gb300 import CgError, ErosionConfig, ErosionStage, synthetic

pytestmark = pytest.mark.gpu


def worlds():
    out = []
    # (W, H, seed, planet radius in Earth radii, profile)
    for W, H, seed, radius, profile in ((128, 64, 3, 1.0, 0), (64, 32, 5, 0.25, 1), (256, 128, 8, 2.0, 0),
                                        (128, 64, 9, 0.6, 1)):
        h, up, rk = synthetic.world(W, H, seed)
        cfg = ErosionConfig(W, H, seed, sea_level=0.70, world_width_km=40075.0 * radius, profile=profile)
        out.append((cfg, h, up, rk))
    return out


def test_batch_matches_single_worlds_and_the_oracle():
    ws = worlds()
    got = ErosionStage.apply_batch(ws)
    for (cfg, h, up, rk), g in zip(ws, got):
        alone = ErosionStage.apply(cfg, h, up, rk, want=()).height
        assert np.array_equal(g.view(np.uint32), alone.view(np.uint32))
        p = cfg.params
        want = oracle.erode_stage(oracle.default_params(p.width, p.height, p.seed, sea_level=0.70,
                                                        world_width_km=p.world_width_km, profile=p.profile),
                                  h, up, rk, want=())["height"]
        assert np.array_equal(g.view(np.uint32), want.view(np.uint32))


def test_batch_reports_a_bad_world_and_runs_the_rest():
    ws = worlds()[:2]
    bad = ErosionConfig(96, 64, 1)   # not a power of two across
    with pytest.raises(CgError, match=r"worlds \[0\]"):
        ErosionStage.apply_batch([(bad, np.zeros((64, 96), np.float32), None, None)] + ws[1:])
