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


def test_batch_of_the_batched_workload_shapes():
    """The batched workload's shape mix: planets of radius U(0.25, 2.0) Earth radii, grids 512 x 256 to
    2048 x 1024 (the nearest power of two to 1024 r rows, capped at 1024 here to keep the test short),
    each world's own seed, P0 and P1 alternating. Every world equals the same world run alone, and the
    worlds up to 1024 x 512 equal the oracle too."""
    shapes = synthetic.batch_shapes(12, seed=2, max_rows=1024)
    shapes += [(512, 256, 77, 0.3), (1024, 512, 78, 0.6)]   # make sure both small shapes are present
    ws = []
    for i, (W, H, seed, radius) in enumerate(shapes):
        h, up, rk = synthetic.world(W, H, seed, uplift="ridges" if i % 3 == 0 else "bands")
        cfg = ErosionConfig(W, H, seed, sea_level=0.70, world_width_km=40075.0 * radius, profile=i % 2)
        ws.append((cfg, h, up, rk))
    got = ErosionStage.apply_batch(ws)
    for (cfg, h, up, rk), g in zip(ws, got):
        p = cfg.params
        alone = ErosionStage.apply(cfg, h, up, rk, want=()).height
        assert np.array_equal(g.view(np.uint32), alone.view(np.uint32)), (p.width, p.height, p.seed)
        if p.height <= 512:
            want = oracle.erode_stage(oracle.default_params(p.width, p.height, p.seed, sea_level=0.70,
                                                            world_width_km=p.world_width_km, profile=p.profile),
                                      h, up, rk, want=())["height"]
            assert np.array_equal(g.view(np.uint32), want.view(np.uint32)), (p.width, p.height, p.seed)
