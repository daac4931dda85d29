"""SeaLevelStage.apply's cut with the enclosure rule and the drowned basins' outlets on the GPU
(cg_sea_level_cut; SeaLevelStage.kt:243-270, 371-437, 478-560), against the oracle: the shoreline,
the land mask, the relative field (bit for bit) and the number of outlet passes. This is the
reference reusing the erosion stage's routing outside the stage: each outlet pass is a fill, a
facet routing with flats, an accumulation and the spillways over the whole grid, then the outlet
notch with belowSea."""
import numpy as np
import pytest

import oracle
from cartogenesis_gb300 import ErosionConfig, SeaLevelStage, synthetic

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("W,H,seed,outlet", [(256, 128, 3, True), (512, 256, 7, True), (512, 256, 7, False),
                                             (1024, 512, 1, True), (2048, 1024, 5, True)])
def test_drained_cut_matches_the_oracle(W, H, seed, outlet):
    h, _, _ = synthetic.world(W, H, seed)
    cfg = ErosionConfig(W, H, seed, sea_level=0.70)
    s1, l1, r1, n1, p1 = SeaLevelStage.drained_cut(cfg, h, post_cut_outlet=outlet)
    s0, l0, r0, n0, p0 = oracle.sea_level_drained_cut(oracle.default_params(W, H, seed, sea_level=0.70), h,
                                                       post_cut_outlet=outlet)
    assert np.float32(s0).view(np.uint32) == np.float32(s1).view(np.uint32)
    assert (n0, p0) == (n1, p1)
    assert np.array_equal(l0, l1)
    diff = np.flatnonzero(r0.view(np.uint32) != r1.view(np.uint32))
    assert diff.size == 0, f"{diff.size} relative cells differ: {diff[:8]}"


def test_drained_cut_after_the_stage():
    """On the terrain a P1 stage leaves, as the engine runs it (the sea-level stage follows erosion)."""
    from cartogenesis_gb300 import ErosionStage
    W, H, seed = 512, 256, 11
    h, up, rk = synthetic.world(W, H, seed)
    eroded = ErosionStage.apply(ErosionConfig(W, H, seed, sea_level=0.70, profile=1), h, up, rk, want=()).height
    cfg = ErosionConfig(W, H, seed, sea_level=0.70)
    s1, l1, r1, n1, p1 = SeaLevelStage.drained_cut(cfg, eroded)
    s0, l0, r0, n0, p0 = oracle.sea_level_drained_cut(oracle.default_params(W, H, seed, sea_level=0.70), eroded)
    assert (n0, p0) == (n1, p1)
    assert np.array_equal(l0, l1) and np.array_equal(r0.view(np.uint32), r1.view(np.uint32))
