"""Property tests of the oracle's round tail over many seeded worlds (hypothesis picks the seeds,
sizes and sea levels): the outlet notch's invariants and the deposition's mass budget hold on every
world, not only on the fixtures."""
import numpy as np
import pytest

hypothesis = pytest.importorskip("hypothesis")
from hypothesis import given, settings, strategies as st  # noqa: E402

import oracle  # noqa: E402
from cartogenesis_gb300 import synthetic  # noqa: E402

LATTICE = 214


@settings(max_examples=25, deadline=None)
@given(seed=st.integers(1, 10_000), shape=st.sampled_from([(64, 32), (128, 64), (128, 128)]),
       sea_level=st.sampled_from([0.55, 0.70, 0.85]))
def test_notch_only_cuts_down_channels_and_margins(seed, shape, sea_level):
    W, H = shape
    h, _, _ = synthetic.world(W, H, seed)
    p = oracle.default_params(W, H, seed, sea_level=sea_level)
    _, land, rel, n = oracle.percentile_cut(h, sea_level)
    filled = oracle.fill_depressions(land, rel)
    flow, _ = oracle.flow_directions(land, rel, filled, seed, 0.5 * W / H, LATTICE)
    area = oracle.accumulate(land, flow, n, np.ones((H, W), np.float32))
    r2, f2, s2 = rel.copy(), filled.copy(), h.copy()
    cells, moved = oracle.breach(p, land, r2, f2, flow, area, float(n), 0.375, s2)
    changed = np.flatnonzero(s2.ravel() != h.ravel())
    assert changed.size <= cells   # a cell on two basins' channels is cut by each
    assert np.all(s2.ravel()[changed] < h.ravel()[changed])
    assert np.array_equal(np.flatnonzero(r2.ravel() != rel.ravel()), changed)
    assert np.all(land.ravel()[changed] == 1)
    assert np.all(r2.ravel()[changed] >= -1e-6)
    pond = oracle.rates(p)[2]
    was_ponded = (filled - rel).ravel() > pond
    assert np.array_equal(np.flatnonzero(f2.ravel() != filled.ravel()), changed[~was_ponded[changed]])
    assert moved >= 0.0


@settings(max_examples=10, deadline=None)
@given(seed=st.integers(1, 10_000), shape=st.sampled_from([(64, 32), (128, 64)]))
def test_deposition_budget_closes_every_round(seed, shape):
    W, H = shape
    h, up, rk = synthetic.world(W, H, seed)
    p = oracle.default_params(W, H, seed, sea_level=0.70, profile=2)
    _, tallies = oracle.erode_stage_switched(p, h, up, rk)
    for incised, deposited, lost, drop in tallies:
        assert abs(incised - (deposited + lost)) <= 0.01 * max(incised, 1e-12)
        assert abs(drop - lost) <= 0.01 * max(lost, 1e-12) + 1e-9
