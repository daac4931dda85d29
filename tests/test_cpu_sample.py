"""The CPU sample the bench times for its CPU baseline and its reference arm: one round of the stage
from the world after its initial sweeps, plus a twelfth of those sweeps. Its rounds must be the
stage's own rounds, so the whole stage taken that way (the initial sweeps, then all 12 sampled
rounds) must equal the oracle's stage bit for bit."""
import numpy as np

import bench
import oracle


def test_stage_rounds_reproduce_the_stage():
    W, H, seed = 256, 128, 3
    h, up, rk = bench.world_inputs(W, H, seed)
    p = oracle.default_params(W, H, seed, sea_level=0.70)
    lim, sweeps = oracle.thermal_limits(p)
    whole = oracle.erode_stage(p, h, up, rk, want=())["height"]
    swept = oracle.thermal_sweep(h, lim, sweeps, p.rate)
    rounds = oracle.stage_rounds(p, swept, up, rk, rounds=12)
    assert np.array_equal(whole.view(np.uint32), rounds.view(np.uint32))
    one = oracle.stage_rounds(p, swept, up, rk, rounds=1)
    assert not np.array_equal(one.view(np.uint32), swept.view(np.uint32))


def test_cpu_sample_runs():
    s = bench.CpuSample(128, 64, 2)
    assert s.share == (s.sweeps + bench.ROUNDS - 1) // bench.ROUNDS
    assert s.step() > 0.0
    assert "128x64" in s.describe(1)
