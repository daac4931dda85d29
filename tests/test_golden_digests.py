"""A regression lock: the oracle's whole-stage outputs on small seeded worlds, for every profile, against the committed
digests (tests/golden/stage_digests.json, written by tests/golden/make_stage_digests.py): any change
to the restatement that moves an output bit shows here. The GPU is held to the oracle itself by the
parity tests."""
import json
import os
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import make_stage_digests as golden  # noqa: E402

TABLE = json.load(open(os.path.join(HERE, "golden", "stage_digests.json")))


@pytest.mark.parametrize("W,H,seed", golden.WORLDS)
@pytest.mark.parametrize("profile", golden.PROFILES)
def test_oracle_stage_matches_committed_digests(W, H, seed, profile):
    want = TABLE[f"{W}x{H}-seed{seed}-P{profile}"]
    got = golden.digests(W, H, seed, profile)
    assert got == want


@pytest.mark.parametrize("W,H,seed", golden.WORLDS)
def test_oracle_belt_replay_matches_committed_digests(W, H, seed):
    assert golden.belt_digests(W, H, seed) == TABLE[f"{W}x{H}-seed{seed}-belt"]
