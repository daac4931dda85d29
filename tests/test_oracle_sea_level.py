"""The oracle's restatement of SeaLevelStage.apply's enclosure rule and drowned-basin outlet passes
(SeaLevelStage.kt:371-437, 478-560), held to the rules as the reference states them:
- with the outlet passes off, the cut is the percentile cut (land stays land) plus the enclosure
  rule: every water body left is the ocean (the largest, the first found of that size) or one larger
  than the largest lake Earth has, and every cell it turned into land stands at its own height
  above the shoreline, (h - s) / landHalfOfField, in float;
- the outlet passes re-cut at the same shoreline, and stop within SeaLevelStage's 16 passes."""
from collections import deque

import numpy as np
import pytest

import oracle
from cartogenesis_gb300 import synthetic


def water_bodies(land):
    """8-connected water bodies, x wrapping, y stopping, numbered from ascending start cells."""
    H, W = land.shape
    body = -np.ones((H, W), np.int64)
    sizes = []
    for r0 in range(H):
        for c0 in range(W):
            if land[r0, c0] or body[r0, c0] >= 0:
                continue
            b = len(sizes)
            body[r0, c0] = b
            q = deque([(r0, c0)])
            n = 0
            while q:
                r, c = q.pop()
                n += 1
                for dr in (-1, 0, 1):
                    rr = r + dr
                    if rr < 0 or rr >= H:
                        continue
                    for dc in (-1, 0, 1):
                        if dr == 0 and dc == 0:
                            continue
                        cc = (c + dc) % W
                        if not land[rr, cc] and body[rr, cc] < 0:
                            body[rr, cc] = b
                            q.append((rr, cc))
            sizes.append(n)
    return body, sizes


@pytest.mark.parametrize("W,H,seed", [(128, 64, 3), (256, 128, 9)])
def test_enclosure_rule(W, H, seed):
    h, _, _ = synthetic.world(W, H, seed)
    p = oracle.default_params(W, H, seed, sea_level=0.70)
    share = 0.00073
    s0, l0, r0, n0 = oracle.percentile_cut(h, 0.70)
    s, land, rel, n, passes = oracle.sea_level_drained_cut(p, h, enclosed_max_share=share, post_cut_outlet=False)
    assert passes == 0 and np.float32(s) == np.float32(s0)
    assert np.all(land[l0 == 1] == 1)   # land stays land
    assert n == int(land.sum())
    world_area = p.world_width_km * p.world_width_km * 0.5
    km2 = (p.world_width_km / W) * (p.world_width_km * 0.5 / H)
    largest_lake = int(share * world_area / km2)
    body, sizes = water_bodies(land.astype(bool))
    if sizes:
        ocean = int(np.argmax(sizes))
        for b, size in enumerate(sizes):
            assert b == ocean or size > largest_lake, (b, size, largest_lake)
    new = (land == 1) & (l0 == 0)
    land_half = np.float32(6000.0) / np.float32(16000.0)
    want = ((h[new] - np.float32(s)) / land_half).astype(np.float32)
    assert np.array_equal(rel[new].view(np.uint32), want.view(np.uint32))
    assert np.array_equal(rel[l0 == 1].view(np.uint32), r0[l0 == 1].view(np.uint32))


def test_outlet_passes_recut_at_the_same_shoreline():
    W, H, seed = 256, 128, 3
    h, _, _ = synthetic.world(W, H, seed)
    p = oracle.default_params(W, H, seed, sea_level=0.70)
    s_off, *_ = oracle.sea_level_drained_cut(p, h, post_cut_outlet=False)
    s, land, rel, n, passes = oracle.sea_level_drained_cut(p, h)
    assert np.float32(s) == np.float32(s_off)
    assert 0 <= passes <= 16
    assert n == int(land.sum())
    # Water stands below the shoreline in relative units (land may too: enclosed lakes).
    assert np.all(rel[land == 0] < 0)
