"""Writes stage_digests.json: SHA-256 digests of the oracle's whole-stage outputs on small seeded
worlds, one per profile (P0 to P3), and of its belts' replay (heights, eroded metres, the books). The reference (Kotlin) cannot run here, so these are not the
reference's own arrays: they pin the oracle to itself, so that a change to the restatement that
moves any output bit is seen, and `tests/test_golden_digests.py` checks them on every CPU run.

Run from the repository root: python tests/golden/make_stage_digests.py
"""
import hashlib
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

import oracle  # noqa: E402
from cartogenesis_gb300 import synthetic  # noqa: E402

WORLDS = [(64, 32, 5), (128, 64, 3), (256, 128, 42)]
PROFILES = [0, 1, 2, 3]
KEYS = ("height", "receivers", "area", "filled", "relative", "is_land", "donors", "basin_of_cell")


def digests(W, H, seed, profile):
    h, up, rk = synthetic.world(W, H, seed)
    out = oracle.erode_stage(oracle.default_params(W, H, seed, sea_level=0.70, profile=profile), h, up, rk,
                             want=KEYS[1:])
    return {k: hashlib.sha256(np.ascontiguousarray(out[k]).tobytes()).hexdigest() for k in KEYS}


def belt_digests(W, H, seed):
    h, up, rk = synthetic.world(W, H, seed)
    t, w, o, win = synthetic.belt_window(W, H, seed)
    hh, eroded, books = oracle.belt_replay(oracle.default_params(W, H, seed), h, t, w, o, win, uplift=up, rock=rk)
    out = {k: hashlib.sha256(np.ascontiguousarray(v).tobytes()).hexdigest() for k, v in
           (("height", hh), ("eroded", eroded))}
    out["books"] = {k: float(v).hex() for k, v in books.items() if isinstance(v, float)}
    out["rounds"], out["belt_cells"] = books["rounds"], books["belt_cells"]
    return out


def main():
    table = {f"{W}x{H}-seed{seed}-P{profile}": digests(W, H, seed, profile)
             for W, H, seed in WORLDS for profile in PROFILES}
    table.update({f"{W}x{H}-seed{seed}-belt": belt_digests(W, H, seed) for W, H, seed in WORLDS})
    with open(os.path.join(HERE, "stage_digests.json"), "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
        f.write("\n")


if __name__ == "__main__":
    main()
