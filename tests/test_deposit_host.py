"""The device's deposition logic (cartogenesis_gb300/csrc/cg_deposit.cuh: a cell's own walk, the
outlined lobes and lake fans) built for the host and run on rounds captured from the oracle, in the
reference's order, in the device's level order, with a level's fans in waves, and with every lake
fan's admission done first and out of order: the sediment, settled heights and loads it leaves must
be the oracle walk's, bit for bit."""
import ctypes as C
import os
import subprocess
import tempfile

import numpy as np
import pytest

import oracle
from cartogenesis_gb300 import abi, synthetic

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def host():
    d = tempfile.mkdtemp()
    lib = os.path.join(d, "libdeposit_host.so")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
                           "-I", os.path.join(ROOT, "include"), "-o", lib,
                           os.path.join(HERE, "native", "deposit_host.cpp")])
    L = C.CDLL(lib)
    vp = C.c_void_p
    L.dep_walk.argtypes = [C.c_int, C.POINTER(abi.ErosionParams), C.c_float, C.c_float, C.c_float, C.c_float, vp,
                           C.c_int] + [vp] * 10 + [C.c_int, vp, vp]
    L.dep_walk.restype = C.c_int
    return L


def run(host, mode, params, c):
    sediment, settled = c["sediment"].copy(), c["settled"].copy()
    arriving = np.zeros_like(c["load"])
    repairs = np.zeros(4, np.int64)
    P = abi.ptr
    st = host.dep_walk(mode, C.byref(params), c["land_cells"], c["land_range"], c["to_relative"], c["shoreline"],
                       P(c["order"]), len(c["order"]), P(c["dirs"]), P(c["land"]), P(c["ground"]), P(c["relative"]),
                       P(c["area"]), P(c["surface"]), P(sediment), P(settled), P(c["load"]), P(c["incised_at"]),
                       c["mouth_id"], P(arriving), P(repairs))
    assert st == 0, st
    return sediment, settled, arriving, tuple(repairs)


@pytest.mark.parametrize("W,H,seed,uplift,rounds", [
    (256, 128, 42, "bands", (0, 5, 11)),
    (512, 256, 7, "bands", (0, 3)),
    (2048, 1024, 1, "ridges", (0,)),
])
def test_device_walk_matches_the_oracle(host, W, H, seed, uplift, rounds):
    h, up, rk = synthetic.world(W, H, seed, uplift=uplift)
    p = oracle.default_params(W, H, seed, sea_level=0.70, profile=2)
    for r in rounds:
        c = oracle.capture_walk(p, h, up, rk, r)
        land = c["land"].astype(bool)
        # The wave mode's host emulation is quadratic in the fans of a crowded level: small worlds only.
        for mode in ((0, 1, 2, 3, 4, 5) if W * H <= 512 * 256 else (0, 1, 3, 4, 5)):
            sediment, settled, arriving, repairs = run(host, mode, p, c)
            assert np.array_equal(sediment.view(np.uint32), c["sediment_after"].view(np.uint32)), (r, mode)
            assert np.array_equal(settled.view(np.uint32), c["settled_after"].view(np.uint32)), (r, mode)
            assert np.array_equal(arriving[land].view(np.uint64), c["load_after"][land].view(np.uint64)), (r, mode)
