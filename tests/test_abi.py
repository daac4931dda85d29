"""The C ABI without a GPU: the library loads, exports every function include/cg_erosion.h declares,
and the ctypes mirror lays the structs out exactly as a C compiler does."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "cg_erosion.h")


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b(cg_[a-z_0-9]+)\s*\(", text)) - {"cg_ctx"})


@pytest.fixture(scope="module")
def lib():
    from cartogenesis_gb300 import build
    build.build()
    return C.CDLL(build.LIB_PATH)


def test_library_exports_every_declared_function(lib):
    from cartogenesis_gb300.runtime import EXPORTS
    names = declared_functions()
    assert len(names) >= 14
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert sorted(EXPORTS) == names


def test_ctypes_structs_match_the_header():
    from cartogenesis_gb300 import abi
    probe = r"""
#include <stdio.h>
#include <stddef.h>
#include "cg_erosion.h"
#define S(T) printf(#T " %zu\n", sizeof(T));
#define O(T, f) printf(#T "." #f " %zu\n", offsetof(T, f));
int main(void) {
  S(cg_erosion_params) S(cg_inputs) S(cg_outputs) S(cg_basins) S(cg_round_stats) S(cg_thermal_limits) S(cg_world)
  O(cg_world, inputs) O(cg_world, outputs)
  O(cg_erosion_params, seed) O(cg_erosion_params, world_width_km) O(cg_erosion_params, years_per_hydraulic_round)
  O(cg_erosion_params, debris_travel_km) O(cg_erosion_params, sea_level) O(cg_erosion_params, profile)
  O(cg_outputs, basins) O(cg_basins, largest) O(cg_round_stats, fill_ties) O(cg_round_stats, ms_total) O(cg_round_stats, ms_relax)
  S(cg_belt_window) S(cg_belt_inputs) S(cg_belt_books) O(cg_belt_window, window_myr)
  O(cg_belt_inputs, provisional_sea_level) O(cg_belt_inputs, history_cell_km) O(cg_belt_books, uplifted_cubic_meters)
  return 0;
}
"""
    with tempfile.TemporaryDirectory() as d:
        src, exe = os.path.join(d, "p.c"), os.path.join(d, "p")
        open(src, "w").write(probe)
        subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), src, "-o", exe])
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split("\n")
    got = dict(line.rsplit(" ", 1) for line in out if line)
    types = {"cg_erosion_params": abi.ErosionParams, "cg_inputs": abi.Inputs, "cg_outputs": abi.Outputs,
             "cg_basins": abi.Basins, "cg_round_stats": abi.RoundStats, "cg_thermal_limits": abi.ThermalLimits,
             "cg_world": abi.World, "cg_belt_window": abi.BeltWindow, "cg_belt_inputs": abi.BeltInputs,
             "cg_belt_books": abi.BeltBooks}
    for k, v in got.items():
        if "." in k:
            t, f = k.split(".")
            assert getattr(types[t], f).offset == int(v), k
        else:
            assert C.sizeof(types[k]) == int(v), k


def test_default_params_match_the_reference_defaults(lib):
    from cartogenesis_gb300 import abi
    import oracle
    p = abi.ErosionParams()
    lib.cg_default_params.argtypes = [C.POINTER(abi.ErosionParams), C.c_int32, C.c_int32, C.c_int64]
    lib.cg_default_params(C.byref(p), 2048, 1024, 1)
    q = oracle.default_params(2048, 1024, 1)
    for f, _ in abi.ErosionParams._fields_:
        assert getattr(p, f) == getattr(q, f), f
    assert p.hydraulic_rounds == 12 and p.abi_version == abi.CG_ABI_VERSION
    lim = abi.ThermalLimits()
    sweeps = C.c_int32()
    lib.cg_thermal_limits_for.argtypes = [C.POINTER(abi.ErosionParams), C.POINTER(abi.ThermalLimits),
                                          C.POINTER(C.c_int32)]
    assert lib.cg_thermal_limits_for(C.byref(p), C.byref(lim), C.byref(sweeps)) == 0
    olim, osweeps = oracle.thermal_limits(q)
    assert (lim.east_west, lim.north_south, lim.diagonal, sweeps.value) == \
        (olim.east_west, olim.north_south, olim.diagonal, osweeps) and osweeps == 96


def test_create_without_a_device_fails_cleanly(lib):
    """No CUDA device here: cg_create reports an error status instead of crashing or falling back."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    h = C.c_void_p()
    lib.cg_create.argtypes = [C.POINTER(C.c_void_p), C.c_int32]
    assert lib.cg_create(C.byref(h), 0) != 0
    assert not h.value
