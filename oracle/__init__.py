"""TEST INFRASTRUCTURE ONLY - the oracle.

A CPU restatement of Cartogenesis's erosion stage (cg_oracle.cpp), loaded through ctypes. Only
the tests, the smoke check and bench.py's CPU-baseline leg may use it, and only as the checker or
the timed CPU stand-in; the product path (cartogenesis_gb300) never imports it.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from cartogenesis_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "liboracle.so")
SOURCES = [os.path.join(HERE, "cg_oracle.cpp")]
# -ffp-contract=off: the JVM never fuses a multiply and an add, and neither may the restatement.
CXXFLAGS = ["-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared", "-Wall"]


def build(force=False):
    """Compile the oracle into oracle/_build/liboracle.so (seconds)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    newest = max(os.path.getmtime(s) for s in SOURCES + [os.path.join(HERE, "..", "include", "cg_erosion.h")])
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= newest:
        return LIB_PATH
    tmp = LIB_PATH + f".{os.getpid()}.tmp"
    subprocess.check_call(["g++", *CXXFLAGS, "-o", tmp, *SOURCES])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        vp, i32, i64, f32, f64 = C.c_void_p, C.c_int32, C.c_int64, C.c_float, C.c_double
        L.or_default_params.argtypes = [C.POINTER(abi.ErosionParams), i32, i32, i64]
        L.or_thermal_limits.argtypes = [C.POINTER(abi.ErosionParams), C.POINTER(abi.ThermalLimits), C.POINTER(i32)]
        L.or_thermal_sweep.argtypes = [i32, i32, vp, vp, f32, f32, f32, i32, f32, i32]
        L.or_percentile_cut.argtypes = [i32, i32, vp, f32, f32, f32, f32, C.POINTER(f32), vp, vp]
        L.or_percentile_cut.restype = i32
        L.or_fill_depressions.argtypes = [i32, i32, vp, vp, vp]
        L.or_flow_directions.argtypes = [i32, i32, vp, vp, vp, i64, f64, i32, i32, i32, vp, vp, vp]
        L.or_drainage_order.argtypes = [i32, i32, vp, vp, i32, vp]
        L.or_accumulate.argtypes = [i32, i32, vp, vp, i32, vp, vp]
        L.or_spillways.argtypes = [i32, i32, vp, vp, vp, vp, f32, vp, C.POINTER(abi.Basins)]
        L.or_spillways.restype = i32
        L.or_incise.argtypes = [C.POINTER(abi.ErosionParams), vp, i32, vp, vp, vp, vp, vp, f32, f32, f32, vp, vp,
                                i32, vp]
        L.or_breach.argtypes = [C.POINTER(abi.ErosionParams), vp, vp, vp, vp, vp, f32, f32, vp, C.POINTER(f64)]
        L.or_breach.restype = i32
        L.or_outlet_rates.argtypes = [C.POINTER(abi.ErosionParams), C.POINTER(f32), C.POINTER(f32), C.POINTER(i32)]
        L.or_erode_stage_switched.argtypes = [C.POINTER(abi.ErosionParams), C.POINTER(abi.Inputs),
                                              C.POINTER(abi.Outputs), vp, vp, i32]
        L.or_erode_stage_switched.restype = i32
        L.or_erode_stage_levels.argtypes = [C.POINTER(abi.ErosionParams), C.POINTER(abi.Inputs),
                                            C.POINTER(abi.Outputs), vp]
        L.or_erode_stage_levels.restype = i32
        L.or_capture_walk.argtypes = [C.POINTER(abi.ErosionParams), C.POINTER(abi.Inputs), i32] + [vp] * 16
        L.or_capture_walk.restype = i32
        L.or_rates.argtypes = [C.POINTER(abi.ErosionParams), C.POINTER(f32), C.POINTER(f32), C.POINTER(f32)]
        L.or_stand_below_today.argtypes = [C.POINTER(abi.ErosionParams), i32]
        L.or_stand_below_today.restype = f32
        L.or_seeded_noise.argtypes = [i32, i32, i64]
        L.or_seeded_noise.restype = f32
        L.or_smooth_seeded_field.argtypes = [i32, i32, i32, i32, i64]
        L.or_smooth_seeded_field.restype = f32
        L.or_erode_stage.argtypes = [C.POINTER(abi.ErosionParams), C.POINTER(abi.Inputs), C.POINTER(abi.Outputs),
                                     vp]
        L.or_erode_stage.restype = i32
        L.or_stage_rounds.argtypes = [C.POINTER(abi.ErosionParams), C.POINTER(abi.Inputs), C.POINTER(abi.Outputs),
                                      i32]
        L.or_stage_rounds.restype = i32
        L.or_hydraulic_apply.argtypes = L.or_erode_stage.argtypes
        L.or_hydraulic_apply.restype = i32
        L.or_erode_stage_fed.argtypes = [C.POINTER(abi.ErosionParams), C.POINTER(abi.Inputs),
                                         C.POINTER(abi.Inputs), C.POINTER(abi.Outputs)]
        L.or_erode_stage_fed.restype = i32
        L.or_sea_level_drained_cut.argtypes = [C.POINTER(abi.ErosionParams), vp, f64, i32, C.POINTER(f32), vp, vp,
                                               C.POINTER(i32), C.POINTER(i32)]
        L.or_sea_level_drained_cut.restype = i32
        L.or_flexure_deflection.argtypes = [C.POINTER(abi.ErosionParams), vp, vp, C.POINTER(f64), C.POINTER(f64)]
        L.or_flexure_deflection.restype = i32
        L.or_belt_replay.argtypes = [C.POINTER(abi.ErosionParams), vp, vp, vp, vp, f64, vp, vp, vp, vp, f32, i32, vp,
                                     i32, f64, vp, vp, vp]
        L.or_belt_replay.restype = i32
        L.or_gaussian_blur.argtypes = [i32, i32, vp, f64, f64]
        L.or_flat_stencil.argtypes = [f64, vp]
        L.or_grow_fan_fixture.argtypes = [i32, i32, i32, f64, f32, f32, f32, i32, i32, f32, vp, i32, vp]
        L.or_grow_fan_fixture.restype = f64
        L.or_fan_hash.argtypes = [i64, i32]
        L.or_fan_hash.restype = i32
        L.or_facet_flip_delta.argtypes = [i32, i32, vp, vp, vp, i64, f64, vp]
        L.or_erode_stage_belts.argtypes = [C.POINTER(abi.ErosionParams), C.POINTER(abi.Inputs), vp, vp, vp, f64, i32,
                                           f64, C.POINTER(abi.Outputs)]
        L.or_erode_stage_belts.restype = i32
        _lib = L
    return _lib


P = abi.ptr


def default_params(width, height, seed=1, **overrides):
    p = abi.ErosionParams()
    lib().or_default_params(C.byref(p), width, height, seed)
    for k, v in overrides.items():
        setattr(p, k, v)
    return p


def thermal_limits(params):
    lim = abi.ThermalLimits()
    sweeps = C.c_int32()
    lib().or_thermal_limits(C.byref(params), C.byref(lim), C.byref(sweeps))
    return lim, sweeps.value


def thermal_sweep(height, limits, sweeps, rate=0.25, skip=True):
    h = np.ascontiguousarray(height, dtype=np.float32)
    H, W = h.shape
    out = np.empty_like(h)
    lib().or_thermal_sweep(W, H, P(h), P(out), limits.east_west, limits.north_south, limits.diagonal, sweeps,
                           rate, 1 if skip else 0)
    return out


def percentile_cut(height, sea_level, lowstand_share=0.0, highest_land=6000.0, deepest_ocean=10000.0):
    h = np.ascontiguousarray(height, dtype=np.float32)
    H, W = h.shape
    is_land = np.empty((H, W), np.uint8)
    rel = np.empty((H, W), np.float32)
    s = C.c_float()
    n = lib().or_percentile_cut(W, H, P(h), sea_level, highest_land, deepest_ocean, lowstand_share, C.byref(s),
                                P(is_land), P(rel))
    return s.value, is_land, rel, n


def fill_depressions(is_land, relative):
    H, W = relative.shape
    il = np.ascontiguousarray(is_land, dtype=np.uint8)
    rel = np.ascontiguousarray(relative, dtype=np.float32)
    out = np.empty_like(rel)
    lib().or_fill_depressions(W, H, P(il), P(rel), P(out))
    return out


def flow_directions(is_land, relative, filled, seed, r, lattice, by_facet=True, over_potential=True,
                    want_surface=False):
    H, W = relative.shape
    il = np.ascontiguousarray(is_land, dtype=np.uint8)
    rel = np.ascontiguousarray(relative, dtype=np.float32)
    fil = np.ascontiguousarray(filled, dtype=np.float32)
    rec = np.empty((H, W), np.int32)
    surf = np.empty((H, W), np.float64) if want_surface else None
    counts = np.zeros(3, np.int32)
    lib().or_flow_directions(W, H, P(il), P(rel), P(fil), seed, r, lattice, int(by_facet), int(over_potential),
                             P(rec), P(surf), P(counts))
    return (rec, surf, counts) if want_surface else (rec, counts)


def drainage_order(is_land, receivers, land_cells):
    H, W = receivers.shape
    il = np.ascontiguousarray(is_land, dtype=np.uint8)
    rec = np.ascontiguousarray(receivers, dtype=np.int32)
    order = np.empty(max(land_cells, 1), np.int32)
    lib().or_drainage_order(W, H, P(il), P(rec), land_cells, P(order))
    return order[:land_cells]


def accumulate(is_land, receivers, land_cells, weights):
    H, W = receivers.shape
    il = np.ascontiguousarray(is_land, dtype=np.uint8)
    rec = np.ascontiguousarray(receivers, dtype=np.int32)
    w = np.ascontiguousarray(weights, dtype=np.float32)
    area = np.empty((H, W), np.float32)
    lib().or_accumulate(W, H, P(il), P(rec), land_cells, P(w), P(area))
    return area


def spillways(is_land, relative, filled, receivers, pond_depth):
    H, W = relative.shape
    N = W * H
    il = np.ascontiguousarray(is_land, dtype=np.uint8)
    rel = np.ascontiguousarray(relative, dtype=np.float32)
    fil = np.ascontiguousarray(filled, dtype=np.float32)
    rec = np.ascontiguousarray(receivers, dtype=np.int32)
    labels = np.empty((H, W), np.int32)
    arrays = {k: np.empty(N, dt) for k, dt in
              [("spill", np.int32), ("entry", np.int32), ("level", np.float32), ("floor", np.float32),
               ("cells", np.int32)]}
    b = abi.Basins(capacity=N, count=0, **{k: P(v) for k, v in arrays.items()})
    n = lib().or_spillways(W, H, P(il), P(rel), P(fil), P(rec), pond_depth, P(labels), C.byref(b))
    out = {k: v[:n].copy() for k, v in arrays.items()}
    out.update(count=n, largest=b.largest, largest_cells=b.largest_cells, largest_depth=b.largest_depth,
               deepest=b.deepest, labels=labels)
    return out


def rates(params):
    a, b, c = C.c_float(), C.c_float(), C.c_float()
    lib().or_rates(C.byref(params), C.byref(a), C.byref(b), C.byref(c))
    return a.value, b.value, c.value


def incise(params, order, directions, is_land, ground, relative, discharge, land_cells, land_range, shoreline,
           erodibility, surface, only_above_base=True, unresolved=None):
    """HydraulicErosion.incise; `surface` (float32, contiguous) is updated in place."""
    dts = (np.int32, np.int32, np.uint8, np.float32, np.float32, np.float32, np.float32)
    # Held in locals for the whole call: ctypes only sees their addresses.
    order, directions, is_land, ground, relative, discharge, erodibility = [
        np.ascontiguousarray(a, dtype=dt).ravel() for a, dt in
        zip((order, directions, is_land, ground, relative, discharge, erodibility), dts)]
    unresolved = None if unresolved is None else np.ascontiguousarray(unresolved, np.float32)
    assert surface.dtype == np.float32 and surface.flags.c_contiguous
    lib().or_incise(C.byref(params), P(order), len(order), P(directions), P(is_land), P(ground), P(relative),
                    P(discharge), land_cells, land_range, shoreline, P(erodibility), P(surface),
                    int(only_above_base), P(unresolved))


def outlet_rates(params):
    """(relativeIncisionCoefficient, notchFallPerCell, outletReachCells) of HydraulicErosion.Rates."""
    a, b, c = C.c_float(), C.c_float(), C.c_int32()
    lib().or_outlet_rates(C.byref(params), C.byref(a), C.byref(b), C.byref(c))
    return a.value, b.value, c.value


def breach(params, is_land, relative, ground, directions, area, land_cells, land_range, surface):
    """HydraulicErosion.breach over the basins of this routing. `relative`, `ground` and `surface`
    (float32, contiguous) are cut in place; returns (cells cut, amount moved)."""
    for a in (relative, ground, surface):
        assert a.dtype == np.float32 and a.flags.c_contiguous
    il = np.ascontiguousarray(is_land, dtype=np.uint8)
    rec = np.ascontiguousarray(directions, dtype=np.int32)
    ar = np.ascontiguousarray(area, dtype=np.float32)
    moved = C.c_double()
    cells = lib().or_breach(C.byref(params), P(il), P(relative), P(ground), P(rec), P(ar), land_cells, land_range,
                            P(surface), C.byref(moved))
    return cells, moved.value


class Switches(C.Structure):
    """or_switches: the round tail's switches and the deposition's knobs, reference defaults."""
    _fields_ = [("outlet_incision", C.c_int32), ("deposition", C.c_int32), ("delta_lobe", C.c_int32),
                ("graded_aggradation", C.c_int32), ("delta_outline", C.c_int32), ("transport_capacity", C.c_float),
                ("deposition_rate", C.c_float), ("delta_share", C.c_float), ("lake_share", C.c_float),
                ("delta_min_catchment_km2", C.c_double), ("delta_reach_km", C.c_double),
                ("delta_freeboard_metres", C.c_float)]

    def __init__(self, profile=2, **knobs):
        on = profile >= 2
        super().__init__(int(profile >= 1), int(on), int(on), int(on), int(on), 20.0, 0.06, 0.15, 0.1, 70000.0,
                         140.625, 48.0)
        for k, v in knobs.items():
            setattr(self, k, v)


def erode_stage_switched(params, height, uplift=None, rock=None, switches=None, thermal=True):
    """The stage with explicit switches; returns (heights, tallies[rounds, 4]) where a tally is
    (incised, deposited, lost, field drop) of one round."""
    H, W = params.height, params.width
    keep = [None if a is None else np.ascontiguousarray(a, dtype=np.float32).reshape(H, W)
            for a in (height, uplift, rock)]
    inputs = abi.Inputs(*[P(a) if a is not None else None for a in keep], None, None)
    out = np.empty((H, W), np.float32)
    o = abi.Outputs(height=P(out))
    tallies = np.zeros((max(params.hydraulic_rounds, 1), 4), np.float64)
    sw = switches if switches is not None else Switches(params.profile)
    st = lib().or_erode_stage_switched(C.byref(params), C.byref(inputs), C.byref(o), C.byref(sw), P(tallies),
                                       int(thermal))
    assert st == 0, st
    return out, tallies


def erode_stage_levels(params, height, uplift=None, rock=None):
    """The stage with the deposition walk in the device's level order; returns (heights, (ponded cells
    replayed, levels redone))."""
    H, W = params.height, params.width
    keep = [None if a is None else np.ascontiguousarray(a, dtype=np.float32).reshape(H, W)
            for a in (height, uplift, rock)]
    inputs = abi.Inputs(*[P(a) if a is not None else None for a in keep], None, None)
    out = np.empty((H, W), np.float32)
    o = abi.Outputs(height=P(out))
    repairs = np.zeros(2, np.int64)
    st = lib().or_erode_stage_levels(C.byref(params), C.byref(inputs), C.byref(o), P(repairs))
    assert st == 0, st
    return out, tuple(int(v) for v in repairs)


def capture_walk(params, height, uplift=None, rock=None, round_=0):
    """The P2 stage's deposition walk of one round: its inputs and, after the reference's order, the
    sediment, settled heights and loads. Returns a dict of arrays and scalars."""
    H, W = params.height, params.width
    N = W * H
    keep = [None if a is None else np.ascontiguousarray(a, dtype=np.float32).reshape(H, W)
            for a in (height, uplift, rock)]
    inputs = abi.Inputs(*[P(a) if a is not None else None for a in keep], None, None)
    spec = [("order", np.int32), ("dirs", np.int32), ("land", np.uint8), ("ground", np.float32),
            ("relative", np.float32), ("area", np.float32), ("surface", np.float32), ("sediment", np.float32),
            ("settled", np.float32), ("load", np.float64), ("incised_at", np.float64)]
    a = {k: np.zeros(N, dt) for k, dt in spec}
    scalars = np.zeros(4, np.float32)
    ints = np.zeros(2, np.int32)
    after = {k: np.zeros(N, dt) for k, dt in [("sediment_after", np.float32), ("settled_after", np.float32),
                                               ("load_after", np.float64)]}
    st = lib().or_capture_walk(C.byref(params), C.byref(inputs), round_, *[P(a[k]) for k, _ in spec], P(scalars),
                               P(ints), *[P(v) for v in after.values()])
    assert st == 0, st
    a.update(after)
    a["order"] = a["order"][:ints[0]]
    a.update(land_cells=float(scalars[0]), land_range=float(scalars[1]), to_relative=float(scalars[2]),
             shoreline=float(scalars[3]), mouth_id=int(ints[1]))
    return a


def stand_below_today(params, round_):
    return lib().or_stand_below_today(C.byref(params), round_)


def seeded_noise(c, r, seed):
    return lib().or_seeded_noise(c, r, seed)


def stage_rounds(params, height, uplift=None, rock=None, rounds=1):
    """The first `rounds` rounds of the stage from already swept heights (no initial sweeps)."""
    H, W = params.height, params.width
    keep = [None if a is None else np.ascontiguousarray(a, dtype=np.float32).reshape(H, W)
            for a in (height, uplift, rock)]
    inputs = abi.Inputs(*[P(a) if a is not None else None for a in keep], None, None)
    out = np.empty((H, W), np.float32)
    o = abi.Outputs(height=P(out))
    st = lib().or_stage_rounds(C.byref(params), C.byref(inputs), C.byref(o), rounds)
    assert st == 0, st
    return out


def erode_stage(params, height, uplift=None, rock=None, rain=None, veg=None, thermal=True, want=("receivers", "area", "filled",
                                                                                    "relative", "is_land", "order",
                                                                                    "basin_of_cell", "donors"),
                refreshed=None):
    """The whole stage on the oracle. refreshed = (rain, veg) (either may be None) is the weather of the
    halfway refresh when params.climate_feed is set; (rain, veg) is then the opening weather."""
    H, W = params.height, params.width
    N = W * H
    keep = []

    def f32(a):
        if a is None:
            return None
        a = np.ascontiguousarray(a, dtype=np.float32).reshape(H, W)
        keep.append(a)
        return a

    h, up, rk, rn, vg = map(f32, (height, uplift, rock, rain, veg))
    inputs = abi.Inputs(P(h), P(up), P(rk), P(rn), P(vg))
    outs = {"height": np.empty((H, W), np.float32)}
    kinds = {"receivers": np.int32, "area": np.float32, "filled": np.float32, "relative": np.float32,
             "is_land": np.uint8, "order": np.int32, "basin_of_cell": np.int32, "donors": np.int32}
    for k in want:
        outs[k] = np.empty((H, W), kinds[k])
    basins_arrays = {k: np.empty(N, dt) for k, dt in
                     [("spill", np.int32), ("entry", np.int32), ("level", np.float32), ("floor", np.float32),
                      ("cells", np.int32)]}
    basins = abi.Basins(capacity=N, count=0, **{k: P(v) for k, v in basins_arrays.items()})
    o = abi.Outputs(**{k: P(v) for k, v in outs.items()}, basins=C.pointer(basins))
    stats = (abi.RoundStats * max(params.hydraulic_rounds, 1))()
    if refreshed is not None:
        rn2, vg2 = map(f32, refreshed)
        fed = abi.Inputs(None, None, None, P(rn2), P(vg2))
        st = lib().or_erode_stage_fed(C.byref(params), C.byref(inputs), C.byref(fed), C.byref(o))
    else:
        fn = lib().or_erode_stage if thermal else lib().or_hydraulic_apply
        st = fn(C.byref(params), C.byref(inputs), C.byref(o), C.cast(stats, C.c_void_p))
    assert st == 0, st
    outs["basins"] = {k: v[:basins.count].copy() for k, v in basins_arrays.items()}
    outs["basins"].update(count=basins.count, largest=basins.largest, largest_cells=basins.largest_cells,
                          largest_depth=basins.largest_depth, deepest=basins.deepest)
    outs["stats"] = [{f: getattr(s, f) for f, _ in abi.RoundStats._fields_} for s in stats]
    return outs


def sea_level_drained_cut(params, height, enclosed_max_share=0.00073, post_cut_outlet=True):
    """SeaLevelStage.apply's cut with the enclosure rule and the drowned basins' outlets:
    (shoreline, is_land, relative, land_cells, passes)."""
    H, W = params.height, params.width
    h = np.ascontiguousarray(height, dtype=np.float32).reshape(H, W)
    land = np.empty((H, W), np.uint8)
    rel = np.empty((H, W), np.float32)
    s, n, passes = C.c_float(), C.c_int32(), C.c_int32()
    st = lib().or_sea_level_drained_cut(C.byref(params), P(h), enclosed_max_share, int(post_cut_outlet), C.byref(s),
                                        P(land), P(rel), C.byref(n), C.byref(passes))
    assert st == 0, st
    return s.value, land, rel, n.value, passes.value


def flexure_deflection(params, load):
    """Isostasy.Flexure.deflectionMetres: (deflection in metres, rigidity D, restoring dRho g)."""
    H, W = params.height, params.width
    ld = np.ascontiguousarray(load, dtype=np.float32).reshape(H, W)
    out = np.empty((H, W), np.float32)
    d, r = C.c_double(), C.c_double()
    assert lib().or_flexure_deflection(C.byref(params), P(ld), P(out), C.byref(d), C.byref(r)) == 0
    return out, d.value, r.value


BELT_BOOKS = ("uplifted_cubic_meters", "cut_cubic_meters", "exported_to_sea_cubic_meters",
              "exported_to_land_cubic_meters", "shed_beside_cubic_meters")


def belt_replay(params, height, tectonic_km, wear_km, onset_myr_ago, window_myr, uplift=None, rain=None, cover=None,
                rock=None, provisional_sea_level=None, shield_cut=True, unresolved=None, rebound=True,
                history_cell_km=80.0):
    """BeltErosion.replay: (height after, eroded metres, dict of the BeltReplay figures)."""
    H, W = params.height, params.width

    def f32(a):
        return None if a is None else np.ascontiguousarray(a, dtype=np.float32).reshape(H, W)

    h = f32(height).copy()
    t, w, o, u, ra, cv, rk, ur = (f32(a) for a in (tectonic_km, wear_km, onset_myr_ago, uplift, rain, cover, rock,
                                                  unresolved))
    eroded = np.zeros((H, W), np.float32)
    counts = np.zeros(2, np.int32)
    books = np.zeros(5, np.float64)
    sea = params.sea_level if provisional_sea_level is None else provisional_sea_level
    assert lib().or_belt_replay(C.byref(params), P(h), P(t), P(w), P(o), float(window_myr), P(u), P(ra), P(cv), P(rk),
                                float(sea), int(bool(shield_cut)), P(ur), int(bool(rebound)),
                                float(history_cell_km), P(eroded), P(counts), P(books)) == 0
    out = {"rounds": int(counts[0]), "belt_cells": int(counts[1])}
    out.update({k: float(v) for k, v in zip(BELT_BOOKS, books)})
    return h, eroded, out


def gaussian_blur(field, sigma_across, sigma_down):
    """GaussianBlur.apply on a copy of `field`."""
    f = np.ascontiguousarray(field, dtype=np.float32).copy()
    H, W = f.shape
    lib().or_gaussian_blur(W, H, P(f), float(sigma_across), float(sigma_down))
    return f


def erode_stage_belts(params, height, window, uplift=None, rock=None, rain=None, veg=None, rebound=True,
                      history_cell_km=80.0, want=("receivers",)):
    """ErosionStage.apply with the belts' window: window = (tectonic_km, wear_km, onset_myr_ago,
    window_myr); the replay runs on the swept terrain with the opening weather (rain, veg) before
    round 0. Returns the outputs as erode_stage does (height plus `want`)."""
    H, W = params.height, params.width
    keep = []

    def f32(a):
        if a is None:
            return None
        a = np.ascontiguousarray(a, dtype=np.float32).reshape(H, W)
        keep.append(a)
        return a

    h, up, rk, rn, vg, t, w, o = map(f32, (height, uplift, rock, rain, veg) + tuple(window[:3]))
    inputs = abi.Inputs(P(h), P(up), P(rk), P(rn), P(vg))
    kinds = {"receivers": np.int32, "area": np.float32, "filled": np.float32, "relative": np.float32,
             "is_land": np.uint8, "order": np.int32, "donors": np.int32}
    outs = {"height": np.empty((H, W), np.float32)}
    for k in want:
        outs[k] = np.empty((H, W), kinds[k])
    o_ = abi.Outputs(**{k: P(v) for k, v in outs.items()})
    assert lib().or_erode_stage_belts(C.byref(params), C.byref(inputs), P(t), P(w), P(o), float(window[3]),
                                      int(bool(rebound)), float(history_cell_km), C.byref(o_)) == 0
    return outs


def flat_stencil(r):
    """FlatRouting.stencil: (east-west, north-south, diagonal) weights on cells r as tall as wide."""
    w = np.zeros(3, np.float64)
    lib().or_flat_stencil(float(r), P(w))
    return tuple(float(x) for x in w)


def facet_flip_delta(surface, mask, raised, seed, r):
    """Per cell of `mask`, the relative change of the routing surface at the `raised` cells (the flats'
    potentials; the rest is exact) that could change its facet receiver, to first order; +inf where
    none could."""
    rs = np.ascontiguousarray(surface, dtype=np.float64)
    H, W = rs.shape
    m = np.ascontiguousarray(mask, dtype=np.uint8)
    rz = np.ascontiguousarray(raised, dtype=np.uint8)
    out = np.empty((H, W), np.float64)
    lib().or_facet_flip_delta(W, H, P(rs), P(m), P(rz), int(seed), float(r), P(out))
    return out


def fan_hash(seed, index):
    """DeltaFan.hash(seed, index)."""
    return lib().or_fan_hash(int(seed), int(index))


def grow_fan_fixture(surface, apex, r, reach, out_x, out_y, hash_, grooved=False, wobble=0.30, bent=False):
    """DeltaFan.growFan on `surface` as DeltaOutlineTest drives it: every cell accepted, the distance bent
    by 1 - surface when `bent`, every level 0. Returns (sediment laid per cell, volume laid)."""
    s = np.ascontiguousarray(surface, dtype=np.float32)
    H, W = s.shape
    sed = np.empty((H, W), np.float32)
    laid = lib().or_grow_fan_fixture(W, H, int(apex), float(r), float(reach), float(out_x), float(out_y), int(hash_),
                                     int(bool(grooved)), float(wobble), P(s), int(bool(bent)), P(sed))
    return sed, laid
