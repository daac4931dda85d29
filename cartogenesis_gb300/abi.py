"""ctypes mirror of include/cg_erosion.h.

The structs below follow the header field by field; ctypes lays them out with the C compiler's
alignment rules, so a change to one side must be made to the other.
"""
import ctypes as C

CG_ABI_VERSION = 2

CG_OK, CG_CANCELLED, CG_TIMEOUT, CG_BAD_ARG, CG_OOM, CG_CUDA, CG_UNSUPPORTED, CG_INEXACT = range(8)
STATUS_NAMES = {
    CG_OK: "OK", CG_CANCELLED: "CANCELLED", CG_TIMEOUT: "TIMEOUT", CG_BAD_ARG: "BAD_ARG",
    CG_OOM: "OOM", CG_CUDA: "CUDA", CG_UNSUPPORTED: "UNSUPPORTED", CG_INEXACT: "INEXACT",
}
CG_MODE_REF32 = 0
CG_PROFILE_P0, CG_PROFILE_P1, CG_PROFILE_P2, CG_PROFILE_P3 = 0, 1, 2, 3


class ThermalLimits(C.Structure):
    _fields_ = [("east_west", C.c_float), ("north_south", C.c_float), ("diagonal", C.c_float)]


class ErosionParams(C.Structure):
    _fields_ = [
        ("abi_version", C.c_uint32),
        ("width", C.c_int32),
        ("height", C.c_int32),
        ("mode", C.c_int32),
        ("seed", C.c_int64),
        ("world_width_km", C.c_double),
        ("highest_land_metres", C.c_float),
        ("deepest_ocean_metres", C.c_float),
        ("years_per_hydraulic_round", C.c_double),
        ("enabled", C.c_int32),
        ("critical_fall_metres_per_km", C.c_float),
        ("debris_travel_km", C.c_double),
        ("rate", C.c_float),
        ("hydraulic_rounds", C.c_int32),
        ("bedrock_erodibility_per_year", C.c_float),
        ("facet_routing", C.c_int32),
        ("flat_potential", C.c_int32),
        ("sea_level", C.c_float),
        ("lowstand_metres", C.c_float),
        ("receiver_clamp", C.c_int32),
        ("shield_cut", C.c_int32),
        ("profile", C.c_int32),
        ("climate_feed", C.c_int32),
        ("mantle_density", C.c_float),
        ("deflection_fill_density", C.c_float),
        ("gravity", C.c_float),
        ("continental_crust_density", C.c_float),
        ("elastic_thickness_km", C.c_float),
        ("youngs_modulus_gpa", C.c_float),
        ("poisson_ratio", C.c_float),
        ("reserved", C.c_int32),
    ]


class Weather(C.Structure):
    _fields_ = [("rainfall_mm", C.c_void_p), ("vegetation_density", C.c_void_p)]


class Inputs(C.Structure):
    _fields_ = [
        ("height", C.c_void_p),
        ("uplift_mm_per_year", C.c_void_p),
        ("rock_erodibility", C.c_void_p),
        ("rainfall_mm", C.c_void_p),
        ("vegetation_density", C.c_void_p),
    ]


class Basins(C.Structure):
    _fields_ = [
        ("capacity", C.c_int32),
        ("count", C.c_int32),
        ("spill", C.c_void_p),
        ("entry", C.c_void_p),
        ("level", C.c_void_p),
        ("floor", C.c_void_p),
        ("cells", C.c_void_p),
        ("largest", C.c_int32),
        ("largest_cells", C.c_int32),
        ("largest_depth", C.c_float),
        ("deepest", C.c_float),
    ]


class Outputs(C.Structure):
    _fields_ = [
        ("height", C.c_void_p),
        ("receivers", C.c_void_p),
        ("area", C.c_void_p),
        ("filled", C.c_void_p),
        ("relative", C.c_void_p),
        ("is_land", C.c_void_p),
        ("order", C.c_void_p),
        ("basin_of_cell", C.c_void_p),
        ("donors", C.c_void_p),
        ("basins", C.POINTER(Basins)),
    ]


class RoundStats(C.Structure):
    _fields_ = [
        ("round", C.c_int32),
        ("land_cells", C.c_int32),
        ("shoreline", C.c_float),
        ("basins", C.c_int32),
        ("flats", C.c_int32),
        ("flats_kept", C.c_int32),
        ("raised_cells", C.c_int32),
        ("levels", C.c_int32),
        ("fill_ties", C.c_int64),
        ("fill_unresolved", C.c_int64),
        ("kernel_launches", C.c_int64),
        ("ms_total", C.c_double),
        ("ms_cut", C.c_double),
        ("ms_fill", C.c_double),
        ("ms_route", C.c_double),
        ("ms_tree", C.c_double),
        ("ms_incise", C.c_double),
        ("ms_relax", C.c_double),
        ("ms_deposit", C.c_double),
        ("deposit_replayed", C.c_int32),
        ("deposit_redone", C.c_int32),
        ("deposit_refitted", C.c_int32),
        ("deposit_waves", C.c_int32),
        ("ms_deposit_walks", C.c_double),
        ("ms_deposit_schedule", C.c_double),
        ("ms_deposit_lakes", C.c_double),
        ("ms_deposit_seas", C.c_double),
        ("ms_deposit_repairs", C.c_double),
        ("ms_flexure", C.c_double),
    ]


class World(C.Structure):
    """cg_world: one world of a batch."""
    _fields_ = [
        ("params", ErosionParams),
        ("inputs", Inputs),
        ("outputs", Outputs),
    ]


class BeltWindow(C.Structure):
    """cg_belt_window: BeltWindow, the belts' history over the exposure window."""
    _fields_ = [
        ("tectonic_km", C.c_void_p),
        ("wear_km", C.c_void_p),
        ("onset_myr_ago", C.c_void_p),
        ("window_myr", C.c_double),
    ]


class BeltInputs(C.Structure):
    """cg_belt_inputs: the rest of BeltErosion.replay's arguments."""
    _fields_ = [
        ("uplift_mm_per_year", C.c_void_p),
        ("rainfall_mm", C.c_void_p),
        ("cover_density", C.c_void_p),
        ("rock_erodibility", C.c_void_p),
        ("unresolved_relief", C.c_void_p),
        ("provisional_sea_level", C.c_float),
        ("shield_cut", C.c_int32),
        ("rebound", C.c_int32),
        ("history_cell_km", C.c_double),
    ]


class BeltBooks(C.Structure):
    """cg_belt_books: BeltReplay's figures."""
    _fields_ = [
        ("rounds", C.c_int32),
        ("belt_cells", C.c_int32),
        ("uplifted_cubic_meters", C.c_double),
        ("cut_cubic_meters", C.c_double),
        ("exported_to_sea_cubic_meters", C.c_double),
        ("exported_to_land_cubic_meters", C.c_double),
        ("shed_beside_cubic_meters", C.c_double),
    ]


def ptr(a):
    """Address of a numpy array's data, or None."""
    return None if a is None else a.ctypes.data
