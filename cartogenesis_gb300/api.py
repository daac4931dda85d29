"""Python mirror of the reference's entry points for the erosion stage, on libcg_erosion.so.

Names, argument meanings and units follow the Kotlin (P = worldgen/src/commonMain/kotlin/com/
cartogenesis/worldgen/pipeline, MA = .../worldgen/math):
  GpuErosionAccelerator.erode  -> ErosionAccelerator.erode   (P/ErosionAccelerator.kt:38-45)
  ErosionStage.apply           -> ErosionStage.apply         (P/ErosionStage.kt:110-183)
  SeaLevelStage.percentile_cut -> SeaLevelStage.percentileCut (P/SeaLevelStage.kt:146-200)
  FlowRouting.*                -> FlowRouting.fillDepressions, flowDirections, drainageOrder,
                                  accumulate, spillways (P/FlowRouting.kt)
  HydraulicErosion.breach      -> HydraulicErosion.breach    (P/HydraulicErosion.kt:1931-2171)
  BeltErosion.replay           -> BeltErosion.replay         (P/BeltErosion.kt:96-425)
  GaussianBlur.apply           -> GaussianBlur.apply         (MA/GaussianBlur.kt:44-111)
Arrays are numpy, row-major [height, width]. Every call runs on the GPU; none falls back to a CPU.
"""
import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import abi
from .runtime import CgError, Context, load_library

P = abi.ptr

_default_ctx = None


def default_context():
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


@dataclass
class ThermalLimits:
    """ThermalLimits (P/ErosionAccelerator.kt:58-65), field units per neighbour kind."""
    east_west: float
    north_south: float
    diagonal: float

    def to_c(self):
        return abi.ThermalLimits(self.east_west, self.north_south, self.diagonal)


class ErosionConfig:
    """The WorldGenConfig fields the stage reads, as cg_erosion_params.

    ErosionConfig(width, height, seed, sea_level=0.70, hydraulic_rounds=12, ...): any field of
    cg_erosion_params may be given by name; the rest keep the reference defaults.
    """

    def __init__(self, width, height, seed=1, **fields):
        self.params = abi.ErosionParams()
        load_library().cg_default_params(C.byref(self.params), width, height, seed)
        for k, v in fields.items():
            if not hasattr(self.params, k):
                raise AttributeError(f"cg_erosion_params has no field {k}")
            setattr(self.params, k, v)

    def __getattr__(self, name):
        return getattr(self.__dict__["params"], name)

    @property
    def cells(self):
        return self.params.width * self.params.height

    def thermal_limits(self):
        lim = abi.ThermalLimits()
        sweeps = C.c_int32()
        st = load_library().cg_thermal_limits_for(C.byref(self.params), C.byref(lim), C.byref(sweeps))
        if st != abi.CG_OK:
            raise CgError(st, "cg_thermal_limits_for")
        return ThermalLimits(lim.east_west, lim.north_south, lim.diagonal), sweeps.value


def _f32(a, shape):
    if a is None:
        return None
    a = np.ascontiguousarray(a, dtype=np.float32)
    if a.size != shape[0] * shape[1]:
        raise ValueError(f"array of {a.size} cells for a {shape[1]} x {shape[0]} grid")
    return a.reshape(shape)


class GpuErosionAccelerator:
    """ErosionAccelerator on the GB300: the thermal sweeps alone (P/ErosionAccelerator.kt:38-45)."""

    name = "GB300 (sm_103a)"

    def __init__(self, ctx=None):
        self.ctx = ctx or default_context()

    def erode(self, width, height, heights, limits, passes, rate):
        """`passes` sweeps; `heights` is not modified and the result is a new array."""
        h = _f32(heights, (height, width))
        out = np.empty_like(h)
        with self.ctx.lock:
            self.ctx.check(self.ctx.lib.cg_thermal_sweeps(self.ctx.handle, width, height, P(h), P(out),
                                                          limits.to_c(), passes, rate))
        return out


class ErosionResult:
    """ErosionResult (P/ErosionStage.kt:11-22) plus the last round's routing the C ABI hands back."""

    def __init__(self, height, **extra):
        self.height = height
        self.swept_on_device = True
        self.__dict__.update(extra)


class ErosionStage:
    """ErosionStage.apply on the GPU (P/ErosionStage.kt:133-183 with HydraulicErosion.apply)."""

    WANT = ("receivers", "area", "filled", "relative", "is_land", "order", "basin_of_cell", "donors")
    KINDS = {"receivers": np.int32, "area": np.float32, "filled": np.float32, "relative": np.float32,
             "is_land": np.uint8, "order": np.int32, "basin_of_cell": np.int32, "donors": np.int32}

    @staticmethod
    def apply(config, height, uplift_mm_per_year=None, rock_erodibility=None, rainfall_mm=None,
              vegetation_density=None, want=WANT, ctx=None):
        ctx = ctx or default_context()
        H, W = config.params.height, config.params.width
        keep = [_f32(a, (H, W)) for a in (height, uplift_mm_per_year, rock_erodibility, rainfall_mm,
                                         vegetation_density)]
        inputs = abi.Inputs(*[P(a) for a in keep])
        outs = {"height": np.empty((H, W), np.float32)}
        for k in want:
            outs[k] = np.empty((H, W), ErosionStage.KINDS[k])
        N = W * H
        barrays = {k: np.empty(N, dt) for k, dt in [("spill", np.int32), ("entry", np.int32),
                                                    ("level", np.float32), ("floor", np.float32),
                                                    ("cells", np.int32)]}
        basins = abi.Basins(capacity=N, count=0, **{k: P(v) for k, v in barrays.items()})
        o = abi.Outputs(**{k: P(v) for k, v in outs.items()}, basins=C.pointer(basins))
        rounds = max(config.params.hydraulic_rounds, 1)
        stats = (abi.RoundStats * rounds)()
        with ctx.lock:
            ctx.check(ctx.lib.cg_erode_stage(ctx.handle, C.byref(config.params), C.byref(inputs), C.byref(o),
                                             C.cast(stats, C.c_void_p)))
        outs["basins"] = {k: v[:min(basins.count, N)].copy() for k, v in barrays.items()}
        outs["basins"].update(count=basins.count, largest=basins.largest, largest_cells=basins.largest_cells,
                              largest_depth=basins.largest_depth, deepest=basins.deepest)
        outs["stats"] = [{f: getattr(s, f) for f, _ in abi.RoundStats._fields_} for s in stats]
        return ErosionResult(**outs)


    @staticmethod
    def apply_batch(worlds, ctx=None):
        """Many worlds in one call (cg_erode_batch): `worlds` is a list of (config, height, uplift, rock)
        tuples (uplift and rock may be None), grids of any shapes. Returns one height array per world,
        each exactly what ErosionStage.apply gives for that world alone."""
        ctx = ctx or default_context()
        keep, descs, outs = [], (abi.World * len(worlds))(), []
        for i, (config, height, uplift, rock) in enumerate(worlds):
            H, W = config.params.height, config.params.width
            arrays = [_f32(a, (H, W)) for a in (height, uplift, rock)]
            out = np.empty((H, W), np.float32)
            keep.append(arrays)
            outs.append(out)
            descs[i].params = config.params
            descs[i].inputs = abi.Inputs(*[P(a) for a in arrays], None, None)
            descs[i].outputs = abi.Outputs(height=P(out))
        status = (C.c_int32 * max(len(worlds), 1))()
        with ctx.lock:
            st = ctx.lib.cg_erode_batch(ctx.handle, len(worlds), descs, C.cast(status, C.c_void_p))
            if st != abi.CG_OK:
                bad = [i for i in range(len(worlds)) if status[i] != abi.CG_OK]
                raise CgError(st, f"worlds {bad} failed: " + ctx.lib.cg_last_error(ctx.handle).decode(errors="replace"))
        return outs


class StageRounds:
    """The stage round by round with its world resident on the device (cg_stage_begin,
    cg_erode_rounds, cg_stage_height, cg_stage_finish): where HydraulicErosion.apply asks for the
    weather (P/HydraulicErosion.kt:655-661, 809-813) the caller reads the field and solves it."""

    def __init__(self, config, height, uplift_mm_per_year=None, rock_erodibility=None, rainfall_mm=None,
                 vegetation_density=None, ctx=None):
        self.ctx = ctx or default_context()
        self.config = config
        H, W = config.params.height, config.params.width
        self.shape = (H, W)
        self._keep = [_f32(a, (H, W)) for a in (height, uplift_mm_per_year, rock_erodibility, rainfall_mm,
                                               vegetation_density)]
        inputs = abi.Inputs(*[P(a) for a in self._keep])
        with self.ctx.lock:
            self.ctx.check(self.ctx.lib.cg_stage_begin(self.ctx.handle, C.byref(config.params), C.byref(inputs)))
        self.next_round = 0

    def rounds(self, end_round, rainfall_mm=None, vegetation_density=None, new_weather=False):
        """Rounds [next_round, end_round). With new_weather (or any weather field given) the weather is
        replaced from next_round on; a field left None is the default (rain 1, no cover)."""
        H, W = self.shape
        weather = None
        if new_weather or rainfall_mm is not None or vegetation_density is not None:
            self._weather = [_f32(a, (H, W)) for a in (rainfall_mm, vegetation_density)]
            weather = abi.Weather(*[P(a) for a in self._weather])
        first = self.next_round
        stats = (abi.RoundStats * max(end_round - first, 1))()
        with self.ctx.lock:
            self.ctx.check(self.ctx.lib.cg_erode_rounds(self.ctx.handle, first, end_round,
                                                        C.byref(weather) if weather is not None else None,
                                                        C.cast(stats, C.c_void_p)))
        self.next_round = end_round
        return [{f: getattr(s, f) for f, _ in abi.RoundStats._fields_} for s in stats[:max(end_round - first, 0)]]

    def replay_belts(self, window, rainfall_mm=None, vegetation_density=None, rebound=True, history_cell_km=80.0):
        """BeltErosion.replay on the resident swept terrain before round 0 (cg_stage_replay_belts), as
        HydraulicErosion.apply runs it (P/HydraulicErosion.kt:680-688): the stage's uplift, rock, sea
        level and shield_cut, the given opening weather (or, with neither field given, the weather the
        world was begun with), no sub-grid relief. Returns the BeltReplay."""
        H, W = self.shape
        fields = [_f32(a, (H, W)) for a in (window.tectonic_km, window.wear_km, window.onset_myr_ago)]
        win = abi.BeltWindow(*[P(a) for a in fields], float(window.window_myr))
        weather = None
        if rainfall_mm is not None or vegetation_density is not None:
            wk = [_f32(a, (H, W)) for a in (rainfall_mm, vegetation_density)]
            weather = abi.Weather(*[P(a) for a in wk])
        eroded = np.empty((H, W), np.float32)
        books = abi.BeltBooks()
        with self.ctx.lock:
            self.ctx.check(self.ctx.lib.cg_stage_replay_belts(self.ctx.handle, C.byref(win),
                                                              C.byref(weather) if weather is not None else None,
                                                              int(bool(rebound)), float(history_cell_km), P(eroded),
                                                              C.byref(books)))
        return BeltReplay(books.rounds, books.belt_cells, books.uplifted_cubic_meters, books.cut_cubic_meters,
                          books.exported_to_sea_cubic_meters, books.exported_to_land_cubic_meters,
                          books.shed_beside_cubic_meters, eroded)

    def height(self):
        out = np.empty(self.shape, np.float32)
        with self.ctx.lock:
            self.ctx.check(self.ctx.lib.cg_stage_height(self.ctx.handle, P(out)))
        return out

    def finish(self, want=("receivers",)):
        H, W = self.shape
        outs = {"height": np.empty((H, W), np.float32)}
        for k in want:
            outs[k] = np.empty((H, W), ErosionStage.KINDS[k])
        o = abi.Outputs(**{k: P(v) for k, v in outs.items()})
        with self.ctx.lock:
            self.ctx.check(self.ctx.lib.cg_stage_finish(self.ctx.handle, C.byref(o)))
        return ErosionResult(**outs)

    @staticmethod
    def apply_fed(config, height, provisional_weather, uplift_mm_per_year=None, rock_erodibility=None,
                  want=("receivers",), ctx=None):
        """ErosionStage.apply with ErosionConfig.climateFeed: provisional_weather(field, round) returns the
        (rainfall_mm, vegetation_density) solved on `field`, asked on the swept terrain (round 0) and at
        round hydraulic_rounds / 2, as HydraulicErosion.apply asks provisionalWeather."""
        run = StageRounds(config, height, uplift_mm_per_year, rock_erodibility, ctx=ctx)
        R = config.params.hydraulic_rounds
        half = R // 2 if R > 1 else R
        rain, veg = provisional_weather(run.height(), 0)
        run.rounds(half, rain, veg, new_weather=True)
        if half < R:
            rain, veg = provisional_weather(run.height(), half)
            run.rounds(R, rain, veg, new_weather=True)
        return run.finish(want)


class SeaLevelStage:
    @staticmethod
    def drained_cut(config, height, enclosed_sea_max_share=0.00073, post_cut_outlet=True, ctx=None):
        """SeaLevelStage.apply's cut with its enclosure rule and the drowned basins' outlets
        (P/SeaLevelStage.kt:243-270, 371-437, 478-560): (shoreline, is_land, relative, land_cells, passes)."""
        ctx = ctx or default_context()
        H, W = config.params.height, config.params.width
        h = _f32(height, (H, W))
        land = np.empty((H, W), np.uint8)
        rel = np.empty((H, W), np.float32)
        s, n, passes = C.c_float(), C.c_int32(), C.c_int32()
        with ctx.lock:
            ctx.check(ctx.lib.cg_sea_level_cut(ctx.handle, C.byref(config.params), P(h), enclosed_sea_max_share,
                                               int(post_cut_outlet), C.byref(s), P(land), P(rel), C.byref(n),
                                               C.byref(passes)))
        return s.value, land, rel, n.value, passes.value

    @staticmethod
    def percentile_cut(height, sea_level_fraction, lowstand_share_of_field=0.0, highest_land_metres=6000.0,
                       deepest_ocean_metres=10000.0, ctx=None):
        """SeaLevelStage.percentileCut: (shoreline, is_land, relative, land_cells)."""
        ctx = ctx or default_context()
        h = np.ascontiguousarray(height, dtype=np.float32)
        H, W = h.shape
        is_land = np.empty((H, W), np.uint8)
        rel = np.empty((H, W), np.float32)
        s = C.c_float()
        n = C.c_int32()
        with ctx.lock:
            ctx.check(ctx.lib.cg_percentile_cut(ctx.handle, W, H, P(h), sea_level_fraction, highest_land_metres,
                                                deepest_ocean_metres, lowstand_share_of_field, C.byref(s),
                                                P(is_land), P(rel), C.byref(n)))
        return s.value, is_land, rel, n.value


def sequential_sum(values, mask=None, mode=0, ctx=None):
    """The reference's `var s = 0.0; for (c in cells) s += v[c]` over the cells where mask is set (all when
    mask is None), v = values (mode 0) or 1 - 0.5 values (mode 1), bit for bit, on the device. Returns
    (sum, counts): blocks of 8192 values taken whole, pieces of 1024 reduced, pieces added one by one."""
    ctx = ctx or default_context()
    x = np.ascontiguousarray(values, dtype=np.float32).ravel()
    m = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint8).ravel()
    if m is not None and m.size != x.size:
        raise ValueError("mask and values differ in size")
    s = C.c_double()
    counts = np.zeros(3, np.int64)
    with ctx.lock:
        ctx.check(ctx.lib.cg_sequential_sum(ctx.handle, P(x) if x.size else None, None if m is None else P(m), mode,
                                            x.size, C.byref(s), P(counts)))
    return s.value, counts


class Isostasy:
    class Flexure:
        """Isostasy.Flexure (P/Isostasy.kt:277-411): the plate's bend under a load, on the device."""

        def __init__(self, config, ctx=None):
            self.config = config
            self.ctx = ctx or default_context()
            self.rigidity = None
            self.restoring = None

        def deflection_metres(self, load_pascals):
            """deflectionMetres(loadPascals, deflection): the bend in metres, positive down."""
            H, W = self.config.params.height, self.config.params.width
            ld = _f32(load_pascals, (H, W))
            out = np.empty((H, W), np.float32)
            d, r = C.c_double(), C.c_double()
            with self.ctx.lock:
                self.ctx.check(self.ctx.lib.cg_flexure_deflection(self.ctx.handle, C.byref(self.config.params), P(ld),
                                                                  P(out), C.byref(d), C.byref(r)))
            self.rigidity, self.restoring = d.value, r.value
            return out


def sequential_sum_f64(terms, ctx=None):
    """`var s = 0.0; for (v in terms) s += v` over double terms in the order given, bit for bit, on the
    device (the belts' replay keeps its books with it)."""
    ctx = ctx or default_context()
    x = np.ascontiguousarray(terms, dtype=np.float64).ravel()
    s = C.c_double()
    with ctx.lock:
        ctx.check(ctx.lib.cg_sequential_sum_f64(ctx.handle, P(x) if x.size else None, x.size, C.byref(s)))
    return s.value


class GaussianBlur:
    """GaussianBlur (MA/GaussianBlur.kt): a Gaussian of a spread on the ground, x wrapping, y clamped."""

    @staticmethod
    def apply(field, sigma_across_cells, sigma_down_cells, ctx=None):
        """Blurs `field` (float32 [H, W]) in place, as GaussianBlur.apply does."""
        ctx = ctx or default_context()
        f = np.ascontiguousarray(field, dtype=np.float32).copy()
        H, W = f.shape
        with ctx.lock:
            ctx.check(ctx.lib.cg_gaussian_blur(ctx.handle, W, H, P(f), float(sigma_across_cells),
                                               float(sigma_down_cells)))
        field[...] = f
        return field


@dataclass
class BeltWindow:
    """BeltWindow (P/BeltErosion.kt:19-24): per cell, km thickened and worn over the window and when the
    thickening began (Myr ago, negative where none did); the window's length in Myr."""
    tectonic_km: np.ndarray
    wear_km: np.ndarray
    onset_myr_ago: np.ndarray
    window_myr: float


@dataclass
class BeltReplay:
    """BeltReplay (P/BeltErosion.kt:35-47)."""
    rounds: int
    belt_cells: int
    uplifted_cubic_meters: float
    cut_cubic_meters: float
    exported_to_sea_cubic_meters: float
    exported_to_land_cubic_meters: float
    shed_beside_cubic_meters: float
    eroded_meters: np.ndarray


class BeltErosion:
    @staticmethod
    def replay(config, surface, window, present_uplift_mm_per_year=None, rainfall_mm=None, cover_density=None,
               rock_erodibility=None, provisional_sea_level=None, shield_cut=True, unresolved_relief=None,
               rebound=True, history_cell_km=80.0, ctx=None):
        """BeltErosion.replay (P/BeltErosion.kt:96-425) on the device: `surface` (the height field,
        [H, W]) is replayed in place, as the reference's array is. `rebound` is IsostasyConfig.enabled,
        `history_cell_km` TectonicsConfig.historyCellKm; the provisional sea level defaults to the
        config's sea_level. Returns the BeltReplay, its eroded_meters a new [H, W] array."""
        ctx = ctx or default_context()
        p = config.params
        H, W = p.height, p.width
        h = _f32(surface, (H, W)).copy()
        fields = [_f32(a, (H, W)) if a is not None else None
                  for a in (window.tectonic_km, window.wear_km, window.onset_myr_ago, present_uplift_mm_per_year,
                            rainfall_mm, cover_density, rock_erodibility, unresolved_relief)]
        tect, wear, onset, upl, rain, cover, rock, unres = fields
        win = abi.BeltWindow(P(tect), P(wear), P(onset), float(window.window_myr))
        sea = p.sea_level if provisional_sea_level is None else provisional_sea_level
        ins = abi.BeltInputs(P(upl), P(rain), P(cover), P(rock), P(unres), float(sea), int(bool(shield_cut)),
                             int(bool(rebound)), float(history_cell_km))
        eroded = np.empty((H, W), np.float32)
        books = abi.BeltBooks()
        with ctx.lock:
            ctx.check(ctx.lib.cg_belt_replay(ctx.handle, C.byref(p), P(h), C.byref(win), C.byref(ins), P(eroded),
                                             C.byref(books)))
        surface[...] = h
        return BeltReplay(books.rounds, books.belt_cells, books.uplifted_cubic_meters, books.cut_cubic_meters,
                          books.exported_to_sea_cubic_meters, books.exported_to_land_cubic_meters,
                          books.shed_beside_cubic_meters, eroded)


class FlowRouting:
    @staticmethod
    def route_cut(config, is_land, relative, land_cells, weights=None, ctx=None):
        """fillDepressions, flowDirections, accumulate (weights, or all ones) and drainageOrder of one
        cut in a single device call, as DrownedValleys, RiverStage and GlaciationStage run them on their
        own cut (cg_route_cut). Returns (filled, receivers, area, order)."""
        ctx = ctx or default_context()
        p = config.params
        H, W = p.height, p.width
        il = np.ascontiguousarray(is_land, dtype=np.uint8).reshape(H, W)
        rel = _f32(relative, (H, W))
        w = _f32(weights, (H, W))
        filled = np.empty((H, W), np.float32)
        recv = np.empty((H, W), np.int32)
        area = np.empty((H, W), np.float32)
        order = np.empty(max(int(land_cells), 1), np.int32)
        with ctx.lock:
            ctx.check(ctx.lib.cg_route_cut(ctx.handle, C.byref(p), P(il), P(rel), int(land_cells), P(w), P(filled),
                                           P(recv), P(area), P(order)))
        return filled, recv, area, order[:int(land_cells)]

    @staticmethod
    def fill_depressions(is_land, elevation, ctx=None, with_ties=False):
        ctx = ctx or default_context()
        rel = np.ascontiguousarray(elevation, dtype=np.float32)
        H, W = rel.shape
        il = np.ascontiguousarray(is_land, dtype=np.uint8)
        out = np.empty_like(rel)
        ties, unresolved = C.c_int64(), C.c_int64()
        with ctx.lock:
            ctx.check(ctx.lib.cg_fill_depressions(ctx.handle, W, H, P(il), P(rel), P(out), C.byref(ties),
                                                  C.byref(unresolved)))
        return (out, ties.value, unresolved.value) if with_ties else out

    @staticmethod
    def flow_directions(is_land, elevation, filled, seed, cell_height_in_cell_widths, smooth_lattice_columns,
                        by_facet=True, over_potential=True, want_surface=False, ctx=None):
        ctx = ctx or default_context()
        rel = np.ascontiguousarray(elevation, dtype=np.float32)
        H, W = rel.shape
        il = np.ascontiguousarray(is_land, dtype=np.uint8)
        fil = np.ascontiguousarray(filled, dtype=np.float32)
        rec = np.empty((H, W), np.int32)
        surf = np.empty((H, W), np.float64) if want_surface else None
        counts = np.zeros(3, np.int32)
        with ctx.lock:
            ctx.check(ctx.lib.cg_flow_directions(ctx.handle, W, H, P(il), P(rel), P(fil), seed,
                                                 cell_height_in_cell_widths, smooth_lattice_columns, int(by_facet),
                                                 int(over_potential), P(rec), P(surf), P(counts)))
        return (rec, surf, counts) if want_surface else (rec, counts)

    @staticmethod
    def drainage_order(is_land, receivers, land_cells, ctx=None):
        ctx = ctx or default_context()
        rec = np.ascontiguousarray(receivers, dtype=np.int32)
        H, W = rec.shape
        il = np.ascontiguousarray(is_land, dtype=np.uint8)
        order = np.empty(max(land_cells, 1), np.int32)
        with ctx.lock:
            ctx.check(ctx.lib.cg_drainage_order(ctx.handle, W, H, P(il), P(rec), land_cells, P(order)))
        return order[:land_cells]

    @staticmethod
    def accumulate(is_land, receivers, land_cells, weights, ctx=None):
        ctx = ctx or default_context()
        rec = np.ascontiguousarray(receivers, dtype=np.int32)
        H, W = rec.shape
        il = np.ascontiguousarray(is_land, dtype=np.uint8)
        w = np.ascontiguousarray(weights, dtype=np.float32)
        area = np.empty((H, W), np.float32)
        with ctx.lock:
            ctx.check(ctx.lib.cg_accumulate(ctx.handle, W, H, P(il), P(rec), land_cells, P(w), P(area)))
        return area

    @staticmethod
    def spillways(is_land, elevation, filled, receivers, pond_depth, ctx=None):
        ctx = ctx or default_context()
        rel = np.ascontiguousarray(elevation, dtype=np.float32)
        H, W = rel.shape
        N = W * H
        il = np.ascontiguousarray(is_land, dtype=np.uint8)
        fil = np.ascontiguousarray(filled, dtype=np.float32)
        rec = np.ascontiguousarray(receivers, dtype=np.int32)
        labels = np.empty((H, W), np.int32)
        arrays = {k: np.empty(N, dt) for k, dt in [("spill", np.int32), ("entry", np.int32),
                                                   ("level", np.float32), ("floor", np.float32),
                                                   ("cells", np.int32)]}
        b = abi.Basins(capacity=N, count=0, **{k: P(v) for k, v in arrays.items()})
        with ctx.lock:
            ctx.check(ctx.lib.cg_spillways(ctx.handle, W, H, P(il), P(rel), P(fil), P(rec), pond_depth, P(labels),
                                           C.byref(b)))
        out = {k: v[:b.count].copy() for k, v in arrays.items()}
        out.update(count=b.count, largest=b.largest, largest_cells=b.largest_cells, largest_depth=b.largest_depth,
                   deepest=b.deepest, labels=labels)
        return out


class HydraulicErosion:
    @staticmethod
    def breach(config, is_land, relative, ground, directions, area, land_cells, land_range, surface, ctx=None):
        """HydraulicErosion.breach (belowSea false, nothing carried) over the basins of this routing.
        `relative`, `ground` and `surface` (float32, C-contiguous) are cut in place, as the reference
        cuts its arrays; returns the number of cells the notch lowered."""
        ctx = ctx or default_context()
        H, W = config.params.height, config.params.width
        for a in (relative, ground, surface):
            if a.dtype != np.float32 or not a.flags.c_contiguous or a.size != W * H:
                raise ValueError("relative, ground and surface must be C-contiguous float32 grids")
        il = np.ascontiguousarray(is_land, dtype=np.uint8)
        rec = np.ascontiguousarray(directions, dtype=np.int32)
        ar = np.ascontiguousarray(area, dtype=np.float32)
        cells = C.c_int32()
        with ctx.lock:
            ctx.check(ctx.lib.cg_breach(ctx.handle, C.byref(config.params), P(il), P(relative), P(ground), P(rec),
                                        P(ar), land_cells, land_range, P(surface), C.byref(cells)))
        return cells.value
