// The Kotlin side of the drop-in: a HydraulicAccelerator seam beside the reference's
// ErosionAccelerator, and its binding to libcg_erosion.so through the Foreign Function & Memory API
// (java.lang.foreign, JDK 22+). Lives in the desktop module of a Cartogenesis checkout; it cannot
// be compiled in this repository (no JVM here), so it is kept as source.
package com.cartogenesis.desktop

import com.cartogenesis.worldgen.model.FloatField
import com.cartogenesis.worldgen.model.WorldGenConfig
import com.cartogenesis.worldgen.pipeline.BeltWindow
import com.cartogenesis.worldgen.pipeline.ErosionAccelerator
import com.cartogenesis.worldgen.pipeline.SeaLevelResult
import com.cartogenesis.worldgen.pipeline.ThermalLimits
import java.lang.foreign.Arena
import java.lang.foreign.FunctionDescriptor
import java.lang.foreign.Linker
import java.lang.foreign.MemoryLayout
import java.lang.foreign.MemorySegment
import java.lang.foreign.SymbolLookup
import java.lang.foreign.ValueLayout.ADDRESS
import java.lang.foreign.ValueLayout.JAVA_DOUBLE
import java.lang.foreign.ValueLayout.JAVA_FLOAT
import java.lang.foreign.ValueLayout.JAVA_INT
import java.lang.foreign.ValueLayout.JAVA_LONG
import java.lang.invoke.MethodHandle
import java.nio.file.Path
import kotlinx.coroutines.CancellationException

/** The whole erosion stage on a device: ErosionStage.apply's hydraulic rounds and relaxation. */
interface HydraulicAccelerator {
    val name: String

    /** Whether this accelerator runs the stage `config` asks for; the engine keeps its own rounds if not. */
    fun supports(config: WorldGenConfig): Boolean

    /**
     * The stage's result heights, or throws; there is no CPU fallback once this is selected.
     * `weather` is asked for the rounds' weather where HydraulicErosion.apply asks provisionalWeather
     * (HydraulicErosion.kt:655-661, 809-813): with climateFeed on, on the swept terrain before round 0
     * and again before round hydraulicRounds / 2, each time with the terrain as it stands and the
     * round about to cut; with it off it is never called and the rounds cut with no weather.
     * `window` (ErosionTectonics.window, or null) is the belts' history: the belts are replayed on the
     * swept terrain with the opening weather before round 0 (BeltErosion.replay, HydraulicErosion.kt:680-688).
     */
    fun erodeStage(config: WorldGenConfig, height: FloatField, upliftMmPerYear: FloatField?,
                   rockErodibility: FloatField?, window: BeltWindow?,
                   weather: ((FloatField, Int) -> Pair<FloatArray, FloatArray>)?): FloatField
}

/** cg_erosion.h's status codes. */
private fun check(status: Int, ctx: MemorySegment, lastError: MethodHandle) {
    if (status == 0) return
    val message = (lastError.invokeExact(ctx) as MemorySegment).reinterpret(512).getString(0)
    when (status) {
        1 -> throw CancellationException(message)
        else -> throw IllegalStateException("cg_erosion status $status: $message")
    }
}

class GbErosion(library: Path, device: Int = 0) : ErosionAccelerator, HydraulicAccelerator, AutoCloseable {
    private val linker = Linker.nativeLinker()
    private val lookup = SymbolLookup.libraryLookup(library, Arena.global())
    private fun fn(name: String, desc: FunctionDescriptor): MethodHandle =
        linker.downcallHandle(lookup.find(name).orElseThrow(), desc)

    private val create = fn("cg_create", FunctionDescriptor.of(JAVA_INT, ADDRESS, JAVA_INT))
    private val destroy = fn("cg_destroy", FunctionDescriptor.ofVoid(ADDRESS))
    private val lastError = fn("cg_last_error", FunctionDescriptor.of(ADDRESS, ADDRESS))
    private val defaults = fn("cg_default_params", FunctionDescriptor.ofVoid(ADDRESS, JAVA_INT, JAVA_INT, JAVA_LONG))
    private val limitsLayout = MemoryLayout.structLayout(JAVA_FLOAT, JAVA_FLOAT, JAVA_FLOAT)
    private val sweeps = fn("cg_thermal_sweeps", FunctionDescriptor.of(JAVA_INT, ADDRESS, JAVA_INT, JAVA_INT, ADDRESS,
        ADDRESS, limitsLayout, JAVA_INT, JAVA_FLOAT))
    private val stage = fn("cg_erode_stage", FunctionDescriptor.of(JAVA_INT, ADDRESS, ADDRESS, ADDRESS, ADDRESS, ADDRESS))
    private val begin = fn("cg_stage_begin", FunctionDescriptor.of(JAVA_INT, ADDRESS, ADDRESS, ADDRESS))
    private val rounds = fn("cg_erode_rounds", FunctionDescriptor.of(JAVA_INT, ADDRESS, JAVA_INT, JAVA_INT, ADDRESS, ADDRESS))
    private val current = fn("cg_stage_height", FunctionDescriptor.of(JAVA_INT, ADDRESS, ADDRESS))
    private val finish = fn("cg_stage_finish", FunctionDescriptor.of(JAVA_INT, ADDRESS, ADDRESS))
    private val replayBelts = fn("cg_stage_replay_belts", FunctionDescriptor.of(JAVA_INT, ADDRESS, ADDRESS, ADDRESS,
        JAVA_INT, JAVA_DOUBLE, ADDRESS, ADDRESS))
    private val routeCutFn = fn("cg_route_cut", FunctionDescriptor.of(JAVA_INT, ADDRESS, ADDRESS, ADDRESS, ADDRESS,
        JAVA_INT, ADDRESS, ADDRESS, ADDRESS, ADDRESS, ADDRESS))
    private val seaCut = fn("cg_sea_level_cut", FunctionDescriptor.of(JAVA_INT, ADDRESS, ADDRESS, ADDRESS, JAVA_DOUBLE,
        JAVA_INT, ADDRESS, ADDRESS, ADDRESS, ADDRESS, ADDRESS))
    private val ctx: MemorySegment

    override val name = "GB300 (cg_erosion)"

    init {
        Arena.ofConfined().use { a ->
            val out = a.allocate(ADDRESS)
            val st = create.invokeExact(out, device) as Int
            require(st == 0) { "cg_create failed with status $st" }
            ctx = out.get(ADDRESS, 0)
        }
    }

    /** ErosionAccelerator.erode: the sweeps alone, same contract as the GL accelerator. */
    override suspend fun erode(width: Int, height: Int, heights: FloatArray, limits: ThermalLimits, passes: Int,
                               rate: Float): FloatArray? = Arena.ofConfined().use { a ->
        val input = a.allocateFrom(JAVA_FLOAT, *heights)
        val output = a.allocate(JAVA_FLOAT, heights.size.toLong())
        val lim = a.allocate(limitsLayout)
        lim.set(JAVA_FLOAT, 0, limits.eastWest); lim.set(JAVA_FLOAT, 4, limits.northSouth)
        lim.set(JAVA_FLOAT, 8, limits.diagonal)
        check(sweeps.invokeExact(ctx, width, height, input, output, lim, passes, rate) as Int, ctx, lastError)
        output.toArray(JAVA_FLOAT)
    }

    // cg_profile: P0 without the outlet notch; P1 with it (HydraulicErosion.breach and the closing
    // breach); P2 with deposition and its lobed, outlined and graded deltas too; P3 is P2 with the
    // plate flexure (the reference's default). Any other mix of those switches is not a profile the
    // library runs: -1.
    private fun profileOf(config: WorldGenConfig): Int {
        val e = config.erosion
        val deltas = e.deltaLobe && e.deltaOutline && e.gradedAggradation
        val flexure = config.isostasy.enabled && config.isostasy.flexure
        return when {
            e.deposition && e.outletIncision && deltas -> if (flexure) 3 else 2
            flexure -> -1
            !e.deposition && !e.deltaLobe && e.outletIncision -> 1
            !e.deposition && !e.deltaLobe && !e.outletIncision -> 0
            else -> -1
        }
    }

    // The part of the stage the library does not run is the relief finer than the grid
    // (orogenicExcessKm), which the engine checks beside this. The flexure's transform lines must fit a
    // CTA: width <= 8192, height <= 4096.
    override fun supports(config: WorldGenConfig): Boolean {
        val profile = profileOf(config)
        return profile >= 0 && (profile < 3 || (config.width <= 8192 && config.height <= 4096))
    }

    override fun erodeStage(config: WorldGenConfig, height: FloatField, upliftMmPerYear: FloatField?,
                            rockErodibility: FloatField?, window: BeltWindow?,
                            weather: ((FloatField, Int) -> Pair<FloatArray, FloatArray>)?): FloatField =
        Arena.ofConfined().use { a ->
            // cg_erosion_params, 144 bytes (offsets as in cg_erosion.h, checked by the C tests).
            val p = a.allocate(144, 8)
            defaults.invokeExact(p, config.width, config.height, config.seed)
            p.set(JAVA_DOUBLE, 24, config.scale.worldWidthKm)
            p.set(JAVA_FLOAT, 32, config.scale.highestLandMetres)
            p.set(JAVA_FLOAT, 36, config.scale.deepestOceanMetres)
            p.set(JAVA_DOUBLE, 40, config.scale.yearsPerHydraulicRound)
            p.set(JAVA_INT, 48, if (config.erosion.enabled) 1 else 0)
            p.set(JAVA_FLOAT, 52, config.erosion.criticalFallMetresPerKm)
            p.set(JAVA_DOUBLE, 56, config.erosion.debrisTravelKm)
            p.set(JAVA_FLOAT, 64, config.erosion.rate)
            p.set(JAVA_INT, 68, config.erosion.hydraulicRounds)
            p.set(JAVA_FLOAT, 72, config.erosion.bedrockErodibilityPerYear)
            p.set(JAVA_INT, 76, if (config.facetRouting) 1 else 0)
            p.set(JAVA_INT, 80, if (config.flatPotential) 1 else 0)
            p.set(JAVA_FLOAT, 84, config.seaLevel)
            p.set(JAVA_FLOAT, 88, config.sea.lowstandMetres)
            p.set(JAVA_INT, 100, profileOf(config))
            val fed = config.erosion.climateFeed && weather != null
            p.set(JAVA_INT, 104, if (fed) 1 else 0)   // climate_feed
            val iso = config.isostasy   // IsostasyConfig, read by P3's flexure
            p.set(JAVA_FLOAT, 108, iso.mantleDensity)
            p.set(JAVA_FLOAT, 112, iso.deflectionFillDensity)
            p.set(JAVA_FLOAT, 116, iso.gravity)
            p.set(JAVA_FLOAT, 120, iso.continentalCrustDensity)
            p.set(JAVA_FLOAT, 124, iso.elasticThicknessKm)
            p.set(JAVA_FLOAT, 128, iso.youngsModulusGPa)
            p.set(JAVA_FLOAT, 132, iso.poissonRatio)
            fun field(f: FloatArray?) = if (f == null) MemorySegment.NULL else a.allocateFrom(JAVA_FLOAT, *f)
            val inputs = a.allocate(40, 8)
            inputs.set(ADDRESS, 0, field(height.data))
            inputs.set(ADDRESS, 8, field(upliftMmPerYear?.data))
            inputs.set(ADDRESS, 16, field(rockErodibility?.data))
            val result = a.allocate(JAVA_FLOAT, height.data.size.toLong())
            val outputs = a.allocate(80, 8)   // cg_outputs: height, then nine optional pointers
            outputs.set(ADDRESS, 0, result)
            if (!fed && window == null) {
                check(stage.invokeExact(ctx, p, inputs, outputs, MemorySegment.NULL) as Int, ctx, lastError)
            } else {
                // Stop where HydraulicErosion.apply asks the weather (climateFeed) or replays the belts.
                check(begin.invokeExact(ctx, p, inputs) as Int, ctx, lastError)
                val total = config.erosion.hydraulicRounds
                val half = if (total > 1) total / 2 else total
                fun askWeather(round: Int): MemorySegment {
                    if (!fed) return MemorySegment.NULL
                    check(current.invokeExact(ctx, result) as Int, ctx, lastError)
                    val (rain, cover) = weather!!(FloatField(config.width, config.height, result.toArray(JAVA_FLOAT)), round)
                    val w = a.allocate(16, 8)   // cg_weather
                    w.set(ADDRESS, 0, field(rain))
                    w.set(ADDRESS, 8, field(cover))
                    return w
                }
                val opening = askWeather(0)
                if (window != null) {
                    val win = a.allocate(32, 8)   // cg_belt_window
                    win.set(ADDRESS, 0, field(window.tectonicKm.data))
                    win.set(ADDRESS, 8, field(window.wearKm.data))
                    win.set(ADDRESS, 16, field(window.onsetMyrAgo.data))
                    win.set(JAVA_DOUBLE, 24, window.windowMyr)
                    val books = a.allocate(48, 8)   // cg_belt_books
                    check(replayBelts.invokeExact(ctx, win, opening, if (config.isostasy.enabled) 1 else 0,
                                                  config.tectonics.historyCellKm, MemorySegment.NULL, books) as Int,
                          ctx, lastError)
                }
                var done = 0
                for (end in (if (fed) listOf(half, total) else listOf(total)).distinct()) {
                    val w = if (done == 0) opening else askWeather(done)
                    check(rounds.invokeExact(ctx, done, end, w, MemorySegment.NULL) as Int, ctx, lastError)
                    done = end
                }
                check(finish.invokeExact(ctx, outputs) as Int, ctx, lastError)
            }
            FloatField(config.width, config.height, result.toArray(JAVA_FLOAT))
        }

    /**
     * SeaLevelStage.applyWithValleyBar's first three steps (SeaLevelStage.kt:243-270): the percentile cut,
     * the enclosure rule and the drowned basins' outlet passes, on the device. Returns the
     * SeaLevelResult the rest of the stage (DrownedValleys, LittoralGrading, the shelf) continues from.
     */
    fun drainedCut(config: WorldGenConfig, height: FloatField, enclosedSeaMaxShare: Double,
                   postCutOutlet: Boolean): SeaLevelResult = Arena.ofConfined().use { a ->
        val p = a.allocate(144, 8)
        defaults.invokeExact(p, config.width, config.height, config.seed)
        p.set(JAVA_DOUBLE, 24, config.scale.worldWidthKm)
        p.set(JAVA_FLOAT, 32, config.scale.highestLandMetres)
        p.set(JAVA_FLOAT, 36, config.scale.deepestOceanMetres)
        p.set(JAVA_INT, 76, if (config.facetRouting) 1 else 0)
        p.set(JAVA_INT, 80, if (config.flatPotential) 1 else 0)
        p.set(JAVA_FLOAT, 84, config.seaLevel)
        val cells = height.data.size.toLong()
        val h = a.allocateFrom(JAVA_FLOAT, *height.data)
        val shoreline = a.allocate(JAVA_FLOAT)
        val land = a.allocate(cells)
        val relative = a.allocate(JAVA_FLOAT, cells)
        val count = a.allocate(JAVA_INT)
        check(seaCut.invokeExact(ctx, p, h, enclosedSeaMaxShare, if (postCutOutlet) 1 else 0, shoreline, land,
                                 relative, count, MemorySegment.NULL) as Int, ctx, lastError)
        val isLand = BooleanArray(cells.toInt()) { land.get(java.lang.foreign.ValueLayout.JAVA_BYTE, it.toLong()) != 0.toByte() }
        SeaLevelResult(shoreline.get(JAVA_FLOAT, 0), isLand,
                       FloatField(config.width, config.height, relative.toArray(JAVA_FLOAT)), count.get(JAVA_INT, 0))
    }

    /** What [routeCut] hands back: FlowRouting's fill, receivers, accumulation and drainage order. */
    class RoutedCut(val filled: FloatField, val receivers: IntArray, val area: FloatField, val order: IntArray)

    /**
     * The routing the stages after the erosion run on their own cut (DrownedValleys.kt:411-421,
     * RiverStage.kt:228-240 and 306-308, GlaciationStage.kt:371-385), in one call: fillDepressions,
     * flowDirections, accumulate with `weights` (null: the `{ 1f }` weights) and drainageOrder.
     */
    fun routeCut(config: WorldGenConfig, isLand: BooleanArray, relative: FloatField, landCells: Int,
                 weights: FloatArray?): RoutedCut = Arena.ofConfined().use { a ->
        val p = a.allocate(144, 8)
        defaults.invokeExact(p, config.width, config.height, config.seed)
        p.set(JAVA_DOUBLE, 24, config.scale.worldWidthKm)
        p.set(JAVA_INT, 76, if (config.facetRouting) 1 else 0)
        p.set(JAVA_INT, 80, if (config.flatPotential) 1 else 0)
        val cells = relative.data.size.toLong()
        val land = a.allocate(cells)
        for (i in 0 until cells.toInt()) land.set(java.lang.foreign.ValueLayout.JAVA_BYTE, i.toLong(), if (isLand[i]) 1 else 0)
        val rel = a.allocateFrom(JAVA_FLOAT, *relative.data)
        val w = if (weights == null) MemorySegment.NULL else a.allocateFrom(JAVA_FLOAT, *weights)
        val filled = a.allocate(JAVA_FLOAT, cells)
        val receivers = a.allocate(JAVA_INT, cells)
        val area = a.allocate(JAVA_FLOAT, cells)
        val order = a.allocate(JAVA_INT, maxOf(landCells, 1).toLong())
        check(routeCutFn.invokeExact(ctx, p, land, rel, landCells, w, filled, receivers, area, order) as Int, ctx, lastError)
        RoutedCut(FloatField(config.width, config.height, filled.toArray(JAVA_FLOAT)), receivers.toArray(JAVA_INT),
                  FloatField(config.width, config.height, area.toArray(JAVA_FLOAT)),
                  order.toArray(JAVA_INT).copyOf(landCells))
    }

    override fun close() {
        destroy.invokeExact(ctx)
    }
}
