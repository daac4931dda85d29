// The Kotlin side of the drop-in: a HydraulicAccelerator seam beside the reference's
// ErosionAccelerator, and its binding to libcg_erosion.so through the Foreign Function & Memory API
// (java.lang.foreign, JDK 22+). Lives in the desktop module of a Cartogenesis checkout; it cannot
// be compiled in this repository (no JVM here), so it is kept as source.
package com.cartogenesis.desktop

import com.cartogenesis.worldgen.model.FloatField
import com.cartogenesis.worldgen.model.WorldGenConfig
import com.cartogenesis.worldgen.pipeline.ErosionAccelerator
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

    /** The stage's result heights, or throws; there is no CPU fallback once this is selected. */
    fun erodeStage(config: WorldGenConfig, height: FloatField, upliftMmPerYear: FloatField?,
                   rockErodibility: FloatField?, rainfallMm: FloatArray?, vegetation: FloatArray?): FloatField
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

    // cg_profile: P0 without the outlet notch, P1 with it (HydraulicErosion.breach and the closing
    // breach); deposition is P2, which the library does not run yet.
    private fun profileOf(config: WorldGenConfig): Int = when {
        config.erosion.deposition -> 2
        config.erosion.outletIncision -> 1
        else -> 0
    }

    override fun supports(config: WorldGenConfig): Boolean = profileOf(config) <= 1

    override fun erodeStage(config: WorldGenConfig, height: FloatField, upliftMmPerYear: FloatField?,
                            rockErodibility: FloatField?, rainfallMm: FloatArray?, vegetation: FloatArray?): FloatField =
        Arena.ofConfined().use { a ->
            // cg_erosion_params, 112 bytes (offsets as in cg_erosion.h, checked by the C tests).
            val p = a.allocate(112, 8)
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
            fun field(f: FloatArray?) = if (f == null) MemorySegment.NULL else a.allocateFrom(JAVA_FLOAT, *f)
            val inputs = a.allocate(40, 8)
            inputs.set(ADDRESS, 0, field(height.data))
            inputs.set(ADDRESS, 8, field(upliftMmPerYear?.data))
            inputs.set(ADDRESS, 16, field(rockErodibility?.data))
            inputs.set(ADDRESS, 24, field(rainfallMm))
            inputs.set(ADDRESS, 32, field(vegetation))
            val result = a.allocate(JAVA_FLOAT, height.data.size.toLong())
            val outputs = a.allocate(80, 8)   // cg_outputs: height, then nine optional pointers
            outputs.set(ADDRESS, 0, result)
            check(stage.invokeExact(ctx, p, inputs, outputs, MemorySegment.NULL) as Int, ctx, lastError)
            FloatField(config.width, config.height, result.toArray(JAVA_FLOAT))
        }

    override fun close() {
        destroy.invokeExact(ctx)
    }
}
