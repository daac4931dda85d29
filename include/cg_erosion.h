/*
 * cg_erosion.h - C ABI of the GB300-native erosion stage.
 *
 * This library replaces Cartogenesis's per-round erosion stage on one GPU:
 *   ErosionStage.apply -> HydraulicErosion.apply, with the thermal relaxation between rounds
 *   (worldgen/src/commonMain/kotlin/com/cartogenesis/worldgen/pipeline/ErosionStage.kt:133-183,
 *    .../pipeline/HydraulicErosion.kt:596-1506).
 * The reference has exactly one device seam, ErosionAccelerator.erode
 * (.../pipeline/ErosionAccelerator.kt:15-45); cg_thermal_sweeps keeps its contract. The hydraulic
 * rounds have no seam in the reference, so cg_erode_stage is the new one a Kotlin
 * `HydraulicAccelerator` binds through FFM or JNI in place of HydraulicErosion.apply.
 *
 * Conventions
 *  - Every function returns a cg_status; no exception crosses the ABI.
 *  - Buffers are caller-owned HOST memory unless a name says `_dev`. Inputs are never written.
 *  - Grids are row-major, cell = row * width + column; x wraps east-west, y stops at the poles
 *    (FloatField, .../model/FloatField.kt:7).
 *  - Heights are in the height field's own 0..1 units; relative elevations are shoreline-relative,
 *    1 = WorldScale.highestLandMetres above, -1 = deepestOceanMetres below.
 *  - One context per thread, or serialise calls on a context. cg_cancel may be called from any
 *    thread or a signal handler.
 *  - No CPU fallback: if the device cannot run the job the call fails with a status.
 */
#ifndef CG_EROSION_H
#define CG_EROSION_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CG_ABI_VERSION 2u

typedef enum cg_status {
    CG_OK = 0,
    CG_CANCELLED = 1,   /* cg_cancel was seen between phases; outputs are not written */
    CG_TIMEOUT = 2,     /* a bounded device-side wait ran out; the context stays usable */
    CG_BAD_ARG = 3,     /* a size, pointer or parameter failed validation */
    CG_OOM = 4,         /* device or pinned-host allocation failed */
    CG_CUDA = 5,        /* a CUDA call failed; cg_last_error says which */
    CG_UNSUPPORTED = 6, /* a switch the library does not implement */
    CG_INEXACT = 7      /* a result could not be made the reference's exactly (a fill tie left
                           unordered by the repairs' guard); outputs are not written */
} cg_status;

/* Parity mode. REF32 is the reference's own arithmetic (FP32 field, FP64 where Kotlin promotes). */
typedef enum cg_mode { CG_MODE_REF32 = 0 } cg_mode;

/*
 * Round-tail profile. P0: uplift, percentile cut, weights, fill, routing, accumulation, incision
 * and relaxation (climateFeed, deposition, outletIncision, flexure and the belt replay off).
 * P1: P0 with ErosionConfig.outletIncision: each round's notch before the incision and the closing
 * breach before the last relaxation (HydraulicErosion.kt:1002-1028, 1404-1442); the routing outputs
 * are then the closing pass's, as its notch left them. P0 and P1 have ErosionConfig.deltaLobe off
 * (the closing mouths pass belongs to P2). P2: P1 with ErosionConfig.deposition, deltaLobe,
 * deltaOutline and gradedAggradation (the reference's default round tail): each round's deposition
 * walk with its sea lobes and lake fans, settle and the closing mouths pass (HydraulicErosion.kt:
 * 1068-1349, 1351-1364, 1451-1462, 1804-1892; DeltaFan.kt). P3: P2 with IsostasyConfig.flexure (the
 * reference's default): at the top of every round, after the uplift, the plate bends under the load
 * the rounds have put on it, a mirrored 2D FFT low-pass of the column change (Isostasy.Flexure,
 * Isostasy.kt:277-411; HydraulicErosion.kt:707-725, 856-880). P3 needs width <= 8192 and
 * height <= 4096 (a transform line in one CTA's shared memory).
 */
typedef enum cg_profile { CG_PROFILE_P0 = 0, CG_PROFILE_P1 = 1, CG_PROFILE_P2 = 2, CG_PROFILE_P3 = 3 } cg_profile;

/* ThermalLimits (.../pipeline/ErosionAccelerator.kt:58-65): steepest drop per neighbour kind. */
typedef struct cg_thermal_limits {
    float east_west;
    float north_south;
    float diagonal;
} cg_thermal_limits;

/*
 * The WorldGenConfig fields the stage reads (.../model/WorldGenConfig.kt: WorldScale 32-304,
 * ErosionConfig 2068-2496, WorldGenConfig 3236-3384, SeaConfig.lowstandMetres 1580), plus the
 * test-only switches ErodeBlocking exposes (.../jvmMain/.../pipeline/ErodeBlocking.kt:61-104).
 * cg_default_params fills the reference defaults.
 */
typedef struct cg_erosion_params {
    uint32_t abi_version;                 /* CG_ABI_VERSION */
    int32_t  width;                       /* cells across, a power of two */
    int32_t  height;                      /* cells down, a power of two */
    int32_t  mode;                        /* cg_mode */
    int64_t  seed;                        /* WorldGenConfig.seed */
    /* WorldScale */
    double   world_width_km;              /* 40075 */
    float    highest_land_metres;         /* 6000 */
    float    deepest_ocean_metres;        /* 10000 */
    double   years_per_hydraulic_round;   /* 336476.4 */
    /* ErosionConfig */
    int32_t  enabled;                     /* 1 */
    float    critical_fall_metres_per_km; /* 60 */
    double   debris_travel_km;            /* 1875 */
    float    rate;                        /* 0.25 */
    int32_t  hydraulic_rounds;            /* 12 */
    float    bedrock_erodibility_per_year;/* 1e-6 */
    /* WorldGenConfig top level */
    int32_t  facet_routing;               /* 1 */
    int32_t  flat_potential;              /* 1 */
    float    sea_level;                   /* 0.71 */
    float    lowstand_metres;             /* SeaConfig.lowstandMetres, 120 */
    /* Test switches, never set by a production caller */
    int32_t  receiver_clamp;              /* 1: HydraulicErosion.incise onlyAboveBase */
    int32_t  shield_cut;                  /* 1: incision takes the cover's factor */
    int32_t  profile;                     /* cg_profile */
    /* ErosionConfig.climateFeed: the rounds cut with the provisional weather, solved by the caller on
       the swept terrain and again at round hydraulic_rounds / 2 (HydraulicErosion.kt:655-661,
       809-813). The weather solve is the caller's (a climate stage, not this path), so a stage with
       it set runs through cg_stage_begin / cg_erode_rounds, which stop where the weather is asked;
       cg_erode_stage refuses it. 0 in the P0-P2 profiles. */
    int32_t  climate_feed;
    /* IsostasyConfig, the plate flexure of profile P3 (Isostasy.Flexure, .../pipeline/Isostasy.kt:
       277-411; M:WorldGenConfig.kt:1348-1476) */
    float    mantle_density;              /* 3300 */
    float    deflection_fill_density;     /* 0 */
    float    gravity;                     /* 9.81 */
    float    continental_crust_density;   /* 2835: the load's density */
    float    elastic_thickness_km;        /* 30 */
    float    youngs_modulus_gpa;          /* 70 */
    float    poisson_ratio;               /* 0.25 */
    int32_t  reserved;
} cg_erosion_params;

/* Per-cell inputs of one world (ErosionTectonics + the weather the rounds cut with). */
typedef struct cg_inputs {
    const float* height;               /* required: uplifted terrain, field units */
    const float* uplift_mm_per_year;   /* or NULL: ErosionTectonics.upliftRateMmPerYear */
    const float* rock_erodibility;     /* or NULL: ErosionTectonics.rockErodibility */
    const float* rainfall_mm;          /* or NULL (all 1): HydraulicErosion.Weather.rainfallMm */
    const float* vegetation_density;   /* or NULL (all 0): HydraulicErosion.Weather.vegetationDensity */
} cg_inputs;

/* The last round's basins (FlowRouting.Spillways, .../pipeline/FlowRouting.kt:519-544). */
typedef struct cg_basins {
    int32_t  capacity;       /* entries each array below holds */
    int32_t  count;          /* basins found (may exceed capacity: arrays then hold the first) */
    int32_t* spill;          /* pour point or -1 */
    int32_t* entry;          /* lowest exit, ties on index, or -1 */
    float*   level;
    float*   floor;
    int32_t* cells;
    int32_t  largest;
    int32_t  largest_cells;
    float    largest_depth;
    float    deepest;
} cg_basins;

/* What cg_erode_stage hands back. Every pointer except height may be NULL. */
typedef struct cg_outputs {
    float*    height;          /* required: N, the stage's result (ErosionResult.height) */
    int32_t*  receivers;       /* N: last round's flowDirections, -1 = none */
    float*    area;            /* N: last round's accumulate */
    float*    filled;          /* N: last round's fillDepressions */
    float*    relative;        /* N: last round's shoreline-relative field */
    uint8_t*  is_land;         /* N: last round's land mask */
    int32_t*  order;           /* N: last round's drainageOrder, land cells first */
    int32_t*  basin_of_cell;   /* N: last round's basin label of each ponded cell, else -1 */
    int32_t*  donors;          /* N: last round's donor count (land donors into a land cell) */
    cg_basins* basins;         /* last round's spillways */
} cg_outputs;

/* One hydraulic round's bookkeeping, an observer only (like RoundMass). */
typedef struct cg_round_stats {
    int32_t round;
    int32_t land_cells;
    float   shoreline;
    int32_t basins;
    int32_t flats;              /* FlatRouting.Surface.flats */
    int32_t flats_kept;         /* FlatRouting.Surface.flatsKept */
    int32_t raised_cells;       /* FlatRouting.Surface.raisedCells */
    int32_t levels;             /* drainage levels (longest donor chain + 1) */
    int64_t fill_ties;          /* cells whose fill parent was decided on a quantised-key tie */
    int64_t fill_unresolved;    /* of those, ties the fill could not order exactly (expected 0) */
    int64_t kernel_launches;    /* kernels this library launched for the round */
    double  ms_total;           /* device time of the round, milliseconds (CUDA events) */
    double  ms_cut;             /* uplift, percentile cut and weights */
    double  ms_fill;            /* fillDepressions */
    double  ms_route;           /* flat potentials and receivers */
    double  ms_tree;            /* donor counts, drainage keys and accumulation */
    double  ms_incise;          /* the implicit incision (P1, P2: with the round's notch) */
    double  ms_relax;           /* the round's thermal sweeps */
    double  ms_deposit;         /* P2's deposition walk and, in the last round, settle, the closing
                                   breach (P1, P2: its cut, fill, routing and notch) and the mouths pass */
    int32_t deposit_replayed;   /* P2: ponded cells whose settled height the level schedule replayed */
    int32_t deposit_redone;     /* P2: cells with a mouth refitted, the later fans of their level laid again */
    int32_t deposit_refitted;   /* P2: dry cells whose own walk was taken again with their donors as
                                   the reference's walk showed them */
    int32_t deposit_waves;      /* P2: the lake fans' laying waves over the round's levels */
    /* P2: where the deposition walk's time went (device clock, milliseconds): the own walks and the
       mouths' listing; the laying schedules; the lake fans and sea lobes laid (each waiting on the
       earlier ones that share its cells or tiles); the level logs' assembly; and the mouth-conflict
       searches, relays and last repairs. */
    double  ms_deposit_walks;
    double  ms_deposit_schedule;
    double  ms_deposit_lakes;           /* the lake fans and sea lobes laid */
    double  ms_deposit_seas;            /* the level logs assembled */
    double  ms_deposit_repairs;
    double  ms_flexure;         /* P3: the uplift and the plate flexure at the top of the round (ms_cut then
                                   holds the cut and the weights alone); 0 below P3 */
} cg_round_stats;

typedef struct cg_ctx cg_ctx;

/* Fills reference defaults (WorldGenConfig(seed, width, height), P0 switches). */
void cg_default_params(cg_erosion_params* params, int32_t width, int32_t height, int64_t seed);

/* The thermal limits and sweep count the reference derives (ErosionStage.kt:412-437). */
cg_status cg_thermal_limits_for(const cg_erosion_params* params, cg_thermal_limits* limits,
                                int32_t* sweeps);

cg_status cg_create(cg_ctx** ctx, int32_t device);
void      cg_destroy(cg_ctx* ctx);
/* Async-signal-safe: sets a flag the stage polls between phases and rounds. */
void      cg_cancel(cg_ctx* ctx);
/* The message of the last failure on this context (static storage, never NULL). */
const char* cg_last_error(const cg_ctx* ctx);
/*
 * The CUDA stream every kernel of this context runs on (a cudaStream_t), for callers that time the
 * stage with events on the launching stream or order their own work after it. No counterpart in the
 * reference.
 */
void*     cg_stream(const cg_ctx* ctx);
/* Kernels this context has launched since it was created. No counterpart in the reference. */
int64_t   cg_kernel_launches(const cg_ctx* ctx);
/*
 * This GPU's measured FP64 fused multiply-add rate in GFLOP/s (a chain of independent FMAs on every
 * SM, best of four timed launches): the ceiling of the phases the reference computes in double, for
 * their roofline. No counterpart in the reference.
 */
cg_status cg_probe_fp64_rate(cg_ctx* ctx, double* gflops);

/*
 * ErosionAccelerator.erode (.../pipeline/ErosionAccelerator.kt:38-45; ErosionStage.kt:235-403):
 * `passes` Musgrave sweeps over heights_in into heights_out (a separate array).
 */
cg_status cg_thermal_sweeps(cg_ctx* ctx, int32_t width, int32_t height, const float* heights_in,
                            float* heights_out, cg_thermal_limits limits, int32_t passes, float rate);

/*
 * cg_thermal_sweeps for callers that cannot allocate device memory. No counterpart in the
 * reference. Some callers must not call cudaMalloc: a JVM inside a memory-accounted container
 * lending buffers it owns, a renderer that owns every allocation on its device, code replaying a
 * graph captured elsewhere. This entry point needs no context and allocates nothing: the caller
 * passes the input and output as device pointers (different buffers; the input is not written),
 * and the one scratch field lives in a file-scope device array sized for grids of up to 2^20 cells
 * (4 MiB, held by every GPU that loads the library until exit). Larger grids, a non-power-of-two
 * side, input and output byte ranges that overlap at all, or negative passes return CG_BAD_ARG.
 * Every CUDA context holds its own copy of the array: the first call in a context (the primary one
 * or a driver-API context the caller made current) looks up the array's address with that context
 * current, so make it before any stream capture. Calls share the array: calls whose work overlaps
 * on the GPU race. `stream` is a cudaStream_t or NULL; the call returns when the work is queued.
 */
cg_status cg_thermal_sweeps_noalloc(const float* heights_in_dev, float* heights_out_dev, int32_t width,
                                    int32_t height, cg_thermal_limits limits, int32_t passes, float rate,
                                    void* stream);

/*
 * ErosionStage.apply (.../pipeline/ErosionStage.kt:133-183) with HydraulicErosion.apply
 * (.../pipeline/HydraulicErosion.kt:596-1506): the initial thermal sweeps, then the hydraulic
 * rounds, each relaxed by sweepsFor/rounds sweeps. `stats`, if not NULL, receives one entry per
 * round (hydraulic_rounds entries).
 */
cg_status cg_erode_stage(cg_ctx* ctx, const cg_erosion_params* params, const cg_inputs* inputs,
                         cg_outputs* outputs, cg_round_stats* stats);

/*
 * cg_erode_stage on a world already resident on this context's device: every pointer of `inputs_dev`
 * is device memory (read only), and `height_out_dev` (device, N floats, may alias nothing in the
 * inputs) receives the result. No host<->device copy of the fields; the caller's stream is not
 * used, the call returns when the stage is done. Returns the last round's land-cell count in
 * *land_cells (may be NULL). No counterpart in the reference, which has no device-resident world;
 * it is the same stage as cg_erode_stage for callers that keep the world in HBM.
 */
cg_status cg_erode_stage_dev(cg_ctx* ctx, const cg_erosion_params* params, const cg_inputs* inputs_dev,
                             float* height_out_dev, cg_round_stats* stats, int32_t* land_cells);

/* ---- The belts' replay (BeltErosion.replay, .../pipeline/BeltErosion.kt:96-425) ----
 *
 * Before the hydraulic rounds, when the plate stage hands the erosion the belts' recent history
 * (ErosionTectonics.window; HydraulicErosion.kt:680-688), each young belt is lowered to where its crust
 * stood when the exposure window opened, raised again round by round at the rate its own thickening
 * came at, and cut as it rises: about a hundred rounds over the belt cells alone, each with a priority
 * flood over the belts, the facet rule, the Kahn order, the implicit incision, the spoil carried to the
 * belts' outlets and the rounds' thermal sweeps, and every ten rounds the crust's Airy rebound of the
 * rock taken (a Gaussian of GaussianBlur, .../math/GaussianBlur.kt, at the crust map's spread). */
/* BeltWindow (BeltErosion.kt:19-24): per cell, what tectonics did to the crust over the window. */
typedef struct cg_belt_window {
    const float* tectonic_km;      /* N: km of thickness thickened over the window */
    const float* wear_km;          /* N: km the orogens' wear took over it */
    const float* onset_myr_ago;    /* N: when the thickening began, Myr ago; < 0 where none did */
    double       window_myr;       /* the window's length, Myr (PlateResult.exposureWindowMyr, 40) */
} cg_belt_window;
/* The rest of BeltErosion.replay's arguments (host buffers, N floats each where given). */
typedef struct cg_belt_inputs {
    const float* uplift_mm_per_year;   /* or NULL: presentUpliftMmPerYear */
    const float* rainfall_mm;          /* or NULL (all 1): the opening weather's rain */
    const float* cover_density;        /* or NULL (all 0): the opening weather's cover */
    const float* rock_erodibility;     /* or NULL */
    const float* unresolved_relief;    /* or NULL: UnresolvedRelief in the height field's units */
    float        provisional_sea_level;/* the sea fraction the opening cut takes (WorldGenConfig.seaLevel) */
    int32_t      shield_cut;           /* 1: the cover's shielding in the incision's factor */
    int32_t      rebound;              /* IsostasyConfig.enabled: the crust answers the rock taken */
    double       history_cell_km;      /* TectonicsConfig.historyCellKm (80): the rebound's spread is 0.6 of it */
} cg_belt_inputs;
/* BeltReplay (BeltErosion.kt:35-47) without erodedMeters, which the call writes to its own buffer. */
typedef struct cg_belt_books {
    int32_t rounds;                         /* 0 where the replay does nothing (BeltReplay.NOTHING) */
    int32_t belt_cells;
    double  uplifted_cubic_meters;
    double  cut_cubic_meters;
    double  exported_to_sea_cubic_meters;
    double  exported_to_land_cubic_meters;
    double  shed_beside_cubic_meters;
} cg_belt_books;
/* ---- The stage round by round, its world resident on the context between calls ----
 *
 * HydraulicErosion.apply asks for the weather twice when ErosionConfig.climateFeed is on: on the
 * terrain the initial sweeps left, and again at the top of round hydraulic_rounds / 2 on the terrain
 * the rounds have left (HydraulicErosion.kt:655-661, 809-813, through provisionalWeather,
 * HydraulicErosion.kt:410-470). That solve is a climate stage and stays the caller's. These calls
 * split ErosionStage.apply where the weather is asked, with the world held in HBM in between:
 *   cg_stage_begin (inputs, initial sweeps) -> cg_stage_height (solve the weather) ->
 *   cg_erode_rounds(0, R/2, weather A) -> cg_stage_height (solve again) ->
 *   cg_erode_rounds(R/2, R, weather B) -> cg_stage_finish (outputs).
 * Without climate_feed any split of [0, R) gives cg_erode_stage's result bit for bit (SURVEY's
 * round-granular resume). Any other call on the context ends the resident world. */

/* The weather the rounds cut with from a given round on (HydraulicErosion.Weather). */
typedef struct cg_weather {
    const float* rainfall_mm;          /* or NULL (all 1) */
    const float* vegetation_density;   /* or NULL (all 0) */
} cg_weather;

/* Uploads the world and runs the initial thermal sweeps (ErosionStage.kt:163-172). inputs'
 * rainfall and cover, if given, are the weather of the first rounds. */
cg_status cg_stage_begin(cg_ctx* ctx, const cg_erosion_params* params, const cg_inputs* inputs);

/*
 * Runs rounds [first_round, end_round) of the resident world (first_round = the rounds run so far),
 * each with its relaxation and, in the last round, the stage's closing passes. `weather` (may be
 * NULL: keep the current one) replaces the weather from first_round on. With climate_feed the call
 * at round 0 and the call at round hydraulic_rounds / 2 must bring the weather, and no call may run
 * across round hydraulic_rounds / 2. `stats` (may be NULL) receives one entry per round run. If a
 * round finds no land the rounds stop there, as in the reference; later calls do nothing.
 */
cg_status cg_erode_rounds(cg_ctx* ctx, int32_t first_round, int32_t end_round, const cg_weather* weather,
                          cg_round_stats* stats);

/*
 * The belts' replay (BeltErosion.replay, see cg_belt_replay below) on the resident world, where
 * HydraulicErosion.apply runs it: after the initial sweeps and the opening weather, before round 0
 * (HydraulicErosion.kt:680-688). It reads the stage's uplift and rock, `weather` (may be NULL: the
 * weather the world was begun with; with climate_feed, the opening weather the caller solved), the
 * stage's sea level and shield_cut, and no sub-grid relief (the rounds take none). `rebound` is
 * IsostasyConfig.enabled and `history_cell_km` TectonicsConfig.historyCellKm (80). With profile P3 the
 * flexure's field before the rounds becomes the replayed one, as in the reference. `eroded_meters`
 * (N, host, may be NULL) and `books` receive the replay's results; a stage that erodes nothing
 * (no rounds or no erodibility) replays nothing, as the reference returns before the replay.
 */
cg_status cg_stage_replay_belts(cg_ctx* ctx, const cg_belt_window* window, const cg_weather* weather,
                                int32_t rebound, double history_cell_km, float* eroded_meters,
                                cg_belt_books* books);
/* The resident world's current height field (N floats, host), e.g. for the caller's weather solve. */
cg_status cg_stage_height(cg_ctx* ctx, float* height);

/* After the last round: cg_erode_stage's outputs for the resident world, which is then released. */
cg_status cg_stage_finish(cg_ctx* ctx, cg_outputs* outputs);

/* One world of a batch: its own grid, seed and scale, host inputs and host outputs. */
typedef struct cg_world {
    cg_erosion_params params;
    cg_inputs inputs;
    cg_outputs outputs;     /* outputs.height required */
} cg_world;

/*
 * Many worlds in one call (seeds and planet sizes of different grid shapes): each world's result is
 * exactly cg_erode_stage's on that world. The worlds run one after another on this context's device,
 * reusing its buffers (grown to the largest world). `status` (may be NULL, n_worlds entries) receives each
 * world's cg_status. Returns CG_OK if every world succeeded, else the first failure's status; a
 * failed world does not stop the others, except CG_CANCELLED, which stops the batch (the worlds not
 * run get CG_CANCELLED). No counterpart in the reference, which generates one world at a time.
 */
cg_status cg_erode_batch(cg_ctx* ctx, int32_t n_worlds, const cg_world* worlds, cg_status* status);

/* ---- The stage's routing functions, each run alone on host buffers (FlowRouting, SeaLevelStage) ---- */

/*
 * FlowRouting's routing of one sea-level cut in one call, as the stages after the erosion run it on
 * their own cut: fillDepressions, flowDirections (params' seed, cell aspect, lattice, facet_routing and
 * flat_potential), accumulate with `weights` (all ones when NULL, the `{ 1f }` of DrownedValleys) and
 * drainageOrder (land cells first, land_cells entries). DrownedValleys.kt:411-421, RiverStage.kt:228-240
 * and 306-308 (with the runoff as weights), GlaciationStage.kt:371-385 (the order for its ice walk).
 * Host buffers; `receivers` is required, `filled`, `area` and `order` may be NULL.
 */
cg_status cg_route_cut(cg_ctx* ctx, const cg_erosion_params* params, const uint8_t* is_land, const float* relative,
                       int32_t land_cells, const float* weights, float* filled, int32_t* receivers, float* area,
                       int32_t* order);
/* SeaLevelStage.percentileCut (.../pipeline/SeaLevelStage.kt:146-200, 579-651). */
cg_status cg_percentile_cut(cg_ctx* ctx, int32_t width, int32_t height, const float* heights,
                            float sea_level_fraction, float highest_land_metres,
                            float deepest_ocean_metres, float lowstand_share_of_field,
                            float* shoreline, uint8_t* is_land, float* relative,
                            int32_t* land_cells);

/*
 * SeaLevelStage.apply's cut up to the drowned basins' outlets (.../pipeline/SeaLevelStage.kt:243-270):
 * the percentile cut at today's stand, the enclosure rule (markUnreachableWaterAsLand, :371-437: every
 * water body but the ocean no larger than enclosed_sea_max_share of the planet's map area becomes land)
 * and, with post_cut_outlet, up to 16 outlet passes over the basins whose floor lies below the
 * shoreline (drainDrownedBasins, :478-560: fill, routing, accumulation and spillways over the whole
 * grid, the notch with belowSea, then the re-cut at the same shoreline). The reference runs the
 * erosion stage's routing here, outside the stage. The drowned valleys, littoral grading and shelf
 * that follow in SeaLevelStage.apply are not this library's. `height` is host memory and is not
 * written (the passes cut a copy); `passes` (may be NULL) receives the outlet passes that cut.
 * Defaults: SeaConfig.enclosedSeaMaxShareOfSurface 0.00073, postCutOutlet 1.
 */
cg_status cg_sea_level_cut(cg_ctx* ctx, const cg_erosion_params* params, const float* height,
                           double enclosed_sea_max_share, int32_t post_cut_outlet, float* shoreline,
                           uint8_t* is_land, float* relative, int32_t* land_cells, int32_t* passes);

/*
 * Isostasy.Flexure(config).deflectionMetres(load, out) (.../pipeline/Isostasy.kt:277-372, over
 * math/Fft.kt's Fft2D): the plate's bend, in metres (positive down), under `load` pascals (host memory,
 * width x height of `params`), bit-exact to the reference's transform: the load less its mean, mirrored
 * about each pole to 2 x height rows, the low-pass 1 / (dRho g + D k^4) with the zero-frequency term
 * dropped. `rigidity` (D) and `restoring` (dRho g) may be NULL. Needs width <= 8192 and height <= 4096.
 */
cg_status cg_flexure_deflection(cg_ctx* ctx, const cg_erosion_params* params, const float* load,
                                float* deflection, double* rigidity, double* restoring);

/*
 * The reference's sequential double sum of a float field, `var s = 0.0; for (c in cells) s += v[c]`,
 * bit for bit: the sums behind normaliseOverLand's rain mean and shieldingOverLand's cover mean
 * (.../pipeline/HydraulicErosion.kt:476-486, 557-567; mode 1 sums 1 - 0.5 x, the cover's factor) and
 * deflectionMetres' load mean (.../pipeline/Isostasy.kt:337-339). Cells with mask[c] == 0 are skipped
 * (mask may be NULL). Host buffers. The stage computes these sums on the device the same way; this entry
 * point exposes the primitive on its own. The sum is not a chain of n double additions: blocks of values
 * are reduced in parallel to integer walks inside the running sum's binade (the one state a walk carries
 * is the parity of the sum's mantissa, which decides ties), and only where the sum crosses a binade are
 * values added one at a time. `counts` (3 entries, may be NULL) receives blocks of 8192 values taken
 * whole, pieces of 1024 reduced on the spot, and pieces added one value at a time.
 */
cg_status cg_sequential_sum(cg_ctx* ctx, const float* x, const uint8_t* mask, int32_t mode, int64_t n,
                            double* sum, int64_t* counts);

/* FlowRouting.fillDepressions (.../pipeline/FlowRouting.kt:52-111). */
cg_status cg_fill_depressions(cg_ctx* ctx, int32_t width, int32_t height, const uint8_t* is_land,
                              const float* relative, float* filled, int64_t* ties,
                              int64_t* unresolved);

/*
 * FlowRouting.flowDirections (.../pipeline/FlowRouting.kt:179-216) with FlatRouting.surfaceOf
 * (.../pipeline/FlatRouting.kt:58-138). `surface` (N doubles) may be NULL; `flat_counts` may be
 * NULL or receives {flats, flatsKept, raisedCells}.
 */
cg_status cg_flow_directions(cg_ctx* ctx, int32_t width, int32_t height, const uint8_t* is_land,
                             const float* relative, const float* filled, int64_t seed,
                             double cell_height_in_cell_widths, int32_t smooth_lattice_columns,
                             int32_t by_facet, int32_t over_potential, int32_t* receivers,
                             double* surface, int32_t* flat_counts);

/* FlowRouting.drainageOrder (.../pipeline/FlowRouting.kt:695-729); `order` holds land_cells. */
cg_status cg_drainage_order(cg_ctx* ctx, int32_t width, int32_t height, const uint8_t* is_land,
                            const int32_t* receivers, int32_t land_cells, int32_t* order);

/* FlowRouting.accumulate (.../pipeline/FlowRouting.kt:485-511) with per-cell weights. */
cg_status cg_accumulate(cg_ctx* ctx, int32_t width, int32_t height, const uint8_t* is_land,
                        const int32_t* receivers, int32_t land_cells, const float* weights,
                        float* area);

/* FlowRouting.spillways (.../pipeline/FlowRouting.kt:573-677). */
cg_status cg_spillways(cg_ctx* ctx, int32_t width, int32_t height, const uint8_t* is_land,
                       const float* relative, const float* filled, const int32_t* receivers,
                       float pond_depth, int32_t* basin_of_cell, cg_basins* basins);

/*
 * HydraulicErosion.breach (.../pipeline/HydraulicErosion.kt:1931-2171), the outlet notch of profile
 * P1, over the basins FlowRouting.spillways finds on this routing (`ground` is the filled surface):
 * belowSea false, nothing carried. `relative`, `ground` and `surface` (the height field) are cut in
 * place; `cells_cut` (may be NULL) receives the cells the notch lowered. Rates come from `params`.
 */
cg_status cg_breach(cg_ctx* ctx, const cg_erosion_params* params, const uint8_t* is_land,
                    float* relative, float* ground, const int32_t* receivers, const float* area,
                    float land_cells, float land_range, float* surface, int32_t* cells_cut);

/*
 * The sequential double sum over n double terms given in the order they are added, `var s = 0.0;
 * for (v in x) s += v`, bit for bit, by the same parallel walks (host buffers). The belts' replay keeps
 * its books with it; a running total is carried by laying it first. No counterpart in the reference.
 */
cg_status cg_sequential_sum_f64(cg_ctx* ctx, const double* x, int64_t n, double* sum);
/*
 * BeltErosion.replay on host buffers: `height` (N, the height field) is replayed in place, `eroded_meters`
 * (N, may be NULL) receives the metres each cell lost, `books` the replay's figures. Reads params' grid,
 * seed, WorldScale, ErosionConfig (rounds, erodibility, rate, critical fall, debris travel), facet_routing
 * and flat_potential (the opening's routing) and the isostasy densities. Bit-identical to the reference's
 * arithmetic; CG_INEXACT if a belt flood's quantised-key ties cannot be ordered exactly.
 */
cg_status cg_belt_replay(cg_ctx* ctx, const cg_erosion_params* params, float* height, const cg_belt_window* window,
                         const cg_belt_inputs* inputs, float* eroded_meters, cg_belt_books* books);
/* GaussianBlur.apply (.../math/GaussianBlur.kt:44-111) in place on a host field: x wraps, y clamps; a
 * sigma of zero or less leaves that axis alone. The taps are the Gaussian at cell centres to 4 sigma,
 * normalised, computed on the host. */
cg_status cg_gaussian_blur(cg_ctx* ctx, int32_t width, int32_t height, float* field, double sigma_across,
                           double sigma_down);

#ifdef __cplusplus
}
#endif

#endif /* CG_EROSION_H */
