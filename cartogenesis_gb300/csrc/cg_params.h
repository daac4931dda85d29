// Host-side derivation of the stage's constants from the configuration, as the reference derives
// them once per generation: WorldScale (M/WorldGenConfig.kt:32-304), HydraulicErosion.Rates
// (P/HydraulicErosion.kt:203-312), ErosionStage.thermalLimits / sweepsFor (ErosionStage.kt:412-437),
// HydraulicErosion.standBelowToday (HydraulicErosion.kt:365-373). Same float and double steps as the
// Kotlin, so every constant a kernel receives has the reference's bits.
#pragma once

#include <cmath>
#include <cstring>

#include "../../include/cg_erosion.h"

namespace cg {

struct ScaleF {
    double world_width_km;
    float highest_land;
    float deepest_ocean;
    double years_per_round;
    float relief_span() const { return highest_land + deepest_ocean; }
    float land_half() const { return highest_land / relief_span(); }
    float sea_half() const { return deepest_ocean / relief_span(); }
    float relief_share_of_metres(float m) const { return m / highest_land; }
    float field_share_of_metres(float m) const { return m / relief_span(); }
    double cell_width_km(int w) const { return world_width_km / w; }
    double cell_height_km(int h) const { return world_width_km * 0.5 / h; }
    double world_area_km2() const { return world_width_km * world_width_km * 0.5; }
};

inline ScaleF scale_of(const cg_erosion_params& p) {
    return ScaleF{p.world_width_km, p.highest_land_metres, p.deepest_ocean_metres, p.years_per_hydraulic_round};
}

inline void default_params(cg_erosion_params* p, int width, int height, int64_t seed) {
    std::memset(p, 0, sizeof(*p));
    p->abi_version = CG_ABI_VERSION;
    p->width = width;
    p->height = height;
    p->mode = CG_MODE_REF32;
    p->seed = seed;
    p->world_width_km = 40075.0;                 // WorldScale.EARTH_EQUATOR_KM
    p->highest_land_metres = 6000.0f;
    p->deepest_ocean_metres = 10000.0f;
    p->years_per_hydraulic_round = 336476.4;
    p->enabled = 1;
    p->critical_fall_metres_per_km = 60.0f;
    p->debris_travel_km = 1875.0;
    p->rate = 0.25f;
    p->hydraulic_rounds = 12;
    p->bedrock_erodibility_per_year = 1e-6f;
    p->facet_routing = 1;
    p->flat_potential = 1;
    p->sea_level = 0.71f;
    p->lowstand_metres = 120.0f;
    p->receiver_clamp = 1;
    p->shield_cut = 1;
    p->profile = CG_PROFILE_P0;
    p->mantle_density = 3300.0f;
    p->deflection_fill_density = 0.0f;
    p->gravity = 9.81f;
    p->continental_crust_density = 2835.0f;
    p->elastic_thickness_km = 30.0f;
    p->youngs_modulus_gpa = 70.0f;
    p->poisson_ratio = 0.25f;
}

// WorldGenConfig.wholeCellsFor: kotlin.math.round rounds half to even (nearbyint).
inline int whole_cells_for(const cg_erosion_params& p, double km, int at_least) {
    float cells = (float)(km * p.width / p.world_width_km);
    int r = (int)std::nearbyint(cells);
    return r < at_least ? at_least : r;
}

inline int sweeps_for(const cg_erosion_params& p) { return whole_cells_for(p, p.debris_travel_km, 0); }

inline cg_thermal_limits thermal_limits(const cg_erosion_params& p) {
    ScaleF s = scale_of(p);
    double critical_per_km = (double)p.critical_fall_metres_per_km / (double)s.relief_span();
    double cw = s.cell_width_km(p.width), ch = s.cell_height_km(p.height);
    cg_thermal_limits l;
    l.east_west = (float)(critical_per_km * cw);
    l.north_south = (float)(critical_per_km * ch);
    l.diagonal = (float)(critical_per_km * std::sqrt(cw * cw + ch * ch));
    return l;
}

inline int smooth_field_lattice_columns(double world_width_km) {
    int r = (int)std::nearbyint(world_width_km / 187.5);   // FlowRouting.SMOOTH_FIELD_PERIOD_KM
    return r < 1 ? 1 : r;
}

struct RatesF {
    float incision_coefficient;
    float courant_coefficient;
    float pond_depth;
    float step_ns;
    float step_diag;
    double cell_height_in_cell_widths;
    // The outlet notch's constants (profile P1).
    float relative_incision_coefficient;   // HydraulicErosion.kt:246-247
    float notch_fall_per_cell;             // HydraulicErosion.kt:281-282, NOTCH_FALL_METRES_PER_KM 0.0025
    int outlet_reach_cells;                // HydraulicErosion.kt:303, ErosionConfig.outletReachKm 1500
};

inline RatesF rates_of(const cg_erosion_params& p) {
    ScaleF s = scale_of(p);
    RatesF r;
    double sl = (double)p.sea_level;
    sl = sl < 0.0 ? 0.0 : (sl > 1.0 ? 1.0 : sl);
    double land_area = (1.0 - sl) * s.world_area_km2();
    double per_year = (double)p.bedrock_erodibility_per_year * s.years_per_round;
    double geometry = std::sqrt(land_area) / s.world_width_km;
    double ratio = (double)s.highest_land / (double)s.relief_span();
    r.incision_coefficient = (float)(per_year * geometry * ratio);
    r.courant_coefficient = r.incision_coefficient / s.land_half() * (float)p.width;
    r.pond_depth = s.relief_share_of_metres(24.0f);   // HydraulicErosion.POND_DEPTH_METRES
    r.cell_height_in_cell_widths = s.cell_height_km(p.height) / s.cell_width_km(p.width);
    double cr = r.cell_height_in_cell_widths;
    r.step_ns = (float)cr;                          // GroundSteps.northSouth
    r.step_diag = (float)std::sqrt(1.0 + cr * cr);  // GroundSteps.diagonal
    r.relative_incision_coefficient = r.incision_coefficient * s.relief_span() / s.highest_land;
    r.notch_fall_per_cell = s.relief_share_of_metres(0.0025f * (float)s.cell_width_km(p.width));
    r.outlet_reach_cells = whole_cells_for(p, 1500.0, 1);
    return r;
}

inline float stand_below_today(const cg_erosion_params& p, int round) {
    ScaleF s = scale_of(p);
    float lowstand = s.field_share_of_metres(p.lowstand_metres);
    int rounds = p.hydraulic_rounds;
    if (lowstand <= 0.0f || rounds <= 1) return 0.0f;
    int rising = (int)((float)rounds * 0.25f);   // TRANSGRESSION_SHARE
    if (rising < 1) rising = 1;
    int held = rounds - rising;
    if (round < held) return lowstand;
    return lowstand * (float)(rounds - 1 - round) / (float)rising;
}

}  // namespace cg
