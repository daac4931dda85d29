"""Roofline bookkeeping for the stage's phases.

Algorithmic bytes per cell and round are the compulsory reads and writes of each phase, with
B = 4 bytes per height (the REF32 field):
  cut (uplift 4 + 2B, sea-level cut 3B + B + 1, weights 12)   41
  fill (B + 1 + B)                                               9
  route (routing surface 2B + 8, receivers 8 + 4)               28
  tree (donor counts, keys, accumulation: 4+4+4+4+B)            20
  incise (5B + 8 + B)                                           32
  deposit (P2's walk: routing, cut and load inputs 33, incisedAt 8, load 8, settled and sediment
           read and written 16, hand-off 8, order and rank 8)     81
  relax (s sweeps, a read and a write of the field each: 2B s)   8 s
The plate flexure (P3) is bound by the FP64 pipe instead: its two 2D transforms over the W x 2H
mirrored grid take 5 flops per point per radix-2 stage, 20 (log2 W + log2 2H) flops per map cell
and round, against the FP64 rate the bench measures on the GPU it runs on (cg_probe_fp64_rate).
The peak is the measured HBM copy bandwidth of the GB300s (MEASURED_PEAKS.json, written by
the pool's driver), else the recipe's fallback of 6.8 TB/s.
"""
import json
import os

BYTES_PER_CELL = {"ms_cut": 41.0, "ms_fill": 9.0, "ms_route": 28.0, "ms_tree": 20.0, "ms_incise": 32.0,
                  "ms_deposit": 81.0}
PHASE_KERNELS = {
    "ms_cut": "k_minmax, k_row_counts, k_bin_sums, k_bracket_*, k_land_and_water, k_uplift, k_unit_weights",
    "ms_fill": "k_fill_init, k_jump, k_mark_drained, k_relax_tiles, k_check_ties",
    "ms_route": "k_surface, k_cc_*, k_flat_solve_warp/_sm/_cl, k_flat_solve, k_receivers",
    "ms_tree": "k_links, k_sources, k_walk",
    "ms_incise": "k_depth_*, k_incise_levels (P1, P2: the notch's k_footprint_*, k_breach_waves)",
    "ms_deposit": "k_round_begin, k_rank_of, k_level_bounds, k_deposit_levels, k_settle, k_mouths_levels "
                  "(last round: the closing breach's cut, fill, routing and notch)",
    "ms_relax": "thermal_sweeps_kernel",
    "ms_flexure": "k_uplift, k_flex_load, k_flex_mean, k_fft_lines, k_transpose, k_flex_apply",
}
FALLBACK_HBM_GBS = 6800.0


def peak_hbm(root):
    path = os.path.join(root, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM_GBS, "fallback"


def phase_bytes_per_cell(phase, sweeps_per_round):
    if phase == "ms_relax":
        return 8.0 * sweeps_per_round
    return BYTES_PER_CELL[phase]


def sweep_launches(sweeps):
    """Fused thermal launches for `sweeps` sweeps: two sweeps per launch, one for an odd rest."""
    return (sweeps + 1) // 2


def flexure_flops_per_cell(W, H):
    return 20.0 * ((W.bit_length() - 1) + ((2 * H).bit_length() - 1))


def roofline_entry(cfg, phase_ms_per_stage, root, traffic=None, fp64_gflops=None):
    """The roofline object for the dominant kernel, the thermal sweeps of the relax phase.

    phase_ms_per_stage maps ms_* to that phase's device milliseconds summed over a stage's rounds
    (CUDA events the library records on its stream around each phase, over the timed steps). The
    relax phase is nothing but the fused sweep launches, so their average launch duration is the
    phase's time over its launches, and a launch's algorithmic bytes are a read and a write of the
    height field per sweep it fuses (8 B per cell-sweep). `traffic` is the DRAM bytes of one launch
    from an ncu capture, or None. The other phases follow under "phases", each against its own
    compulsory bytes per cell and round (the module docstring).
    """
    p = cfg.params
    N = p.width * p.height
    rounds = max(p.hydraulic_rounds, 1)
    _, sweeps = cfg.thermal_limits()
    per_round = max(sweeps // rounds, 1)
    launches = sweep_launches(per_round)
    peak, kind = peak_hbm(root)
    ms_launch = phase_ms_per_stage["ms_relax"] / rounds / launches
    algo = 8.0 * N * per_round / launches   # bytes per launch (average over the round's launches)
    achieved = algo / (ms_launch / 1000.0) / 1e9 if ms_launch > 0 else 0.0
    phases = {}
    for k, v in phase_ms_per_stage.items():
        if k == "ms_total" or v <= 0:
            continue
        if k == "ms_flexure":
            gfs = flexure_flops_per_cell(p.width, p.height) * N / (v / rounds / 1000.0) / 1e9
            phases["flexure"] = {"achieved": round(gfs, 1), "unit": "GFLOP/s (FP64)",
                                 "frac": round(gfs / fp64_gflops, 4) if fp64_gflops else None,
                                 "peak": round(fp64_gflops, 1) if fp64_gflops else None,
                                 "ms_per_round": round(v / rounds, 3), "kernels": PHASE_KERNELS[k]}
            continue
        gbs = phase_bytes_per_cell(k, per_round) * N / (v / rounds / 1000.0) / 1e9
        phases[k[3:]] = {"achieved": round(gbs, 1), "frac": round(gbs / peak, 4),
                         "ms_per_round": round(v / rounds, 3), "kernels": PHASE_KERNELS[k]}
    return {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "traffic": traffic, "peak_kind": kind,
            "kernel": "thermal_sweeps_kernel (relax phase)", "launches_per_round": launches,
            "algorithmic_bytes_per_launch": algo, "ms_per_launch": round(ms_launch, 4), "phases": phases}
