"""Roofline bookkeeping for the stage's phases.

Algorithmic bytes per cell and round are the compulsory reads and writes of each phase, with
B = 4 bytes per height (the REF32 field):
  cut (uplift 4 + 2B, sea-level cut 3B + B + 1, weights 12)   41
  fill (B + 1 + B)                                               9
  route (routing surface 2B + 8, receivers 8 + 4)               28
  tree (donor counts, keys, accumulation: 4+4+4+4+B)            20
  incise (5B + 8 + B)                                           32
  relax (s sweeps, a read and a write of the field each: 2B s)   8 s
The peak is the measured HBM copy bandwidth of the GB300s (MEASURED_PEAKS.json, written by
the pool's driver), else the recipe's fallback of 6.8 TB/s.
"""
import json
import os

BYTES_PER_CELL = {"ms_cut": 41.0, "ms_fill": 9.0, "ms_route": 28.0, "ms_tree": 20.0, "ms_incise": 32.0}
PHASE_KERNELS = {
    "ms_cut": "k_minmax, k_row_counts, k_bin_sums, k_bracket_*, k_land_and_water, k_uplift, k_unit_weights",
    "ms_fill": "k_fill_init, k_jump, k_mark_drained, k_relax_tiles, k_check_ties",
    "ms_route": "k_surface, k_cc_*, k_flat_solve, k_receivers",
    "ms_tree": "k_donor_count, k_walk",
    "ms_incise": "k_depth_*, k_incise_levels",
    "ms_relax": "thermal_sweeps_kernel",
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


def roofline_entry(cfg, phase_ms_per_stage, root, traffic=None):
    """The roofline object for the phase that takes the most device time over a stage's rounds.

    phase_ms_per_stage maps ms_* to that phase's device milliseconds summed over the stage's
    rounds (CUDA events on the library's stream).
    """
    p = cfg.params
    N = p.width * p.height
    rounds = max(p.hydraulic_rounds, 1)
    _, sweeps = cfg.thermal_limits()
    per_round = max(sweeps // rounds, 1)
    phases = [k for k in phase_ms_per_stage if k != "ms_total"]
    dom = max(phases, key=lambda k: phase_ms_per_stage[k])
    ms_per_round = phase_ms_per_stage[dom] / rounds
    algo = phase_bytes_per_cell(dom, per_round) * N   # bytes per round of that phase
    achieved = algo / (ms_per_round / 1000.0) / 1e9 if ms_per_round > 0 else 0.0
    peak, kind = peak_hbm(root)
    return {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "traffic": traffic, "peak_kind": kind,
            "kernel": f"{dom[3:]} phase ({PHASE_KERNELS[dom]})",
            "algorithmic_bytes_per_launch_group": algo, "ms_per_round": round(ms_per_round, 3)}
