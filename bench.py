"""Benchmark of the GB300 erosion stage: Mcell-rounds/s of the plain (P0, REF32) stage.

A step is one whole erosion stage (ErosionStage.apply: the initial thermal sweeps, 12 hydraulic
rounds and each round's relaxation) over one synthetic world. The workload is the plain method's
single-GPU configuration: 8192 x 4096 cells (33.5M), fBm heights (beta 2) over [-10000, 6000] m at
30% land by area, uplift ridges of 50-4000 m/Myr along 15 great circles, lognormal rock factor;
383 initial sweeps and 31 per round. Inputs are larger than the 129 MB L2 (the height field alone
is 134 MB), so no flush is needed between steps.

  value: the stage on a world already resident in HBM (cg_erode_stage_dev), CUDA events on the
         library's stream;
  e2e:   the same stage through the host-buffer C ABI call (cg_erode_stage) from pinned memory, the
         host->device copy of the world and the device->host copy of the result inside the timing.
  --impl reference: the CPU restatement of the reference's stage (the Kotlin path cannot run here:
         no JVM), all host threads for the thermal sweeps as the reference's parallelChunks does,
         on a bounded sample of the same workload: per step one round of the 12-round stage on the
         same world after its initial sweeps, plus a twelfth of those sweeps.
  --profile 1: the same measurement of profile P1 (P0 with the outlet notch in every round and the
         closing breach); the default is P0, the plain stage the metric names.
Multi-GPU: replicas only (one independent world per rank, seed = rank + 1); the stage does not
shard within a world, so there is no collective on the data path.
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mcell-rounds/s on 1 GB300: plain vs batched vs surrogate at <=5 m height RMSE"
UNIT = "Mcell-rounds/s"
ROUNDS = 12
# DRAM bytes (read + write) of one two-sweep launch of thermal_sweeps_kernel on the 8192 x 4096
# field, read from an ncu capture of that launch (ncu cannot run inside the timed bench); the
# roofline's traffic at that size, null at other sizes.
SWEEP_TRAFFIC_PER_LAUNCH = 227.5e6


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--width", type=int, default=8192)
    ap.add_argument("--height", type=int, default=4096)
    ap.add_argument("--profile", type=int, default=0, choices=[0, 1, 2, 3],
                    help="round-tail profile: 0 = P0 (the plain stage), 1 = P1 (P0 with the outlet notch and the "
                         "closing breach), 2 = P2 (P1 with deposition, its lobed and outlined deltas and the "
                         "closing mouths pass), 3 = P3 (P2 with the plate flexure: the reference's default)")
    ap.add_argument("--case", default=None, choices=["thermal", "stage"],
                    help="one public call on the bench world for a profiler, then exit: `thermal` runs the sweeps "
                         "(--passes of them), `stage` the stage with --rounds rounds; prints nothing to parse")
    ap.add_argument("--batched", type=int, default=0, metavar="WORLDS",
                    help="the batched workload instead: WORLDS planets of radius U(0.25, 2.0) Earth radii (grids "
                         "512 x 256 to 4096 x 2048, each its own seed) through cg_erode_batch, one batch per step")
    ap.add_argument("--belt", action="store_true",
                    help="the belts' replay instead (BeltErosion.replay, about a hundred rounds over the young "
                         "belts of a 40 Myr exposure window) on the --width x --height world, through "
                         "cg_belt_replay; the line reports belt cell-rounds per second")
    ap.add_argument("--passes", type=int, default=4, help="--case thermal: sweeps")
    ap.add_argument("--rounds", type=int, default=2, help="--case stage: hydraulic rounds")
    ap.add_argument("--cpu-sample", type=int, default=1,
                    help="samples of the CPU baseline (one round of the stage on the bench world plus a twelfth "
                         "of its initial sweeps, on the CPU restatement); 0 skips the CPU leg")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def max_over_ranks(values, world):
    """Each timing's maximum over the ranks (the slowest replica decides the whole job's time)."""
    import torch
    t = torch.tensor(values, dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    if world > 1:
        import torch.distributed as dist
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()


def whole_job_rate(cells, steps, world, seconds):
    """Mcell-rounds/s of the whole job: every rank's world, every round of every step."""
    return float(cells) * ROUNDS * steps * world / seconds / 1e6


def world_inputs(W, H, seed):
    from cartogenesis_gb300 import synthetic
    return synthetic.world(W, H, seed, uplift="ridges")


class CpuSample:
    """The CPU restatement (oracle) on a bounded sample of the bench workload itself: one of the
    12 rounds of the stage on the 8192 x 4096 world, taken from the world after its initial sweeps
    (computed once, untimed), plus a twelfth of those initial sweeps, timed together. Cell-rounds
    per sample: the grid's cells times one round."""

    def __init__(self, W, H, threads, profile=0):
        import oracle
        self.oracle = oracle
        self.W, self.H, self.cores, self.profile = W, H, threads, profile
        h, self.up, self.rk = world_inputs(W, H, 1)
        self.p = oracle.default_params(W, H, 1, sea_level=0.70, profile=profile)
        self.lim, self.sweeps = oracle.thermal_limits(self.p)
        self.share = (self.sweeps + ROUNDS - 1) // ROUNDS
        self.swept = oracle.thermal_sweep(h, self.lim, self.sweeps, self.p.rate)

    def step(self):
        t0 = time.perf_counter()
        self.oracle.thermal_sweep(self.swept, self.lim, self.share, self.p.rate)
        self.oracle.stage_rounds(self.p, self.swept, self.up, self.rk, rounds=1)
        return time.perf_counter() - t0

    def describe(self, n):
        notch = (" (P1: the round's notch included, the stage's one closing breach not)" if self.profile == 1
                 else "")
        return (f"round 1 of the 12-round stage on the {self.W}x{self.H} world after its {self.sweeps} initial "
                f"sweeps, plus {self.share} sweeps (a twelfth of them){notch}; median of {n}")


def cpu_baseline(W, H, steps, threads, profile=0):
    s = CpuSample(W, H, threads, profile)
    times = [s.step() for _ in range(max(steps, 1))]
    t = statistics.median(times)
    return W * H / t / 1e6, t, threads, s.describe(len(times))


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count()))
    threads = int(os.environ["OMP_NUM_THREADS"])
    s = CpuSample(args.width, args.height, threads, args.profile)
    for _ in range(args.warmup):
        s.step()
    times = [s.step() for _ in range(max(args.steps, 1))]
    t = sum(times) / len(times)
    value = args.width * args.height / t / 1e6
    sample = s.describe(len(times)).replace("median", "mean")
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": args.gpus,
        "steps": len(times), "warmup": args.warmup, "ms_per_step": round(t * 1000.0, 1), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"plain P{args.profile} erosion stage (REF32), CPU restatement of the reference: "
                               f"{sample}",
                   "grid": [args.width, args.height], "rounds": ROUNDS, "profile": f"P{args.profile}",
                   "sample_rounds_per_step": 1},
        "cpu_baseline": {"value": round(value, 3), "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    import numpy as np
    import torch

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    from cartogenesis_gb300 import Context, ErosionConfig, abi

    W, H = args.width, args.height
    N = W * H
    seed = rank + 1
    h, up, rk = world_inputs(W, H, seed)
    cfg = ErosionConfig(W, H, seed, sea_level=0.70, profile=args.profile)
    ctx = Context(local)
    lib = ctx.lib

    # Device-resident world.
    d_h = torch.from_numpy(h).cuda()
    d_up = torch.from_numpy(up).cuda()
    d_rk = torch.from_numpy(rk).cuda()
    d_out = torch.empty_like(d_h)
    dev_in = abi.Inputs(d_h.data_ptr(), d_up.data_ptr(), d_rk.data_ptr(), None, None)
    stats = (abi.RoundStats * ROUNDS)()
    land = C.c_int32()
    lib_stream = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", local))

    def step_dev(with_stats=False):
        ctx.check(lib.cg_erode_stage_dev(ctx.handle, C.byref(cfg.params), C.byref(dev_in), d_out.data_ptr(),
                                         C.cast(stats, C.c_void_p) if with_stats else None, C.byref(land)))

    # Host path: pinned inputs and result.
    p_h = torch.from_numpy(h).pin_memory()
    p_up = torch.from_numpy(up).pin_memory()
    p_rk = torch.from_numpy(rk).pin_memory()
    p_out = torch.empty(H, W, dtype=torch.float32).pin_memory()
    host_in = abi.Inputs(p_h.data_ptr(), p_up.data_ptr(), p_rk.data_ptr(), None, None)
    host_out = abi.Outputs(height=p_out.data_ptr())

    def step_e2e():
        ctx.check(lib.cg_erode_stage(ctx.handle, C.byref(cfg.params), C.byref(host_in), C.byref(host_out), None))

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        step_dev()

    # The timed steps also fill cg_round_stats: the library records CUDA events on its stream around
    # each phase of each round, which gives the per-phase device times (and the sweep kernel's
    # launch durations for the roofline) over the timed region itself.
    PHASES = ("ms_flexure", "ms_cut", "ms_fill", "ms_route", "ms_tree", "ms_incise", "ms_deposit", "ms_relax",
              "ms_total")
    phase = {k: 0.0 for k in PHASES}
    clocks = ClockSampler(local)
    barrier()
    launches0 = ctx.kernel_launches
    clocks.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for i in range(args.steps):
        ev[i][0].record(lib_stream)
        step_dev(with_stats=True)
        ev[i][1].record(lib_stream)
        for k in PHASES:
            phase[k] += sum(getattr(s, k) for s in stats) / args.steps
    barrier()
    per_round = [{"land": s.land_cells, "flats": s.flats, "raised": s.raised_cells, "levels": s.levels,
                  "fill_ties": s.fill_ties, "fill_unresolved": s.fill_unresolved, "ms": round(s.ms_total, 2),
                  **({"replayed": s.deposit_replayed, "redone": s.deposit_redone, "refitted": s.deposit_refitted,
                      "waves": s.deposit_waves, "ms_deposit": round(s.ms_deposit, 2),
                      "ms_deposit_parts": {name: round(getattr(s, "ms_deposit_" + k), 2)
                                           for name, k in (("walks", "walks"), ("schedule", "schedule"),
                                                           ("laying", "lakes"), ("log", "seas"),
                                                           ("repairs", "repairs"))}}
                     if args.profile >= 2 else {})}
                 for s in stats]
    clk = clocks.stop()
    launches = ctx.kernel_launches - launches0
    step_ms = [a.elapsed_time(b) for a, b in ev]
    t_dev = sum(step_ms) / 1000.0

    # End to end through the host-buffer call.
    for _ in range(1):
        step_e2e()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step_e2e()
    barrier()
    t_e2e = time.perf_counter() - t0

    t_dev, t_e2e = max_over_ranks([t_dev, t_e2e], world)
    value = whole_job_rate(N, args.steps, world, t_dev)
    e2e = whole_job_rate(N, args.steps, world, t_e2e)

    # Roofline of the dominant kernel, the fused thermal sweeps. Their algorithmic traffic is a read
    # and a write of the height field per sweep (8 B per cell-sweep); with two sweeps fused per
    # launch the kernel moves less than that (the traffic key, from ncu).
    from cartogenesis_gb300.perf import roofline_entry
    fp64 = None
    if args.profile >= 3:   # the flexure's transform runs in FP64: its ceiling, measured on this GPU now
        rate = C.c_double()
        ctx.check(lib.cg_probe_fp64_rate(ctx.handle, C.byref(rate)))
        fp64 = rate.value
    roof = roofline_entry(cfg, phase, ROOT, traffic=SWEEP_TRAFFIC_PER_LAUNCH if (W, H) == (8192, 4096) else None,
                          fp64_gflops=fp64)

    line = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(1000.0 * t_dev / args.steps, 2), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"plain P{args.profile} erosion stage (REF32, bit-exact to the reference restatement), "
                               f"{W}x{H} cells, {ROUNDS} rounds, fBm beta 2 + 15 uplift ridges, seed rank+1",
                   "grid": [W, H], "rounds": ROUNDS, "profile": f"P{args.profile}", "sweeps": cfg.thermal_limits()[1],
                   "parallelism": f"replicas x{world}", "l2": "inputs larger than L2 (134 MB height field)"},
        "e2e": {"value": round(e2e, 3), "unit": UNIT, "h2d_bytes_per_step": 3 * 4 * N, "d2h_bytes_per_step": 4 * N},
        "gpu_launches": int(launches),
        "clocks": clk,
        "roofline": roof,
        "phases_ms_per_step": {k: round(v, 2) for k, v in phase.items()},
        "ms_outside_rounds": round(1000.0 * t_dev / args.steps - phase["ms_total"], 2),
        "rounds": per_round,
    }
    if rank == 0 and world == 1 and args.cpu_sample > 0:
        os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count()))
        v, t, cores, sample = cpu_baseline(W, H, args.cpu_sample, int(os.environ["OMP_NUM_THREADS"]), args.profile)
        line["cpu_baseline"] = {"value": round(v, 3), "unit": UNIT, "cores": cores, "kind": "port", "sample": sample}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    ctx.close()
    return 0


def run_case(args):
    """One public call on the bench world, for a profiler: the thermal sweeps alone
    (GpuErosionAccelerator.erode) or the stage with a few rounds (ErosionStage.apply). Each holds only
    what its call needs on the device, so a profiler that saves and restores device memory around a
    replayed kernel has little to save."""
    from cartogenesis_gb300 import ErosionConfig, ErosionStage, GpuErosionAccelerator
    W, H = args.width, args.height
    h, up, rk = world_inputs(W, H, 1)
    cfg = ErosionConfig(W, H, 1, sea_level=0.70, hydraulic_rounds=args.rounds, profile=args.profile)
    t = time.perf_counter()
    if args.case == "thermal":
        limits, _ = cfg.thermal_limits()
        GpuErosionAccelerator().erode(W, H, h, limits, args.passes, cfg.params.rate)
    else:
        ErosionStage.apply(cfg, h, up, rk, want=("receivers",))
    print(f"case {args.case} {W}x{H}: {time.perf_counter() - t:.3f} s", file=sys.stderr)
    return 0


def run_batched(args):
    """The batched workload: `args.batched` worlds of uneven size through the public batch call
    (ErosionStage.apply_batch -> cg_erode_batch), host inputs and outputs, one batch per step. The
    worlds run one after another inside the call; the line reports the batch's whole throughput."""
    import torch
    from cartogenesis_gb300 import ErosionConfig, ErosionStage, synthetic
    from cartogenesis_gb300.api import default_context
    shapes = synthetic.batch_shapes(args.batched, seed=1)
    worlds = []
    for i, (W, H, seed, radius) in enumerate(shapes):
        h, up, rk = synthetic.world(W, H, seed, uplift="ridges")
        cfg = ErosionConfig(W, H, seed, sea_level=0.70, world_width_km=synthetic.EARTH_KM * radius,
                            profile=args.profile)
        worlds.append((cfg, h, up, rk))
    cells = sum(c.params.width * c.params.height for c, _, _, _ in worlds)
    ctx = default_context()
    for _ in range(args.warmup):
        ErosionStage.apply_batch(worlds, ctx=ctx)
    torch.cuda.synchronize()
    clocks = ClockSampler(0)
    clocks.start()
    launches0 = ctx.kernel_launches
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ErosionStage.apply_batch(worlds, ctx=ctx)
    t = time.perf_counter() - t0
    clk = clocks.stop()
    value = cells * ROUNDS * args.steps / t / 1e6
    sizes = {}
    for c, _, _, _ in worlds:
        key = f"{c.params.width}x{c.params.height}"
        sizes[key] = sizes.get(key, 0) + 1
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(1000.0 * t / args.steps, 1), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"batched plain P{args.profile} stage: {len(worlds)} worlds of radius U(0.25, 2.0) "
                               f"Earth radii, 12 rounds each, host inputs and outputs through cg_erode_batch "
                               f"(worlds one after another in the call)",
                   "worlds": sizes, "cells": cells, "rounds": ROUNDS, "profile": f"P{args.profile}",
                   "l2": "most worlds larger than L2"},
        "e2e": {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": 12 * cells,
                "d2h_bytes_per_step": 4 * cells},
        "gpu_launches": int(ctx.kernel_launches - launches0),
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)
    return 0


def run_belt(args):
    """The belts' replay (BeltErosion.replay) through its public host-buffer call: the world's heights,
    window and factors in, the replayed heights and eroded depths out, every copy inside the timing.
    The unit is Mcell-rounds/s over the belt's cells: belt cells x replayed rounds / seconds. The CPU
    leg runs the oracle's replay of the same world over a window cut to --cpu-sample replayed rounds."""
    import oracle
    from cartogenesis_gb300 import BeltErosion, BeltWindow, ErosionConfig, synthetic
    from cartogenesis_gb300.api import default_context
    W, H, seed = args.width, args.height, 3
    h, up, rk = synthetic.world(W, H, seed)
    t, w, o, win = synthetic.belt_window(W, H, seed)
    cfg = ErosionConfig(W, H, seed)
    window = BeltWindow(t, w, o, win)
    ctx = default_context()
    for _ in range(args.warmup):
        r = BeltErosion.replay(cfg, h.copy(), window, up, None, None, rk, ctx=ctx)
    clocks = ClockSampler(0)
    clocks.start()
    launches0 = ctx.kernel_launches
    t0 = time.perf_counter()
    for _ in range(args.steps):
        r = BeltErosion.replay(cfg, h.copy(), window, up, None, None, rk, ctx=ctx)
    dt = (time.perf_counter() - t0) / args.steps
    clk = clocks.stop()
    units = r.belt_cells * r.rounds
    value = units / dt / 1e6
    cpu = None
    if args.cpu_sample > 0:
        p = oracle.default_params(W, H, seed)
        round_myr = p.years_per_hydraulic_round / 1e6
        short = (ROUNDS + args.cpu_sample + 0.5) * round_myr
        tc = time.perf_counter()
        _, _, b = oracle.belt_replay(p, h, t, w, o, short, uplift=up, rock=rk)
        tc = time.perf_counter() - tc
        cpu = {"value": round(b["belt_cells"] * b["rounds"] / tc / 1e6, 4), "unit": UNIT, "cores": 1, "kind": "port",
               "sample": f"the oracle's replay of the same world over a window of {b['rounds']} replayed rounds"}
    n = W * H
    line = {
        "metric": "belt replay Mcell-rounds/s (belt cells x replayed rounds)", "value": round(value, 3), "unit": UNIT,
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1000.0 * dt, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"BeltErosion.replay over {r.belt_cells} belt cells of the {W}x{H} world, "
                               f"{r.rounds} rounds of a 40 Myr window, through the host-buffer call (value = e2e)",
                   "grid": [W, H], "belt_cells": r.belt_cells, "rounds": r.rounds, "l2": "the world's fields exceed L2"
                   if n * 4 > 129e6 else "fits L2"},
        "e2e": {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": 4 * n * 6, "d2h_bytes_per_step": 8 * n},
        "gpu_launches": int(ctx.kernel_launches - launches0),
        "clocks": clk,
        "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    if args.case:
        return run_case(args)
    if args.belt:
        return run_belt(args)
    if args.batched:
        return run_batched(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
