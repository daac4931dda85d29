"""One public call of the library on a seeded synthetic world, for profiling its kernels.

    python -m cartogenesis_gb300.kernel_cases thermal --width 8192 --height 4096 --passes 4
    python -m cartogenesis_gb300.kernel_cases stage --width 4096 --height 2048 --rounds 2

`thermal` runs GpuErosionAccelerator.erode (the ErosionAccelerator sweeps) once; `stage` runs
ErosionStage.apply once with the given number of hydraulic rounds. Each allocates only what its
call needs (a few fields of the grid), so a profiler that replays a captured kernel many times,
saving and restoring device memory around each pass, has little to save. The world is the
benchmark's generator (fBm heights, ridge uplift, rock erodibility) at the given size.
"""
import argparse
import time

from . import synthetic
from .api import ErosionConfig, ErosionStage, GpuErosionAccelerator


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("case", choices=("thermal", "stage"))
    ap.add_argument("--width", type=int, default=8192)
    ap.add_argument("--height", type=int, default=4096)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--passes", type=int, default=4, help="thermal: sweeps")
    ap.add_argument("--rounds", type=int, default=2, help="stage: hydraulic rounds")
    args = ap.parse_args(argv)
    W, H = args.width, args.height
    h, up, rk = synthetic.world(W, H, args.seed, uplift="ridges")
    cfg = ErosionConfig(W, H, args.seed, sea_level=0.70, hydraulic_rounds=args.rounds)
    t = time.perf_counter()
    if args.case == "thermal":
        limits, _ = cfg.thermal_limits()
        out = GpuErosionAccelerator().erode(W, H, h, limits, args.passes, cfg.params.rate)
        summary = f"mean height {float(out.mean()):.4f}"
    else:
        r = ErosionStage.apply(cfg, h, up, rk, want=("receivers",))
        summary = f"land cells {r.stats[-1]['land_cells']}, flats {r.stats[-1]['flats']}"
    print(f"{args.case} {W}x{H}: {time.perf_counter() - t:.3f} s, {summary}")


if __name__ == "__main__":
    main()
