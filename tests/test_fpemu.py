"""The exact sequential-sum emulation the device histogram relies on (csrc/cg_fpemu.h), checked on
the CPU against a plain loop of double additions, bit for bit, on random and adversarial cases
(ties at half an ulp, binade crossings, terms far below and far above the running sum)."""
import os
import subprocess
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

HARNESS = r"""
#include <cstdio>
#include <cstdint>
#include <cstring>
#include "cg_fpemu.h"
int main() {
    double s, w; long long c;
    while (std::scanf("%la %la %lld", &s, &w, &c) == 3) {
        double naive = s;
        for (long long i = 0; i < c; ++i) naive += w;
        double fast = cg::seq_repeat_add(s, w, c);
        uint64_t a, b; std::memcpy(&a, &naive, 8); std::memcpy(&b, &fast, 8);
        std::printf("%d\n", a == b ? 1 : 0);
    }
}
"""


def test_seq_repeat_add_matches_a_plain_loop():
    rng = np.random.default_rng(5)
    cases = []
    for _ in range(3000):
        kind = rng.integers(0, 5)
        if kind == 0:
            s, w = 0.0, float(rng.uniform(1e-3, 1.0))
        elif kind == 1:
            s, w = float(rng.uniform(0, 1e4)), float(rng.uniform(1e-3, 1.0))
        elif kind == 2:   # ties: w a short binary fraction against a sum a few binades up
            s = float(np.ldexp(rng.integers(1, 1 << 20), int(rng.integers(-10, 10))))
            w = float(np.ldexp(rng.integers(1, 64) * 2 + 1, int(rng.integers(-20, 0))))
        elif kind == 3:   # sin() row weights, as the cut adds
            H = int(rng.choice([64, 256, 1024, 4096]))
            row = int(rng.integers(0, H))
            w = float(np.cos(np.pi / 2 - (row + 0.5) / H * np.pi))
            s = float(rng.uniform(0, 2e5))
        else:             # term far above the sum
            s, w = float(rng.uniform(0, 1e-6)), float(rng.uniform(1, 10))
        c = int(rng.integers(0, 3000))
        cases.append((s, w, c))
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "h.cpp")
        exe = os.path.join(d, "h")
        with open(src, "w") as f:
            f.write(HARNESS)
        subprocess.check_call(["g++", "-O2", "-ffp-contract=off", "-std=c++17", "-I",
                               os.path.join(ROOT, "cartogenesis_gb300", "csrc"), src, "-o", exe])
        text = "\n".join(f"{float(s).hex()} {float(w).hex()} {c}" for s, w, c in cases)
        out = subprocess.run([exe], input=text, capture_output=True, text=True, check=True).stdout.split()
    bad = [cases[i] for i, v in enumerate(out) if v != "1"]
    assert len(out) == len(cases)
    assert not bad, bad[:5]
