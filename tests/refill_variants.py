"""Which particles fly together, as a command (CPU only, about a minute at
256^2): the parallel model (the oracle port's so_par_erode) with the
library's rule (freed lanes take the cycle's next ids), with lanes taking
their own id sequences (k, k + L, ...), and with a fixed spawn schedule
(particle j spawning at step floor(400 j / L), L in flight on average),
against the reference semantics with three rand() seeds as the noise floor;
and the largest one-step move of any particle along x or z (the reach from
which a cell's visitors come).

    python -m tests.refill_variants [N] [P] [C]
    python -m tests.refill_variants --fixture stats_1024_plain [SEEDS]   # 1024^2, minutes per run

The second form takes the reference's statistics from the committed fixture
of compiled-reference runs (the benchmark configuration) instead of running
the reference semantics here.

Prints, per variant and model seed, the worst cycle's 1-Wasserstein
distance of the height histograms, log-spectrum distance and mean-height
difference as multiples of the noise floor, and the largest move.
"""
import json
import sys

import numpy as np

from tests import terrain_stats as ts
from tests.conftest import WIND_101
from tests.statistics_check import floors, reference_summaries


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    from oracle import oracle
    if argv[:1] == ["--fixture"]:
        from simplewinderosion_gb300 import terrain
        from tests.conftest import golden
        fx = golden(argv[1])
        n, particles, cycles = int(fx["n"]), int(fx["particles"]), int(fx["cycles"])
        h = terrain.config_plain_large(seed=int(fx["terrain_seed"]), n=n)
        prof, spec, mean = fx["profile"], fx["logspec"], fx["mean"]
        modes = (0, 2)
        seeds = tuple(int(v) for v in argv[2].split(",")) if len(argv) > 2 else (5,)
    else:
        n = int(argv[0]) if len(argv) > 0 else 256
        particles = int(argv[1]) if len(argv) > 1 else 16384
        cycles = int(argv[2]) if len(argv) > 2 else 10
        h, prof, spec, mean = reference_summaries(n, particles, cycles)
        modes, seeds = (0, 1, 2), (5, 6)
    names = {0: "library rule", 1: "own id sequences", 2: "fixed spawn schedule"}
    for mode in modes:
        for seed in seeds:
            p = oracle.Port(n, pspeed=WIND_101, frac_bits=16, lanes=0)
            p.par_spawn_mode(mode)
            p.set_field(0, h)
            cyc, worst, move = 0, np.zeros(3), 0.0
            for c in range(cycles):
                cyc = p.par_erode(particles, 1, seed=seed, cycle=cyc)
                move = max(move, p.par_max_move())
                s = ts.summary(p.get_field(0))
                nw, ns, nm = floors(prof, spec, mean, c)
                d = np.array([ts.w1_profiles(s["profile"], prof[0, c]) / nw,
                              ts.spec_dist_logs(s["logspec"], spec[0, c]) / ns,
                              abs(s["mean"] - mean[0, c]) / max(nm, 1e-4)])
                worst = np.maximum(worst, d)
            print(json.dumps({"variant": names[mode], "seed": seed, "worst_w1_spectrum_mean": worst.round(2).tolist(),
                              "max_move_cells": round(move, 4)}), flush=True)


if __name__ == "__main__":
    main()
