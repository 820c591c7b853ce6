"""Statistics of the parallel mode against the sequential reference at a
chosen size, as a command (minutes of CPU time at 1024^2, so not a pytest
test; tests/test_gpu_statistics.py is the 256^2 test).

    python -m tests.statistics_check N P C LANES[,LANES...]

The reference semantics (the oracle port, bit-identical to the compiled
reference) erode the map C cycles x P particles with three rand() seeds;
their spread is the noise floor. The GPU parallel mode then runs the same map
for each LANES value (0: the default, -1: all at once) and prints the
1-Wasserstein distance between height histograms, the RMS distance between
log radially averaged power spectra, and the mean-height difference, each
also as a multiple of the noise floor. Terrain: the 256^2-style fBm +
sediment below 1024^2, the 1024^2 config (fBm 1/256 + sediment + pyramid)
at 1024^2 and above.
"""
import sys
import time

import numpy as np

import simplewinderosion_gb300 as swe
from oracle import oracle
from simplewinderosion_gb300 import terrain
from tests.conftest import WIND_101
from tests.test_gpu_statistics import spec_dist, w1


def main(argv):
    n, particles, cycles = int(argv[0]), int(argv[1]), int(argv[2])
    lanes_list = [int(v) for v in argv[3].split(",")] if len(argv) > 3 else [0]
    h = terrain.config_plain_small(seed=1, n=n) if n < 1024 else terrain.config_plain_large(seed=2, n=n)
    t0 = time.time()
    seq = []
    for seed in (1, 2, 3):
        p = oracle.Port(n, pspeed=WIND_101)
        p.set_field(0, h)
        p.seed(seed)
        p.erode(particles, cycles)
        seq.append(p.get_field(0))
    a, b, c = seq
    nw = max(w1(b, a), w1(c, a))
    ns = max(spec_dist(b, a), spec_dist(c, a))
    nm = max(abs(b.mean() - a.mean()), abs(c.mean() - a.mean()))
    print(f"{n}^2, {particles} particles x {cycles} cycles; reference runs {time.time() - t0:.0f} s")
    print(f"noise floor: W1 {nw:.5f}  spectrum {ns:.4f}  mean {nm:.5f}")
    for lanes in lanes_list:
        w = swe.World(n, params=swe.Params(pspeed=WIND_101, frac_bits=24, lanes=lanes), seed=11)
        w.upload(swe.Field.HEIGHT, h)
        w.erode(particles, cycles, mode=swe.Mode.PARALLEL)
        g = w.height
        gw, gs, gm = w1(g, a), spec_dist(g, a), abs(g.mean() - a.mean())
        print(f"lanes {lanes:>7}: W1 {gw:.5f} ({gw / nw:.2f}x)  spectrum {gs:.4f} ({gs / ns:.2f}x)  "
              f"mean {gm:.5f}")
        w.close()


if __name__ == "__main__":
    main(sys.argv[1:])
