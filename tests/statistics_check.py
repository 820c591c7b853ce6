"""Statistics of the parallel mode against the sequential reference, as a
command (minutes of CPU time at 1024^2 when the reference runs here, so not a
pytest test; tests/test_gpu_statistics.py and
tests/test_gpu_statistics_1024.py are the tests).

    python -m tests.statistics_check N P C LANES[,LANES...] [--frac-bits F] [--seed S]
    python -m tests.statistics_check --fixture stats_1024_plain LANES[,LANES...] [--frac-bits F]

First form: the reference semantics (the oracle port, bit-identical to the
compiled reference) erode the map C cycles x P particles with three rand()
seeds; their spread is the noise floor. Second form: the same statistics of
the reference runs are read from a committed fixture (tests/golden/, made by
tests/golden/make_stats_1024.py from the compiled reference). The GPU
parallel mode then runs the same map for each LANES value (0: the default,
-1: all at once) and prints, after every cycle, the 1-Wasserstein distance
between height histograms, the RMS distance between log radially averaged
power spectra, and the mean-height difference, each also as a multiple of
the noise floor. Terrain: the 256^2-style fBm + sediment below 1024^2, the
1024^2 config (fBm 1/256 + sediment + pyramid) at 1024^2 and above.
"""
import argparse
import time

import numpy as np

import simplewinderosion_gb300 as swe
from simplewinderosion_gb300 import terrain
from tests import terrain_stats as ts
from tests.conftest import WIND_101, golden


def reference_summaries(n, particles, cycles):
    """[seed][cycle] summaries of three reference-semantics runs (oracle port)."""
    from oracle import oracle
    h = terrain.config_plain_small(seed=1, n=n) if n < 1024 else terrain.config_plain_large(seed=2, n=n)
    out = []
    for seed in (1, 2, 3):
        p = oracle.Port(n, pspeed=WIND_101)
        p.set_field(0, h)
        p.seed(seed)
        runs = []
        for _ in range(cycles):
            p.erode(particles, 1)
            runs.append(ts.summary(p.get_field(0)))
        out.append(runs)
    prof = np.array([[c["profile"] for c in r] for r in out])
    spec = np.array([[c["logspec"] for c in r] for r in out])
    mean = np.array([[c["mean"] for c in r] for r in out])
    return h, prof, spec, mean


def floors(prof, spec, mean, c):
    """Noise floor at cycle index c: the largest distance of the other
    reference seeds' runs from the first seed's."""
    others = range(1, prof.shape[0])
    nw = max(ts.w1_profiles(prof[k, c], prof[0, c]) for k in others)
    ns = max(ts.spec_dist_logs(spec[k, c], spec[0, c]) for k in others)
    nm = max(abs(mean[k, c] - mean[0, c]) for k in others)
    return nw, ns, nm


def gpu_distances(g, prof, spec, mean, c):
    s = ts.summary(g)
    return (ts.w1_profiles(s["profile"], prof[0, c]), ts.spec_dist_logs(s["logspec"], spec[0, c]),
            abs(s["mean"] - mean[0, c]))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("args", nargs="+")
    ap.add_argument("--fixture", default=None)
    ap.add_argument("--frac-bits", type=int, default=24)
    ap.add_argument("--seed", type=int, default=11)
    a = ap.parse_args()
    t0 = time.time()
    if a.fixture:
        fx = golden(a.fixture)
        n, particles, cycles = int(fx["n"]), int(fx["particles"]), int(fx["cycles"])
        h = terrain.config_plain_large(seed=int(fx["terrain_seed"]), n=n)
        prof, spec, mean = fx["profile"], fx["logspec"], fx["mean"]
        lanes_list = [int(v) for v in a.args[0].split(",")]
    else:
        n, particles, cycles = int(a.args[0]), int(a.args[1]), int(a.args[2])
        lanes_list = [int(v) for v in a.args[3].split(",")] if len(a.args) > 3 else [0]
        h, prof, spec, mean = reference_summaries(n, particles, cycles)
    print(f"{n}^2, {particles} particles x {cycles} cycles, Q{32 - a.frac_bits}.{a.frac_bits}; "
          f"reference statistics in {time.time() - t0:.0f} s")
    for c in range(cycles):
        nw, ns, nm = floors(prof, spec, mean, c)
        print(f"cycle {c + 1} noise floor: W1 {nw:.6f}  spectrum {ns:.5f}  mean {nm:.6f}")
    for lanes in lanes_list:
        w = swe.World(n, params=swe.Params(pspeed=WIND_101, frac_bits=a.frac_bits, lanes=lanes), seed=a.seed)
        w.upload(swe.Field.HEIGHT, h)
        m0, _, _ = w.mass_ledger()
        for c in range(cycles):
            t1 = time.time()
            w.erode(particles, 1, mode=swe.Mode.PARALLEL)
            dt = time.time() - t1
            g = w.height
            gw, gs, gm = gpu_distances(g, prof, spec, mean, c)
            nw, ns, nm = floors(prof, spec, mean, c)
            signed = float(np.mean(g, dtype=np.float64)) - float(mean[:, c].mean())
            print(f"lanes {lanes:>8} cycle {c + 1}: W1 {gw:.6f} ({gw / nw:.2f}x)  spectrum {gs:.5f} "
                  f"({gs / ns:.2f}x)  mean {gm:.6f} ({gm / max(nm, 1e-12):.2f}x, GPU - reference average "
                  f"{signed:+.6f})  [{dt * 1e3:.0f} ms]")
        m, inflight, e = w.mass_ledger()
        print(f"lanes {lanes:>8}: ledger map+exported-initial = {m + e - m0} (0 = exact)")
        w.close()


if __name__ == "__main__":
    main()
