"""Check (c) at exactly the benchmarked configuration: the parallel GPU mode
at 1024^2, 1,048,576 particles per cycle, int32 Q16.16 heights and the
default particles in flight (cells/256 = 4,096), against the reference's own
sequential World::erode (source/world.hpp:36-77).

The reference side is the committed fixture tests/golden/stats_1024_plain.npz
(tests/golden/make_stats_1024.py): the compiled reference eroded the same
terrain (the 1024^2 plain-method configuration: fBm 1/256 + 0.1 +- 0.02
sediment + a 0.4/200 pyramid), wind normalize(1,0,1), 1,048,576 particles per
cycle, with six rand() seeds, and the fixture keeps each run's height
quantile profile, log radial spectrum and mean after every cycle. The spread
of the six runs (the largest distance of seeds 2-6 from seed 1) is the noise
floor. After every cycle the GPU run must stay
within 2.5x that floor in the 1-Wasserstein distance of the height
histograms, the log-spectrum distance and the mean height, and its mass
ledger must balance exactly.
"""
import hashlib

import numpy as np
import pytest

import simplewinderosion_gb300 as swe
from simplewinderosion_gb300 import terrain
from tests.conftest import golden
from tests.statistics_check import floors, gpu_distances

pytestmark = pytest.mark.gpu

BOUND = 2.5


def test_bench_configuration_statistics_match_reference():
    fx = golden("stats_1024_plain")
    n, particles, cycles = int(fx["n"]), int(fx["particles"]), int(fx["cycles"])
    assert (n, particles) == (1024, 1048576)
    h = terrain.config_plain_large(seed=int(fx["terrain_seed"]), n=n)
    assert hashlib.sha256(np.ascontiguousarray(h, np.float32).tobytes()).hexdigest() == str(fx["height0_sha256"])
    prof, spec, mean = fx["profile"], fx["logspec"], fx["mean"]
    wind = tuple(float(v) for v in fx["pspeed"])

    # the benchmark's settings: Q16.16, default lanes
    w = swe.World(n, params=swe.Params(pspeed=wind, frac_bits=16, lanes=0), seed=11)
    w.upload(swe.Field.HEIGHT, h)
    m0, _, _ = w.mass_ledger()
    for c in range(cycles):
        w.erode(particles, 1, mode=swe.Mode.PARALLEL)
        gw, gs, gm = gpu_distances(w.height, prof, spec, mean, c)
        nw, ns, nm = floors(prof, spec, mean, c)
        print(f"cycle {c + 1}: W1 {gw:.6f} / floor {nw:.6f} = {gw / nw:.2f}x; spectrum {gs:.5f} / {ns:.5f} = "
              f"{gs / ns:.2f}x; mean {gm:.6f} / {nm:.6f}")
        assert gw <= BOUND * nw, (c, gw, nw)
        assert gs <= BOUND * ns, (c, gs, ns)
        assert gm <= BOUND * max(nm, 1e-4), (c, gm, nm)
    m, inflight, e = w.mass_ledger()
    assert inflight == 0 and m + e == m0
    w.close()

