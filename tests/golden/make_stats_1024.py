"""Generate tests/golden/stats_1024_plain.npz: terrain statistics of the
REFERENCE's sequential World::erode (source/world.hpp:36-77) on the benchmark
workload, so the GPU's parallel mode can be checked statistically at exactly
the settings it is benchmarked at (tests/test_gpu_statistics_1024.py).

Workload: the 1024^2 plain-method terrain (terrain.config_plain_large, seed
2: fBm base frequency 1/256 + 0.1 +- 0.02 sediment + a 0.4/200 pyramid),
wind normalize(1,0,1), 1,048,576 particles per cycle, CYCLES cycles, once
per rand() seed (1 to 6; the spread of the six runs is the noise floor).
For every seed and cycle the file keeps the height map's quantile profile,
log radial spectrum and mean (tests/terrain_stats.py), and a checksum of the
initial heights.

The reference's own headers are compiled by oracle/Makefile for a 1024^2 map
(oracle/_ref/libswe_ref_1024.so); where the sources are absent the oracle
port runs instead (bit-identical, tests/test_oracle_vs_reference.py) and the
file records which. One process per seed (the reference keeps its map in
statics); about 3.5 minutes of one core per cycle for the compiled reference.

    python tests/golden/make_stats_1024.py [CYCLES]
"""
from __future__ import annotations

import hashlib
import multiprocessing as mp
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

OUT = Path(__file__).resolve().parent / "stats_1024_plain.npz"
N, P, TERRAIN_SEED, SEEDS = 1024, 1048576, 2, (1, 2, 3, 4, 5, 6)
WIND_101 = (0.70710677, 0.0, 0.70710677)  # glm::normalize(vec3(1,0,1)) in float


def initial_heights() -> np.ndarray:
    from simplewinderosion_gb300 import terrain
    return terrain.config_plain_large(seed=TERRAIN_SEED, n=N)


def heights_digest(h) -> str:
    return hashlib.sha256(np.ascontiguousarray(h, np.float32).tobytes()).hexdigest()


def run_seed(args):
    seed, cycles = args
    sys.path.insert(0, str(ROOT))
    from oracle import oracle
    from tests import terrain_stats as ts
    h = initial_heights()
    if oracle.reference_available():
        r = oracle.Reference(N)
        r.reset(h)
        r.srand(seed)
        kind = "reference"

        def step():
            r.erode(P, 1, pspeed=WIND_101)
        get = lambda: r.get_field(0)  # noqa: E731
    else:
        p = oracle.Port(N, pspeed=WIND_101)
        p.set_field(0, h)
        p.seed(seed)
        kind = "port"

        def step():
            p.erode(P, 1)
        get = lambda: p.get_field(0)  # noqa: E731
    out = []
    for c in range(cycles):
        t0 = time.time()
        step()
        out.append(ts.summary(get()))
        print(f"seed {seed} cycle {c + 1}: {time.time() - t0:.0f} s", flush=True)
    return kind, out


def main(argv):
    cycles = int(argv[0]) if argv else 3
    from oracle import oracle
    if oracle.reference_available():
        oracle.build_reference(sizes=(N,))
    h = initial_heights()
    ctx = mp.get_context("spawn")
    with ctx.Pool(len(SEEDS)) as pool:
        res = pool.map(run_seed, [(s, cycles) for s in SEEDS])
    kinds = {k for k, _ in res}
    assert len(kinds) == 1
    prof = np.stack([[c["profile"] for c in runs] for _, runs in res]).astype(np.float64)
    spec = np.stack([[c["logspec"] for c in runs] for _, runs in res]).astype(np.float64)
    mean = np.array([[c["mean"] for c in runs] for _, runs in res], np.float64)
    np.savez_compressed(OUT, profile=prof, logspec=spec, mean=mean, n=N, particles=P, cycles=cycles,
                        seeds=np.asarray(SEEDS), terrain_seed=TERRAIN_SEED, pspeed=np.asarray(WIND_101, np.float32),
                        source=kinds.pop(), height0_sha256=heights_digest(h))
    print(f"wrote {OUT}")


if __name__ == "__main__":
    main(sys.argv[1:])
