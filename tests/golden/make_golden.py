"""Generate the golden fixtures in tests/golden/ from the REFERENCE ITSELF.

The reference's World::erode / Wind::fly / World::cascade / quad::_normal
(source/world.hpp, source/wind.hpp, source/cellpool.h) are compiled from their
own sources by oracle/Makefile (oracle/_ref/libswe_ref_<N>.so, with the glm
shim in oracle/glm_shim.hpp), then run on small seeded cases. The outputs are
stored as .npz so machines without the reference sources (the GPU machine) can
check the oracle port and the CUDA kernels against the reference's own
results.

Run from the repository root:  python tests/golden/make_golden.py [--only-new]
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import oracle  # noqa: E402
from simplewinderosion_gb300 import terrain  # noqa: E402

OUT = Path(__file__).resolve().parent
WIND_101 = (0.70710677, 0.0, 0.70710677)  # glm::normalize(vec3(1,0,1)) in float


def fields(ref) -> np.ndarray:
    return np.stack([ref.get_field(f) for f in range(9)])


def erode_case(name, n, seed_terrain, seed_rand, particles, cycles, pspeed=None):
    ref = oracle.Reference(n)
    h0 = terrain.normalise(terrain.fbm(n, n, seed_terrain, 4.0 / n)).astype(np.float32) + np.float32(0.1)
    ref.reset(h0)
    ref.srand(seed_rand)
    calls0 = ref.L.ref_rand_calls()
    ref.erode(particles, cycles, pspeed=pspeed)
    calls = ref.L.ref_rand_calls() - calls0
    np.savez_compressed(OUT / f"{name}.npz", height0=h0, fields=fields(ref), n=n, seed=seed_rand,
                        particles=particles, cycles=cycles,
                        pspeed=np.asarray(pspeed if pspeed else (1.0, 0.0, 0.0), np.float32), rand_calls=calls)


def normals_case(name, n, seed):
    ref = oracle.Reference(n)
    rs = np.random.RandomState(seed)
    h = rs.uniform(0, 0.5, size=(n, n)).astype(np.float32)
    h[: n // 3, : n // 3] = 0.25  # flat patch
    h[n // 2:, :] += 0.3          # cliff
    ref.reset(h)
    np.savez_compressed(OUT / f"{name}.npz", height=h, normals=ref.normals())


def cascade_case(name, n, seed):
    ref = oracle.Reference(n)
    rs = np.random.RandomState(seed)
    h = rs.uniform(0, 0.05, size=(n, n)).astype(np.float32)
    h[3, :] = 0.02                      # ties along a row
    h[5, 5] = 0.5                       # spike
    h[n - 1, n - 1] = 0.3               # corner
    h[0, 4] = -0.2                      # edge pit
    ref.reset(h)
    cells = [(5, 5), (3, 3), (0, 0), (n - 1, n - 1), (0, 4), (n - 1, 2), (3, 4), (6, 6), (5, 5), (2, n - 1)]
    cells += [tuple(c) for c in rs.randint(0, n, size=(30, 2))]
    after = []
    for (x, z) in cells:
        ref.cascade(int(x), int(z))
        after.append(ref.get_field(0))
    np.savez_compressed(OUT / f"{name}.npz", height=h, cells=np.asarray(cells, np.int32), after=np.stack(after))


def cascade_ties_case(name, n, seed):
    """World::cascade on a map full of exact ties (quantised heights, +0 and
    -0) with two NaN cells, at interior, edge and corner cells, next to the
    NaNs and away from them."""
    ref = oracle.Reference(n)
    rs = np.random.RandomState(seed)
    levels = np.asarray([0.0, -0.0, 0.05, 0.1, 0.1, 0.2], np.float32)
    h = levels[rs.randint(0, len(levels), size=(n, n))].astype(np.float32)
    h[4:7, 4:7] = 0.1                   # a plateau: eight equal neighbours
    h[5, 5] = 0.3
    h[9, 9] = np.float32(np.nan)        # interior NaN
    h[0, 11] = np.float32(np.nan)       # edge NaN
    ref.reset(h)
    cells = [(5, 5), (4, 4), (8, 8), (9, 10), (10, 10), (1, 11), (0, 10), (0, 0), (n - 1, n - 1), (0, n - 1),
             (5, 5), (12, 3), (9, 9)]
    cells += [tuple(c) for c in rs.randint(0, n, size=(40, 2))]
    after = []
    for (x, z) in cells:
        ref.cascade(int(x), int(z))
        after.append(ref.get_field(0))
    np.savez_compressed(OUT / f"{name}.npz", height=h, cells=np.asarray(cells, np.int32), after=np.stack(after))


def trace_tape(seed, count, steps):
    """Raw rand()-like turbulence draws for frozen-map traces (regenerated
    from the seed by the tests; numpy's legacy RandomState stream is fixed)."""
    return np.random.RandomState(seed + 1000).randint(0, 2**31 - 1, size=(count, steps, 3)).astype(np.int32)


def trace_case(name, n, seed, count, steps, pspeed):
    ref = oracle.Reference(n)
    rs = np.random.RandomState(seed)
    h = (terrain.normalise(terrain.fbm(n, n, seed, 6.0 / n)) + 0.05).astype(np.float32)
    ref.reset(h)
    spawn = np.stack([rs.randint(0, n, count) + rs.randint(0, 1000, count) / np.float32(1000.0),
                      rs.randint(0, n, count) + rs.randint(0, 1000, count) / np.float32(1000.0)], 1)
    spawn = spawn.astype(np.float32)
    tape = trace_tape(seed, count, steps)
    rec = ref.trace(spawn, steps, tape, pspeed=pspeed)
    np.savez_compressed(OUT / f"{name}.npz", height=h, spawn=spawn, tape_seed=seed, records=rec,
                        pspeed=np.asarray(pspeed, np.float32))


def map_init_case(name, n):
    """quad::map::init's own terrain (the Gaussian bump normalised to [0, 0.5],
    cellpool.h:339-430), from the compiled reference."""
    ref = oracle.Reference(n)
    np.savez_compressed(OUT / f"{name}.npz", height=ref.map_init(0), n=n)


def vertices_case(name, n, seed):
    """updatenode's vertex data (cellpool.h:302-333: position, normal, +x and
    +z edges per cell) on a map with random heights, a flat patch and a
    cliff, captured from the compiled reference's own updatenode."""
    ref = oracle.Reference(n)
    rs = np.random.RandomState(seed)
    h = rs.uniform(0, 0.5, size=(n, n)).astype(np.float32)
    h[: n // 3, : n // 3] = 0.25
    h[n // 2:, :] += 0.3
    ref.reset(h)
    np.savez_compressed(OUT / f"{name}.npz", height=h, vertices=ref.vertices())


def rand_case(name):
    ref = oracle.Reference(8)
    seeds = [0, 1, 7, 12345, 2**31 + 5, 4294967295]
    seqs = []
    for s in seeds:
        ref.srand(s)
        a = np.empty(2000, dtype=np.int32)
        ref.L.ref_rand_sequence(2000, oracle._ptr(a))
        seqs.append(a)
    np.savez_compressed(OUT / f"{name}.npz", seeds=np.asarray(seeds, np.uint64), seqs=np.stack(seqs),
                        order=ref.probe_order())


def main(argv):
    oracle.build_reference(sizes=(8, 16, 32, 48, 64))
    map_init_case("map_init_48", 48)
    vertices_case("vertices_16", 16, 31)
    if "--only-new" in argv:
        return
    rand_case("rand_sequences")
    erode_case("erode_32_default", 32, 11, 5, 40, 4)
    erode_case("erode_64_wind101", 64, 12, 99, 120, 3, pspeed=WIND_101)
    erode_case("erode_16_edges", 16, 13, 3, 60, 5, pspeed=(0.0, 0.0, -1.0))
    normals_case("normals_16", 16, 21)
    cascade_case("cascade_12", 16, 22)
    cascade_ties_case("cascade_ties_nan", 16, 25)
    trace_case("trace_48_wind101", 48, 23, 32, 128, WIND_101)
    trace_case("trace_48_default", 48, 24, 32, 128, (1.0, 0.0, 0.0))
    for p in sorted(OUT.glob("*.npz")):
        print(p.name, p.stat().st_size)


if __name__ == "__main__":
    main(sys.argv[1:])
