"""swe_batch_erode: an ensemble of independent worlds (their own sizes,
seeds, winds and parameters) eroded together must leave every world exactly
as eroding it alone does (fields bit for bit, mass ledger, tallies), both for
the worlds that share the persistent cluster launch and for a world with too
many particles in flight for one cluster, which runs on its own stream."""
import numpy as np
import pytest

import simplewinderosion_gb300 as swe
from simplewinderosion_gb300 import terrain
from tests.conftest import WIND_101, bits

pytestmark = pytest.mark.gpu

# (nx, nz, particles, wind, frac_bits, lanes, seed)
ENSEMBLE = [
    (48, 48, 3000, WIND_101, 24, 0, 3),
    (64, 40, 2500, (0.0, 0.0, -1.0), 16, 37, 4),
    (96, 96, 9000, (1.0, 0.0, 0.0), 24, 2048, 5),
    (33, 70, 1200, swe.wind_direction(-1.0, 0.0, 2.0), 20, 0, 6),
    (128, 128, 16384, WIND_101, 16, 0, 7),
    (128, 128, 16384, (0.0, 0.0, -1.0), 16, -1, 9),  # 16,384 in flight: four lanes a thread in the cluster
    (160, 96, 20000, (0.0, 0.0, 1.0), 24, -1, 8),  # 20,000 in flight: its own launch
]


def _world(nx, nz, wind, frac_bits, lanes, seed):
    h = (terrain.normalise(terrain.fbm(nx, nz, seed, 4.0 / max(nx, nz))) + 0.1).astype(np.float32)
    w = swe.World(nx, nz, params=swe.Params(pspeed=wind, frac_bits=frac_bits, lanes=lanes), seed=100 + seed)
    w.upload(swe.Field.HEIGHT, h)
    return w


def test_batch_equals_worlds_eroded_alone():
    cycles = 2
    batch = [_world(nx, nz, wind, fb, lanes, sd) for nx, nz, _, wind, fb, lanes, sd in ENSEMBLE]
    alone = [_world(nx, nz, wind, fb, lanes, sd) for nx, nz, _, wind, fb, lanes, sd in ENSEMBLE]
    particles = [e[2] for e in ENSEMBLE]
    swe.batch_erode(batch, cycles, particles)
    for w, p in zip(alone, particles):
        w.erode(p, cycles, mode=swe.Mode.PARALLEL)
    for k, (a, b) in enumerate(zip(batch, alone)):
        for f in swe.FIELDS:
            assert np.array_equal(bits(a.download(f)), bits(b.download(f))), (k, f)
        assert a.mass_ledger() == b.mass_ledger(), k
        assert a.stats() == b.stats(), k
        assert a.status() == 0
    # a second batch call continues from where the first left every world
    swe.batch_erode(batch[:3], 1, particles[:3])
    for w, p in zip(alone[:3], particles[:3]):
        w.erode(p, 1, mode=swe.Mode.PARALLEL)
    for k in range(3):
        assert np.array_equal(bits(batch[k].height), bits(alone[k].height)), k
    for w in batch + alone:
        w.close()


def test_batch_rejects_a_world_twice():
    w = _world(32, 32, WIND_101, 24, 0, 1)
    with pytest.raises(swe.SweError) as e:
        swe.batch_erode([w, w], 1, 100)
    assert e.value.code == -1
    w.close()


# the worlds of ENSEMBLE that fit a 4-CTA cluster of 128 threads (at most 2,048 in flight)
SMALL = ENSEMBLE[:5]


@pytest.mark.parametrize("ctas,threads", [(16, 256), (8, 128), (4, 256), (4, 128)])
def test_prepared_batch_any_shape_equals_worlds_alone(ctas, threads):
    cycles = 2
    batch = [_world(nx, nz, wind, fb, lanes, sd) for nx, nz, _, wind, fb, lanes, sd in SMALL]
    alone = [_world(nx, nz, wind, fb, lanes, sd) for nx, nz, _, wind, fb, lanes, sd in SMALL]
    particles = [e[2] for e in SMALL]
    b = swe.Batch(batch, particles)
    b.set_shape(ctas, threads)
    assert b.shape()["ctas_per_cluster"] == ctas and b.shape()["threads_per_cta"] == threads
    b.run(cycles)
    for w, p in zip(alone, particles):
        w.erode(p, cycles, mode=swe.Mode.PARALLEL)
    for k, (a, c) in enumerate(zip(batch, alone)):
        a.sync()
        for f in swe.FIELDS:
            assert np.array_equal(bits(a.download(f)), bits(c.download(f))), (ctas, threads, k, f)
        assert a.mass_ledger() == c.mass_ledger(), k
    b.close()
    for w in batch + alone:
        w.close()


def test_autotuned_batch_equals_worlds_alone():
    batch = [_world(nx, nz, wind, fb, lanes, sd) for nx, nz, _, wind, fb, lanes, sd in ENSEMBLE[:6]]
    alone = [_world(nx, nz, wind, fb, lanes, sd) for nx, nz, _, wind, fb, lanes, sd in ENSEMBLE[:6]]
    particles = [e[2] for e in ENSEMBLE[:6]]
    b = swe.Batch(batch, particles, tune=True)
    shape = b.shape()
    assert shape["tuned_ms"] > 0 and shape["default_ms"] > 0
    assert shape["tuned_ms"] <= shape["default_ms"]
    b.run(1)
    for w, p in zip(alone, particles):
        w.erode(p, 1, mode=swe.Mode.PARALLEL)
    for k, (a, c) in enumerate(zip(batch, alone)):
        a.sync()
        for f in swe.FIELDS:
            assert np.array_equal(bits(a.download(f)), bits(c.download(f))), (shape, k, f)
    # the same signature again: the cached shape, no measurement
    b2 = swe.Batch(batch, particles, tune=True)
    assert b2.shape()["ctas_per_cluster"] == shape["ctas_per_cluster"]
    assert b2.shape()["threads_per_cta"] == shape["threads_per_cta"]
    b.close()
    b2.close()
    for w in batch + alone:
        w.close()


def test_prepared_batch_refuses_a_world_too_large_for_a_cluster():
    w = _world(160, 96, (0.0, 0.0, 1.0), 24, -1, 8)
    with pytest.raises(swe.SweError) as e:
        swe.Batch([w], [20000])
    assert e.value.code == -1
    w.close()
