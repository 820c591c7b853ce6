"""swe_batch_erode_ordered: an ensemble of ORDERED worlds (their own sizes,
rand() seeds or tapes, winds and particle counts), one GPU thread per world,
must leave every world bit for bit as eroding it alone in ORDERED mode does
(which the exact-mode tests pin to the reference's World::erode), and one of
them is checked against the oracle port directly. The large case packs more
than one world per warp."""
import numpy as np
import pytest

import simplewinderosion_gb300 as swe
from oracle import oracle
from simplewinderosion_gb300 import terrain
from tests.conftest import WIND_101, bits

pytestmark = pytest.mark.gpu

# (nx, nz, particles, wind, rand seed)
ENSEMBLE = [
    (32, 32, 40, WIND_101, 1),
    (48, 24, 60, (1.0, 0.0, 0.0), 2),
    (17, 53, 25, (0.0, 0.0, -1.0), 3),
    (64, 64, 0, WIND_101, 4),  # no particles: only the two sweeps
    (40, 40, 80, swe.wind_direction(-1.0, 0.0, 2.0), 5),
]


def _terrain(nx, nz, seed):
    return (terrain.normalise(terrain.fbm(nx, nz, seed, 4.0 / max(nx, nz))) + 0.1).astype(np.float32)


def _world(nx, nz, wind, seed):
    w = swe.World(nx, nz, params=swe.Params(pspeed=wind), seed=seed)
    w.upload(swe.Field.HEIGHT, _terrain(nx, nz, seed))
    return w


def _same(a, b):
    for f in swe.FIELDS:
        if not np.array_equal(bits(a.download(f)), bits(b.download(f))):
            return False
    return a.stats() == b.stats()


def test_ordered_batch_equals_worlds_eroded_alone():
    batch = [_world(nx, nz, wind, sd) for nx, nz, _, wind, sd in ENSEMBLE]
    alone = [_world(nx, nz, wind, sd) for nx, nz, _, wind, sd in ENSEMBLE]
    particles = [e[2] for e in ENSEMBLE]
    # one world draws from a caller tape instead of the rand() replica
    tape = oracle.glibc_rand_sequence(99, 100000)
    batch[1].set_rand_tape(tape)
    alone[1].set_rand_tape(tape)
    swe.batch_erode(batch, 2, particles, mode=swe.Mode.ORDERED)
    for w, p in zip(alone, particles):
        w.erode(p, 2, mode=swe.Mode.ORDERED)
    for k, (a, b) in enumerate(zip(batch, alone)):
        assert _same(a, b), k
        a.sync()
    # the rand() states and the tape cursor carry over to the next call
    swe.batch_erode(batch, 1, particles, mode=swe.Mode.ORDERED)
    for w, p in zip(alone, particles):
        w.erode(p, 1, mode=swe.Mode.ORDERED)
    for k, (a, b) in enumerate(zip(batch, alone)):
        assert _same(a, b), k
    for w in batch + alone:
        w.close()


def test_ordered_batch_world_equals_oracle_port():
    nx, nz, p, wind, sd = 40, 40, 80, WIND_101, 12
    h = _terrain(nx, nz, sd)
    ws = [_world(24, 24, (1.0, 0.0, 0.0), 30), _world(nx, nz, wind, sd)]
    swe.batch_erode(ws, 3, [30, p], mode=swe.Mode.ORDERED)
    port = oracle.Port(nx, nz, pspeed=wind)
    port.set_field(0, h)
    port.seed(sd)
    port.erode(p, 3)
    for f in swe.FIELDS:
        assert np.array_equal(bits(port.get_field(int(f))), bits(ws[1].download(f))), f
    assert ws[1].stats() == port.stats()
    for w in ws:
        w.close()


def test_ordered_batch_packs_worlds_into_warps():
    # more worlds than 8 warps per SM: several worlds share a warp
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    count = 8 * sms + 37
    sizes = [(8 + (k % 5) * 3, 8 + (k % 7) * 2) for k in range(count)]
    batch = [_world(nx, nz, WIND_101, 1000 + k) for k, (nx, nz) in enumerate(sizes)]
    particles = [5 + k % 11 for k in range(count)]
    swe.batch_erode(batch, 1, particles, mode=swe.Mode.ORDERED)
    for k in list(range(0, count, 97)) + [count - 1]:
        nx, nz = sizes[k]
        w = _world(nx, nz, WIND_101, 1000 + k)
        w.erode(particles[k], 1, mode=swe.Mode.ORDERED)
        assert _same(batch[k], w), k
        w.close()
    for w in batch:
        w.close()


def test_ordered_batch_reports_tape_exhaustion_per_world():
    a = _world(16, 16, WIND_101, 1)
    b = _world(16, 16, WIND_101, 2)
    b.set_rand_tape(np.arange(10, dtype=np.int32))
    swe.batch_erode([a, b], 1, [20, 20], mode=swe.Mode.ORDERED)
    a.sync()
    with pytest.raises(swe.SweError) as e:
        b.sync()
    assert e.value.code == -3


def test_ordered_batch_rejects_a_world_twice():
    w = _world(16, 16, WIND_101, 1)
    with pytest.raises(swe.SweError):
        swe.batch_erode([w, w], 1, [5, 5], mode=swe.Mode.ORDERED)
    w.close()
