"""Initial terrains: the host restatement of the device generator against
known properties (CPU), and the device generator against the restatement
(GPU): the reference's bump to one float ulp, fBm with pyramids and a
jittered sediment layer bit for bit."""
import numpy as np
import pytest

import simplewinderosion_gb300 as swe
from simplewinderosion_gb300 import terrain


def test_restated_bump_is_the_reference_terrain():
    # map::init (cellpool.h:380-428): peak 0.5 at (n/4, n/2), >= 0 everywhere
    n = 64
    h = terrain.device_terrain(n, n)
    assert h.shape == (n, n) and h.dtype == np.float32
    assert np.unravel_index(np.argmax(h), h.shape) == (n // 4, n // 2)
    assert h.max() == np.float32(0.5) and h.min() >= 0.0
    assert np.allclose(h, terrain.reference_bump(n), atol=1e-6)


def test_restated_fbm_is_normalised_and_seeded():
    a = terrain.device_terrain(48, 40, seed=7, octaves=6, base_freq=1 / 16)
    b = terrain.device_terrain(48, 40, seed=7, octaves=6, base_freq=1 / 16)
    c = terrain.device_terrain(48, 40, seed=8, octaves=6, base_freq=1 / 16)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    assert a.min() == 0.0 and abs(float(a.max()) - 0.5) < 1e-7
    j = terrain.device_terrain(48, 40, seed=7, octaves=6, base_freq=1 / 16, sediment=0.1, sediment_jitter=0.02)
    d = j.astype(np.float64) - a
    assert 0.08 - 1e-6 <= d.min() and d.max() <= 0.12 + 1e-6 and abs(d.mean() - 0.1) < 2e-3


@pytest.mark.gpu
@pytest.mark.parametrize("nx,nz,kw", [
    (64, 64, {}),
    (100, 37, {}),
    (96, 80, dict(seed=11, octaves=8, base_freq=1 / 32, top=0.5, sediment=0.1, sediment_jitter=0.02,
                  pyramids=[(48, 40, 0.4, 30), (10, 70, 0.2, 12.5)])),
    (256, 256, dict(seed=3, octaves=8, base_freq=1 / 64, persistence=0.45, sediment=0.1, sediment_jitter=0.02)),
])
def test_device_terrain_matches_restatement(nx, nz, kw):
    w = swe.World(nx, nz)
    w.terrain(**kw)
    got = w.height
    want = terrain.device_terrain(nx, nz, **kw)
    if kw.get("octaves", 0) == 0:
        # the bump goes through exp: the device's double exp and the host's
        # may differ in the last bit of a double, never by more than a float ulp
        assert np.max(np.abs(got.view(np.int32) - want.view(np.int32))) <= 1
    else:
        assert np.array_equal(got.view(np.int32), want.view(np.int32))
    m, i, e = w.mass_ledger()
    assert e == 0
    w.close()
