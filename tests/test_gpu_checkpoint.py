"""Checkpoint and resume of the parallel mode: the nine fields, the seed and
the cycle counter are the whole state between cycles, so a fresh world given
them continues bit for bit as the original."""
import numpy as np
import pytest

import simplewinderosion_gb300 as swe
from simplewinderosion_gb300 import terrain
from tests.conftest import WIND_101, bits

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("lanes", [0, -1])
def test_resume_from_checkpoint_is_bitwise(lanes):
    n, particles = 96, 6000
    params = swe.Params(pspeed=WIND_101, frac_bits=24, lanes=lanes)
    h = (terrain.normalise(terrain.fbm(n, n, 4, 4.0 / n)) + 0.1).astype(np.float32)
    a = swe.World(n, params=params, seed=17)
    a.upload(swe.Field.HEIGHT, h)
    a.erode(particles, 2, mode=swe.Mode.PARALLEL)
    assert a.cycle == 2
    saved = {f: a.download(f) for f in swe.FIELDS}
    a.erode(particles, 3, mode=swe.Mode.PARALLEL)

    b = swe.World(n, params=params, seed=17)
    for f, v in saved.items():
        b.upload(f, v)
    b.cycle = 2
    b.erode(particles, 3, mode=swe.Mode.PARALLEL)
    assert b.cycle == a.cycle == 5
    for f in swe.FIELDS:
        assert np.array_equal(bits(a.download(f)), bits(b.download(f))), f
    a.close()
    b.close()
