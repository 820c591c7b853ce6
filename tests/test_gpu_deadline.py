"""The abort path of the parallel mode, on a normal terminating workload.

Every wait inside a PARALLEL cycle (grid barriers, cell-tag waits) has a
deadline, 2 s by default. Here the deadline is cut to a few hundred
nanoseconds, far below one barrier, so the first wait that spins runs out:
the thread sets SWE_STATUS_TIMEOUT, every thread leaves at the same barrier,
the call returns, and the next sync reports SWE_ERR_DEVICE. With the default
deadline restored and fresh fields uploaded, the same world then erodes bit
for bit like a freshly created one. Covered: the bounded-lanes kernel as one
16-CTA cluster and as one CTA per SM, and the all-at-once colour-phase kernel.
Nothing here waits for a flag that is never set: the waits would all end by
themselves a few microseconds later.
"""
import numpy as np
import pytest

import simplewinderosion_gb300 as swe
from simplewinderosion_gb300 import terrain
from tests.conftest import WIND_101, bits

pytestmark = pytest.mark.gpu

N = 96


def _h():
    return (terrain.normalise(terrain.fbm(N, N, 4, 1.0 / 24)) + 0.1).astype(np.float32)


@pytest.mark.parametrize("lanes,particles,form", [
    (0, 9216, "k_par_lanes, one 16-CTA cluster (1,024 lanes)"),
    (8192, 20000, "k_par_lanes, one CTA per SM"),
    (-1, 200000, "k_par_cycle, all particles at once"),
])
def test_short_deadline_aborts_and_world_recovers(lanes, particles, form):
    h = _h()
    params = swe.Params(pspeed=WIND_101, frac_bits=16, lanes=lanes)
    w = swe.World(N, params=params, seed=21)
    w.upload(swe.Field.HEIGHT, h)
    w.set_wait_limit(300)
    w.erode(particles, 1, mode=swe.Mode.PARALLEL, sync=False)
    with pytest.raises(swe.SweError) as e:
        w.sync()
    assert e.value.code == -3, form
    assert "deadline" in str(e.value), form
    assert w.status() == 0  # the sync cleared the status word

    # default deadline, fresh fields, cycle counter back to 0: the same as a new world
    w.set_wait_limit(0)
    zero = np.zeros((N, N), np.float32)
    for f in swe.FIELDS:
        w.upload(f, h if f == swe.Field.HEIGHT else zero)
    w.cycle = 0
    w.erode(particles, 1, mode=swe.Mode.PARALLEL)
    fresh = swe.World(N, params=params, seed=21)
    fresh.upload(swe.Field.HEIGHT, h)
    fresh.erode(particles, 1, mode=swe.Mode.PARALLEL)
    for f in swe.FIELDS:
        assert np.array_equal(bits(w.download(f)), bits(fresh.download(f))), (form, f)
    assert w.mass_ledger() == fresh.mass_ledger()
    w.close()
    fresh.close()
