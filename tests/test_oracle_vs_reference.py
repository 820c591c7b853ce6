"""The CPU port (oracle/swe_oracle.cpp) against the reference's own code
compiled from its headers (oracle/_ref), bit for bit. Needs the reference
sources; skipped where they are absent (the golden fixtures cover that case).

Reference functions exercised: World::erode (source/world.hpp:36-77),
Wind::fly (source/wind.hpp:28-117), World::cascade (world.hpp:79-153),
quad::_normal (source/cellpool.h:200-223).
"""
import numpy as np
import pytest

from oracle import oracle
from simplewinderosion_gb300 import terrain
from tests.conftest import WIND_101, bits

pytestmark = pytest.mark.skipif(not oracle.reference_available(), reason="reference sources not present")


@pytest.fixture(scope="module", autouse=True)
def _built():
    oracle.build_reference(sizes=(8, 16, 32, 64, 128, 256))


def test_rand_argument_order_is_right_to_left():
    # ivec2(r,r), vec2(r,r): first draw -> second component; vec3: z, y, x.
    assert list(oracle.Reference(8).probe_order()) == [1, 0, 1, 0, 2, 1, 0]


@pytest.mark.parametrize("seed", [0, 1, 7, 12345, 2**31 + 5, 4294967295])
def test_rand_replica_matches_libc(seed):
    ref = oracle.Reference(8)
    ref.srand(seed)
    want = np.empty(5000, dtype=np.int32)
    ref.L.ref_rand_sequence(5000, oracle._ptr(want))
    assert np.array_equal(oracle.glibc_rand_sequence(seed, 5000), want)


def _terrain(n, seed):
    return (terrain.normalise(terrain.fbm(n, n, seed, 4.0 / n)) + 0.1).astype(np.float32)


def _compare_fields(ref, port):
    for f in range(9):
        a, b = ref.get_field(f), port.get_field(f)
        assert np.array_equal(bits(a), bits(b)), f"field {f}: max |diff| {np.abs(a - b).max()}"


@pytest.mark.parametrize("n,particles,cycles,seed,wind", [
    (16, 50, 4, 3, None),
    (16, 50, 3, 4, (0.0, 0.0, -1.0)),
    (32, 80, 3, 5, WIND_101),
    (64, 200, 3, 6, None),
    (128, 400, 2, 8, WIND_101),
    (256, 1000, 2, 9, WIND_101),
])
def test_erode_bitwise(n, particles, cycles, seed, wind):
    ref = oracle.Reference(n)
    h = _terrain(n, seed)
    ref.reset(h)
    ref.srand(seed)
    ref.erode(particles, cycles, pspeed=wind)
    port = oracle.Port(n, pspeed=wind or (1.0, 0.0, 0.0))
    port.set_field(0, h)
    port.seed(seed)
    port.erode(particles, cycles)
    _compare_fields(ref, port)


def test_restated_loop_equals_world_erode():
    # The harness's erode-with-pspeed restatement is World::erode itself when
    # pspeed keeps its default (1,0,0).
    n = 32
    h = _terrain(n, 2)
    a = oracle.Reference(n)
    a.reset(h); a.srand(42); a.erode(60, 2)
    fa = [a.get_field(f) for f in range(9)]
    a.reset(h); a.srand(42); a.erode(60, 2, pspeed=(1.0, 0.0, 0.0))
    for f in range(9):
        assert np.array_equal(bits(fa[f]), bits(a.get_field(f)))


def test_port_libc_rand_equals_replica():
    n = 32
    h = _terrain(n, 3)
    p1 = oracle.Port(n); p1.set_field(0, h); p1.seed(77, libc=True); p1.erode(50, 2)
    p2 = oracle.Port(n); p2.set_field(0, h); p2.seed(77); p2.erode(50, 2)
    for f in range(9):
        assert np.array_equal(bits(p1.get_field(f)), bits(p2.get_field(f)))


def test_normals_bitwise():
    n = 16
    rs = np.random.RandomState(1)
    h = rs.uniform(0, 0.5, (n, n)).astype(np.float32)
    h[:5, :5] = 0.25
    h[8:, :] += 0.4
    ref = oracle.Reference(n); ref.reset(h)
    port = oracle.Port(n); port.set_field(0, h)
    assert np.array_equal(bits(ref.normals()), bits(port.normals()))


def test_cascade_bitwise_edges_and_ties():
    n = 16
    rs = np.random.RandomState(2)
    h = rs.uniform(0, 0.05, (n, n)).astype(np.float32)
    h[3, :] = 0.02
    h[7, 7] = 0.6
    h[0, 0] = 0.3
    h[n - 1, 5] = -0.3
    ref = oracle.Reference(n); ref.reset(h)
    port = oracle.Port(n); port.set_field(0, h)
    cells = [(7, 7), (3, 3), (0, 0), (n - 1, n - 1), (n - 1, 5), (3, 0), (6, 7), (7, 7)]
    cells += [tuple(c) for c in rs.randint(0, n, (60, 2))]
    for x, z in cells:
        ref.cascade(int(x), int(z))
        port.cascade(int(x), int(z))
        assert np.array_equal(bits(ref.get_field(0)), bits(port.get_field(0))), (x, z)


@pytest.mark.parametrize("wind", [(1.0, 0.0, 0.0), WIND_101, (0.0, 0.0, -1.0)])
def test_trace_bitwise(wind):
    n, count, steps = 64, 96, 200
    rs = np.random.RandomState(5)
    h = _terrain(n, 5)
    spawn = (rs.randint(0, n, (count, 2)) + rs.randint(0, 1000, (count, 2)) / np.float32(1000)).astype(np.float32)
    tape = rs.randint(0, 2**31 - 1, (count, steps, 3)).astype(np.int32)
    ref = oracle.Reference(n); ref.reset(h)
    want = ref.trace(spawn, steps, tape, pspeed=wind)
    port = oracle.Port(n, pspeed=wind); port.set_field(0, h)
    got = port.trace(spawn, steps, tape)
    assert np.array_equal(bits(want), bits(got))
    # the map really stayed frozen in the reference harness
    assert np.array_equal(bits(ref.get_field(0)), bits(h))


def test_fly_live_bitwise():
    n, steps = 32, 400
    h = _terrain(n, 6)
    rs = np.random.RandomState(6)
    tape = rs.randint(0, 2**31 - 1, (steps, 3)).astype(np.int32)
    ref = oracle.Reference(n); ref.reset(h)
    port = oracle.Port(n); port.set_field(0, h)
    for x, z in [(3.2, 4.7), (10.5, 20.499), (0.0, 31.4)]:
        a, oka = ref.fly_live(x, z, steps, tape)
        b, okb = port.fly_live(x, z, steps, tape)
        assert oka == okb
        assert np.array_equal(bits(a), bits(b))
        for f in range(9):
            assert np.array_equal(bits(ref.get_field(f)), bits(port.get_field(f)))
