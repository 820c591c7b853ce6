"""CUDA parallel fixed-point mode against its CPU model (bit for bit), plus
its invariants: exact mass conservation, determinism, graph reuse, split
calls, and device-side status reporting."""
import numpy as np
import pytest

import simplewinderosion_gb300 as swe
from oracle import oracle
from simplewinderosion_gb300 import terrain
from tests.conftest import WIND_101, bits

pytestmark = pytest.mark.gpu


def _terrain(nx, nz, seed):
    return (terrain.normalise(terrain.fbm(nx, nz, seed, 4.0 / max(nx, nz))) + 0.1).astype(np.float32)


def _pair(nx, nz, seed, wind=WIND_101, frac_bits=24, wseed=5, lanes=0):
    h = _terrain(nx, nz, seed)
    port = oracle.Port(nx, nz, pspeed=wind, frac_bits=frac_bits, lanes=lanes)
    port.set_field(0, h)
    w = swe.World(nx, nz, params=swe.Params(pspeed=wind, frac_bits=frac_bits, lanes=lanes), seed=wseed)
    w.upload(swe.Field.HEIGHT, h)
    return port, w


@pytest.mark.parametrize("nx,nz,particles,cycles,wind,frac_bits,lanes", [
    (16, 16, 64, 3, WIND_101, 24, 0),
    (33, 70, 900, 2, (0.0, 0.0, -1.0), 24, 0),
    (64, 64, 4096, 2, WIND_101, 16, 0),
    (96, 64, 6144, 2, (1.0, 0.0, 0.0), 28, -1),
    (128, 128, 16384, 2, WIND_101, 24, 0),
    (128, 128, 16384, 1, WIND_101, 16, -1),
    (48, 40, 3000, 2, (0.0, 0.0, 1.0), 24, 37),
    # bounded lanes on one CTA per SM, 1 and 2 lanes per thread, dense and sparse
    (64, 64, 20000, 1, WIND_101, 16, -1),
    (64, 64, 70000, 1, WIND_101, 24, -1),
    (160, 96, 45000, 1, (0.0, 0.0, -1.0), 24, 40000),
    # more lanes than that form holds: the colour-phase kernel
    (64, 64, 200000, 1, WIND_101, 24, -1),
    # degenerate shapes: one row, one column, a thin strip on one CTA per SM,
    # and a single lane (one particle at a time)
    (1, 50, 200, 2, WIND_101, 24, 0),
    (50, 1, 200, 2, (1.0, 0.0, 0.0), 24, 0),
    (3, 2000, 6000, 1, (0.0, 0.0, 1.0), 16, 5000),
    (40, 40, 300, 1, WIND_101, 16, 1),
    # a larger map through the cluster (default lanes) and the grid form, and
    # the coarsest fixed-point format
    (256, 256, 32768, 1, WIND_101, 16, 0),
    (256, 256, 32768, 1, (0.0, 0.0, 1.0), 24, 8192),
    (64, 64, 4096, 2, WIND_101, 8, 0),
])
def test_parallel_bitwise_vs_cpu_model(nx, nz, particles, cycles, wind, frac_bits, lanes):
    port, w = _pair(nx, nz, 7, wind, frac_bits, lanes=lanes)
    port.par_erode(particles, cycles, seed=5)
    w.erode(particles, cycles, mode=swe.Mode.PARALLEL)
    for f in swe.FIELDS:
        assert np.array_equal(bits(port.get_field(int(f))), bits(w.download(f))), f
    m, e = port.par_ledger()
    assert w.mass_ledger() == (m, 0, e)
    assert w.stats() == port.stats()


def test_parallel_conserves_mass_exactly_256():
    n = 256
    h = terrain.config_plain_small(seed=1, n=n)
    w = swe.World(n, params=swe.Params(pspeed=WIND_101), seed=9)
    w.upload(swe.Field.HEIGHT, h)
    m0, _, e0 = w.mass_ledger()
    assert e0 == 0
    for _ in range(3):
        w.erode(n * n, 2, mode=swe.Mode.PARALLEL)
        m, i, e = w.mass_ledger()
        assert i == 0 and m + e == m0
    steps, spawned, transfers = w.stats()
    assert spawned == 2 * n * n and steps > spawned and transfers > 0


def test_parallel_deterministic():
    n = 256
    h = terrain.config_plain_small(seed=2, n=n)
    out = []
    for _ in range(2):
        w = swe.World(n, params=swe.Params(pspeed=WIND_101), seed=4)
        w.upload(swe.Field.HEIGHT, h)
        w.erode(n * n, 3, mode=swe.Mode.PARALLEL)
        out.append([w.download(f) for f in swe.FIELDS])
    for a, b in zip(*out):
        assert np.array_equal(bits(a), bits(b))


def test_parallel_split_calls_and_graph_reuse():
    port, w = _pair(48, 48, 3)
    w.erode(500, 2, mode=swe.Mode.PARALLEL)
    w.erode(800, 1, mode=swe.Mode.PARALLEL)   # new graph for a new particle count
    w.erode(500, 1, mode=swe.Mode.PARALLEL)
    cyc = port.par_erode(500, 2, seed=5)
    cyc = port.par_erode(800, 1, seed=5, cycle=cyc)
    port.par_erode(500, 1, seed=5, cycle=cyc)
    assert np.array_equal(bits(port.get_field(0)), bits(w.height))


def test_modes_interleave_through_float_heights():
    port, w = _pair(40, 40, 4)
    w.erode(300, 1, mode=swe.Mode.PARALLEL)
    port.par_erode(300, 1, seed=5)
    h = w.height
    assert np.array_equal(bits(h), bits(port.get_field(0)))
    w.erode(30, 1, mode=swe.Mode.ORDERED)  # float path continues from the converted map
    assert np.isfinite(w.height).all()


def test_zero_particles_and_zero_cycles():
    port, w = _pair(20, 20, 5)
    w.erode(0, 2, mode=swe.Mode.PARALLEL)
    port.par_erode(0, 2, seed=5)
    for f in swe.FIELDS:
        assert np.array_equal(bits(port.get_field(int(f))), bits(w.download(f)))
    w.erode(100, 0, mode=swe.Mode.PARALLEL)
    assert w.stats() == (0, 0, 0)


def test_nonfinite_height_is_reported_not_faulted():
    w = swe.World(32)
    h = _terrain(32, 32, 1)
    h[5, 5] = np.nan
    w.upload(swe.Field.HEIGHT, h)
    with pytest.raises(swe.SweError) as e:
        w.erode(100, 1, mode=swe.Mode.PARALLEL)
    assert e.value.code == -3
    assert "range" in str(e.value)
    w.upload(swe.Field.HEIGHT, _terrain(32, 32, 1))
    w.erode(100, 1, mode=swe.Mode.PARALLEL)  # the world stays usable


def test_upload_download_roundtrip_every_field():
    w = swe.World(17, 29)
    rs = np.random.RandomState(0)
    for f in swe.FIELDS:
        a = rs.standard_normal((17, 29)).astype(np.float32)
        w.upload(f, a)
        assert np.array_equal(bits(w.download(f)), bits(a))
    with pytest.raises(swe.SweError):
        w.upload(swe.Field.HEIGHT, np.zeros(10, np.float32))


@pytest.mark.parametrize("kind,ctas", [(1, 0), (2, 0), (2, 38), (2, 76), (2, 114), (2, 304), (2, 456), (2, 608),
                                       (3, 0), (3, 152), (3, 304)])
def test_launch_forms_give_the_same_result(kind, ctas):
    """Every launch form of the bounded-lanes kernel (one cluster, grids of
    various CTA counts) leaves the world bit for bit as the CPU model does."""
    port, w = _pair(96, 80, 7, WIND_101, 16, wseed=5, lanes=3000)
    w.set_form(kind, ctas)
    port.par_erode(12000, 2, seed=5)
    w.erode(12000, 2, mode=swe.Mode.PARALLEL)
    for f in swe.FIELDS:
        assert np.array_equal(bits(port.get_field(int(f))), bits(w.download(f))), (kind, ctas, f)
    w.close()


def test_autotuner_leaves_the_world_alone_and_keeps_results():
    port, w = _pair(128, 128, 3, WIND_101, 16, wseed=5, lanes=0)
    before = [w.download(f).copy() for f in swe.FIELDS]
    t = w.tune(16384)
    assert t["best_ms"] > 0 and t["default_ms"] > 0 and t["best_ms"] <= t["default_ms"]
    assert w.form() == (t["kind"], t["ctas"])
    for f, b in zip(swe.FIELDS, before):
        assert np.array_equal(bits(w.download(f)), bits(b)), f
    assert w.cycle == 0
    port.par_erode(16384, 1, seed=5)
    w.erode(16384, 1, mode=swe.Mode.PARALLEL)
    for f in swe.FIELDS:
        assert np.array_equal(bits(port.get_field(int(f))), bits(w.download(f))), f
    # cached: the same size, particles and lanes again
    w2 = swe.World(128, params=swe.Params(pspeed=WIND_101, frac_bits=16), seed=5)
    t2 = w2.tune(16384)
    assert (t2["kind"], t2["ctas"]) == (t["kind"], t["ctas"]) and t2["best_ms"] == 0.0
    w.close()
    w2.close()
