"""The CPU port against golden fixtures produced by the reference's own
compiled code (tests/golden/make_golden.py). Runs where the reference
sources are absent too. Bitwise on x86-64 (where the fixtures were made);
on other machines the C library's expf may round differently in rare cases,
so the bound there is 1e-5 absolute, and the count of exact matches is
reported."""
import platform

import numpy as np
import pytest

from oracle import oracle
from simplewinderosion_gb300 import terrain
from tests.conftest import bits, golden

X86 = platform.machine() in ("x86_64", "AMD64")


def _check(want, got, atol=1e-5):
    if X86:
        assert np.array_equal(bits(want), bits(got)), f"max |diff| {np.abs(want - got).max()}"
    else:
        assert np.allclose(want, got, atol=atol, rtol=0), f"max |diff| {np.abs(want - got).max()}"


def test_golden_rand_sequences():
    g = golden("rand_sequences")
    for s, seq in zip(g["seeds"], g["seqs"]):
        assert np.array_equal(oracle.glibc_rand_sequence(int(s), seq.size), seq)
    assert list(g["order"]) == [1, 0, 1, 0, 2, 1, 0]


@pytest.mark.parametrize("name", ["erode_32_default", "erode_64_wind101", "erode_16_edges"])
def test_golden_erode(name):
    g = golden(name)
    n = int(g["n"])
    port = oracle.Port(n, pspeed=tuple(float(v) for v in g["pspeed"]))
    port.set_field(0, g["height0"])
    port.seed(int(g["seed"]))
    port.erode(int(g["particles"]), int(g["cycles"]))
    for f in range(9):
        _check(g["fields"][f], port.get_field(f), atol=1e-4)


def test_golden_normals():
    g = golden("normals_16")
    port = oracle.Port(16)
    port.set_field(0, g["height"])
    _check(g["normals"], port.normals())


def test_golden_cascade():
    g = golden("cascade_12")
    port = oracle.Port(16)
    port.set_field(0, g["height"])
    for (x, z), after in zip(g["cells"], g["after"]):
        port.cascade(int(x), int(z))
        _check(after, port.get_field(0))


def _same_with_nans(want, got):
    # NaN payloads are the platform's; every other value bit for bit
    assert np.array_equal(np.isnan(want), np.isnan(got))
    m = ~np.isnan(want)
    assert np.array_equal(bits(want[m]), bits(got[m]))


def test_golden_cascade_ties_and_nans():
    g = golden("cascade_ties_nan")
    port = oracle.Port(16)
    port.set_field(0, g["height"])
    for (x, z), after in zip(g["cells"], g["after"]):
        port.cascade(int(x), int(z))
        _same_with_nans(after, port.get_field(0))


def trace_tape(seed, count, steps):
    return np.random.RandomState(seed + 1000).randint(0, 2**31 - 1, size=(count, steps, 3)).astype(np.int32)


@pytest.mark.parametrize("name", ["trace_48_default", "trace_48_wind101"])
def test_golden_trace(name):
    g = golden(name)
    rec = g["records"]
    port = oracle.Port(48, pspeed=tuple(float(v) for v in g["pspeed"]))
    port.set_field(0, g["height"])
    got = port.trace(g["spawn"], rec.shape[1], trace_tape(int(g["tape_seed"]), rec.shape[0], rec.shape[1]))
    _check(rec, got, atol=1e-4)


def test_reference_bump_restatement_is_the_compiled_map_init():
    """terrain.reference_bump restates quad::map::init's terrain
    (cellpool.h:380-428): bit for bit what the compiled reference built."""
    g = golden("map_init_48")
    n = int(g["n"])
    assert np.array_equal(bits(terrain.reference_bump(n)), bits(g["height"]))


def test_vertex_restatement_is_the_compiled_updatenode():
    """The vertex layout the library's swe_world_vertices writes (position,
    normal, +x edge, +z edge per cell; edges to cells past the map read height
    0) against the compiled reference's own updatenode (cellpool.h:302-333),
    with the normals from the reference's quad::_normal."""
    g = golden("vertices_16")
    h, v = g["height"], g["vertices"]
    n = h.shape[0]
    m = np.float32(80.0)
    hp = np.zeros((n + 1, n + 1), np.float32)
    hp[:n, :n] = h
    py = (m * h).astype(np.float32)
    assert np.array_equal(v[..., 0], np.broadcast_to(np.arange(n, dtype=np.float32)[:, None], (n, n)))
    assert np.array_equal(bits(v[..., 1]), bits(py))
    assert np.array_equal(bits(v[..., 7]), bits((m * hp[1:, :n]).astype(np.float32) - py))
    assert np.array_equal(bits(v[..., 10]), bits((m * hp[:n, 1:]).astype(np.float32) - py))
    assert np.all(v[..., 6] == 1.0) and np.all(v[..., 11] == 1.0)
    assert np.all(v[..., 8] == 0.0) and np.all(v[..., 9] == 0.0)
