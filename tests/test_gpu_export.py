"""The wind map (SimpleWindErosion.cpp:224-230) from the device, against the
float formula on the host: erf of a float is within a few float ulps of the
correctly rounded value on both sides, and 1 + erf cancels near erf = -1, so
texels agree to a few ulps of 1 in absolute terms. And updatenode's vertices
bit for bit."""
import math

import numpy as np
import pytest

import simplewinderosion_gb300 as swe
from simplewinderosion_gb300 import terrain
from tests.conftest import WIND_101

pytestmark = pytest.mark.gpu


def _host_windmap(mx, my, mz):
    erf = np.vectorize(lambda v: np.float32(math.erf(float(v))), otypes=[np.float32])
    f = lambda m: (np.float32(0.5) * (np.float32(1.0) + erf((np.float32(2.0) * m).astype(np.float32)))).astype(np.float32)
    return np.stack([f(mx), f(my), f(mz), np.ones_like(mx)], axis=-1)


def test_windmap_matches_the_app_formula():
    n = 64
    w = swe.World(n, params=swe.Params(pspeed=WIND_101), seed=3)
    w.upload(swe.Field.HEIGHT, terrain.config_plain_small(seed=2, n=n))
    w.erode(4096, 3, mode=swe.Mode.PARALLEL)
    rng = np.random.default_rng(1)
    # momentum after erosion, plus a few planted values across erf's range
    mx = w.download(swe.Field.MOMENTUMX)
    mx[0, :8] = np.array([0, -0.0, 1e-8, -3.0, 3.0, 0.25, -0.7, 12.0], dtype=np.float32)
    w.upload(swe.Field.MOMENTUMX, mx)
    w.upload(swe.Field.MOMENTUMZ, rng.normal(0, 0.5, size=(n, n)).astype(np.float32))
    got = w.windmap()
    want = _host_windmap(w.download(swe.Field.MOMENTUMX), w.download(swe.Field.MOMENTUMY),
                         w.download(swe.Field.MOMENTUMZ))
    assert got.shape == (n, n, 4)
    assert np.all(got[..., 3] == 1.0)
    err = np.abs(got.astype(np.float64) - want.astype(np.float64))
    assert err.max() <= 4 * 2.0 ** -24, err.max()
    assert np.all((got >= 0.0) & (got <= 1.0))
    w.close()


def _host_vertices(h, normals, mapscale=np.float32(80.0)):
    nx, nz = h.shape
    hp = np.zeros((nx + 1, nz + 1), dtype=np.float32)
    hp[:nx, :nz] = h
    py = (mapscale * h).astype(np.float32)
    out = np.zeros((nx, nz, 12), dtype=np.float32)
    out[..., 0] = np.arange(nx, dtype=np.float32)[:, None]
    out[..., 1] = py
    out[..., 2] = np.arange(nz, dtype=np.float32)[None, :]
    out[..., 3:6] = normals
    out[..., 6] = 1.0
    out[..., 7] = (mapscale * hp[1:, :nz]).astype(np.float32) - py
    out[..., 10] = (mapscale * hp[:nx, 1:]).astype(np.float32) - py
    out[..., 11] = 1.0
    return out


def test_vertices_are_updatenode():
    # normals are pinned against the compiled reference elsewhere
    # (quad::_normal); here positions and edges, and that the normals agree
    w = swe.World(48, 40, seed=2)
    w.terrain(seed=5, octaves=6, base_freq=1 / 16, sediment=0.1, sediment_jitter=0.02)
    v = w.vertices()
    want = _host_vertices(w.height, w.normals())
    assert v.shape == (48, 40, 12)
    assert np.array_equal(v.view(np.int32), want.view(np.int32))
    w.close()


def test_vertices_equal_the_compiled_updatenode():
    """swe_world_vertices bit for bit the compiled reference's own updatenode
    output (tests/golden/vertices_16.npz: positions, normals and edges)."""
    from tests.conftest import golden
    g = golden("vertices_16")
    n = g["height"].shape[0]
    w = swe.World(n, seed=1)
    w.upload(swe.Field.HEIGHT, g["height"])
    assert np.array_equal(w.vertices().view(np.int32), np.asarray(g["vertices"], np.float32).view(np.int32))
    w.close()


def test_device_bump_equals_the_compiled_map_init():
    """swe_world_terrain's octaves-0 terrain against the compiled reference's
    quad::map::init (tests/golden/map_init_48.npz): within one float ulp (the
    device rounds exp(double) its own way)."""
    from tests.conftest import golden
    g = golden("map_init_48")
    n = int(g["n"])
    w = swe.World(n, seed=1)
    w.terrain()
    d = np.abs(w.height.view(np.int32).astype(np.int64) - np.asarray(g["height"], np.float32).view(np.int32))
    assert d.max() <= 1, d.max()
    w.close()
