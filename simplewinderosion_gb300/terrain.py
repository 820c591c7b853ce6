"""Seeded synthetic terrains for the erosion path (host side, numpy).

The reference builds one Gaussian bump normalised to [0, 0.5]
(source/cellpool.h:380-428; its FastNoiseLite fBm loop is commented out,
:388-411). The workloads here use the project's own gradient noise instead:
Perlin's improved noise (K. Perlin, "Improving Noise", SIGGRAPH 2002: quintic
fade 6t^5 - 15t^4 + 10t^3, hashed gradients from a seeded permutation)
summed as fractional Brownian motion. The same array feeds the GPU and the
CPU oracle, so parity never depends on the generator.
"""
from __future__ import annotations

import numpy as np

_GRAD2 = np.array([[1, 1], [-1, 1], [1, -1], [-1, -1], [1, 0], [-1, 0], [0, 1], [0, -1]], dtype=np.float64)


def _fade(t):
    return t * t * t * (t * (t * 6.0 - 15.0) + 10.0)


def perlin2(x: np.ndarray, y: np.ndarray, perm: np.ndarray) -> np.ndarray:
    """Improved gradient noise at points (x, y); perm has 512 entries."""
    xi = np.floor(x).astype(np.int64)
    yi = np.floor(y).astype(np.int64)
    xf = x - xi
    yf = y - yi
    xi &= 255
    yi &= 255
    u = _fade(xf)
    v = _fade(yf)

    def grad(h, dx, dy):
        g = _GRAD2[h & 7]
        return g[..., 0] * dx + g[..., 1] * dy

    aa = perm[perm[xi] + yi]
    ab = perm[perm[xi] + yi + 1]
    ba = perm[perm[xi + 1] + yi]
    bb = perm[perm[xi + 1] + yi + 1]
    x1 = grad(aa, xf, yf) * (1 - u) + grad(ba, xf - 1, yf) * u
    x2 = grad(ab, xf, yf - 1) * (1 - u) + grad(bb, xf - 1, yf - 1) * u
    return x1 * (1 - v) + x2 * v


def fbm(nx: int, nz: int, seed: int, base_freq: float, octaves: int = 8, lacunarity: float = 2.0,
        persistence: float = 0.5, persistence_jitter: float | None = None) -> np.ndarray:
    """fBm of improved noise on an nx*nz grid (row-major [x][z]), float64."""
    rs = np.random.RandomState(seed & 0xFFFFFFFF)
    p = rs.permutation(256)
    perm = np.concatenate([p, p]).astype(np.int64)
    off = rs.uniform(0, 256, size=2)
    xs = np.arange(nx, dtype=np.float64)[:, None]
    zs = np.arange(nz, dtype=np.float64)[None, :]
    out = np.zeros((nx, nz), dtype=np.float64)
    amp, freq = 1.0, base_freq
    pers = persistence if persistence_jitter is None else persistence_jitter
    for _ in range(octaves):
        out += amp * perlin2(xs * freq + off[0], zs * freq + off[1], perm)
        amp *= pers
        freq *= lacunarity
    return out


def normalise(h: np.ndarray, top: float = 0.5) -> np.ndarray:
    """Scale to [0, top], as map::init does for its bump (cellpool.h:416-428)."""
    lo, hi = float(h.min()), float(h.max())
    if hi == lo:
        return np.zeros_like(h)
    return (h - lo) / (hi - lo) * top


def pyramid(nx: int, nz: int, cx: float, cz: float, height: float, base: float) -> np.ndarray:
    """Square pyramid of bedrock: height at the centre, zero at base/2."""
    xs = np.arange(nx, dtype=np.float64)[:, None]
    zs = np.arange(nz, dtype=np.float64)[None, :]
    d = np.maximum(np.abs(xs - cx), np.abs(zs - cz)) / (base / 2.0)
    return height * np.clip(1.0 - d, 0.0, None)


def reference_bump(n: int) -> np.ndarray:
    """The reference's own initial terrain (cellpool.h:380-428) for an n*n
    map: exp(-d^2 n 0.2) around (n/4, n/2)/n, normalised to [0, 0.5]."""
    x = np.arange(n, dtype=np.float32)[:, None] / np.float32(n)
    z = np.arange(n, dtype=np.float32)[None, :] / np.float32(n)
    cx = np.float32((n // 4) / n)
    cz = np.float32((n // 2) / n)
    dx = (x - cx).astype(np.float32)
    dz = (z - cz).astype(np.float32)
    d = np.sqrt((dx * dx + dz * dz).astype(np.float32)).astype(np.float32)
    t = (-d * d * np.float32(n)).astype(np.float32)
    h = np.exp(t.astype(np.float64) * 0.2).astype(np.float32)
    lo = min(0.0, float(h.min()))
    hi = max(0.0, float(h.max()))
    return (0.5 * ((h.astype(np.float64) - lo) / (hi - lo))).astype(np.float32)


def config_plain_small(seed: int = 1, n: int = 256) -> np.ndarray:
    """256^2 bedrock fBm (8 octaves, lacunarity 2, persistence 0.5, base
    frequency 1/64) in [0, 0.5] plus a 0.1 +- 0.02 sediment layer; the single
    height field holds bedrock + sediment."""
    bed = normalise(fbm(n, n, seed, 1.0 / 64.0))
    rs = np.random.RandomState((seed * 7919 + 1) & 0xFFFFFFFF)
    sed = 0.1 + 0.02 * rs.uniform(-1.0, 1.0, size=(n, n))
    return (bed + sed).astype(np.float32)


def config_plain_large(seed: int = 2, n: int = 1024) -> np.ndarray:
    """1024^2 fBm (base frequency 1/256) in [0, 0.5] plus a 0.1 +- 0.02
    sediment layer and a square bedrock pyramid (height 0.4, base 200 cells)
    at the centre."""
    bed = normalise(fbm(n, n, seed, 1.0 / 256.0)) + pyramid(n, n, n / 2, n / 2, 0.4, 200.0 * n / 1024)
    rs = np.random.RandomState((seed * 7919 + 1) & 0xFFFFFFFF)
    sed = 0.1 + 0.02 * rs.uniform(-1.0, 1.0, size=(n, n))
    return (bed + sed).astype(np.float32)


# ---------------------------------------------------------------- device generator
# The library builds terrains on the GPU (swe_world_terrain). Its random
# draws come from splitmix64 (S. Vigna) instead of numpy's generator, and the
# functions below restate its steps on the host, so the two agree to
# rounding: the permutation by Fisher-Yates, two offsets, then one draw per
# cell for the sediment jitter.
_M64 = (1 << 64) - 1
_GOLDEN = 0x9E3779B97F4A7C15


def _splitmix64(state: int) -> tuple[int, int]:
    state = (state + _GOLDEN) & _M64
    z = state
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _M64
    return state, z ^ (z >> 31)


def _mix64_array(s: np.ndarray) -> np.ndarray:
    z = s + np.uint64(_GOLDEN)
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def device_terrain(nx: int, nz: int, seed: int = 0, octaves: int = 0, base_freq: float = 1.0 / 64.0,
                   lacunarity: float = 2.0, persistence: float = 0.5, top: float = 0.5, sediment: float = 0.0,
                   sediment_jitter: float = 0.0, pyramids=()) -> np.ndarray:
    """Host restatement of swe_world_terrain (float32 [nx, nz])."""
    f32 = lambda v: float(np.float32(v))  # the C struct holds floats
    st = seed & _M64
    p = list(range(256))
    for k in range(255, 0, -1):
        st, r = _splitmix64(st)
        j = r % (k + 1)
        p[k], p[j] = p[j], p[k]
    perm = np.array(p + p, dtype=np.int64)
    st, r = _splitmix64(st)
    offx = 256.0 * ((r >> 11) * (1.0 / 9007199254740992.0))
    st, r = _splitmix64(st)
    offz = 256.0 * ((r >> 11) * (1.0 / 9007199254740992.0))
    st, jitter_seed = _splitmix64(st)
    xs = np.arange(nx, dtype=np.float64)[:, None]
    zs = np.arange(nz, dtype=np.float64)[None, :]
    if octaves == 0:
        # map::init's bump in float (cellpool.h:380-385), exp in double
        px = (np.arange(nx, dtype=np.float32) / np.float32(nx))[:, None]
        pz = (np.arange(nz, dtype=np.float32) / np.float32(nz))[None, :]
        dx = (px - np.float32((nx // 4) / np.float32(nx))).astype(np.float32)
        dz = (pz - np.float32((nz // 2) / np.float32(nz))).astype(np.float32)
        d = np.sqrt((dx * dx + dz * dz).astype(np.float32)).astype(np.float32)
        t = ((-d * d).astype(np.float32) * np.float32(nx)).astype(np.float32)
        v = np.exp(t.astype(np.float64) * 0.2).astype(np.float32)
        lo, hi = np.float32(min(0.0, float(v.min()))), np.float32(max(0.0, float(v.max())))
        h = f32(top) * ((v - lo) / (hi - lo)).astype(np.float32).astype(np.float64)
    else:
        v = np.zeros((nx, nz), dtype=np.float64)
        amp, fr = 1.0, f32(base_freq)
        for _ in range(octaves):
            v = v + amp * perlin2(xs * fr + offx, zs * fr + offz, perm)
            amp *= f32(persistence)
            fr *= f32(lacunarity)
        lo, hi = float(v.min()), float(v.max())
        h = (v - lo) / (hi - lo) * f32(top) if hi > lo else np.zeros_like(v)
    for cx, cz, ph, base in pyramids:
        d = np.maximum(np.abs(xs - f32(cx)), np.abs(zs - f32(cz))) / (f32(base) / 2.0)
        h = h + f32(ph) * np.maximum(1.0 - d, 0.0)
    if sediment != 0.0 or sediment_jitter != 0.0:
        idx = np.arange(nx * nz, dtype=np.uint64).reshape(nx, nz)
        with np.errstate(over="ignore"):
            r = _mix64_array(np.uint64(jitter_seed) + idx * np.uint64(_GOLDEN))
        u = (r >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
        h = h + (f32(sediment) + f32(sediment_jitter) * (2.0 * u - 1.0))
    return h.astype(np.float32)
