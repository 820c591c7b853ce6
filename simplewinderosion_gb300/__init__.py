"""GB300 SimpleWindErosion: the erosion hot path (World::erode, Wind::fly,
World::cascade) as CUDA kernels for sm_103a behind a C ABI (include/swe.h).

This module is the Python side of that ABI: a thin ctypes mirror of the
reference's static simulation API (source/world.hpp:9-24, source/wind.hpp:4-26)
used by the tests and the benchmark. All computation happens in
libswe_gb300.so; there is no CPU fallback: without the built library the
first World (or any library call) raises ImportError.
"""
from __future__ import annotations

import ctypes
import enum
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import _lib as _libmod
from ._lib import lib_path

__all__ = ["Params", "Field", "Mode", "World", "SweError", "lib", "lib_path", "FIELDS", "wind_direction"]


class SweError(RuntimeError):
    """A C-ABI call returned a negative status."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"swe error {code}: {msg}")
        self.code = code


class Field(enum.IntEnum):
    """Cell fields in quad::cell order (source/cellpool.h:226-240)."""

    HEIGHT = 0
    MASSFLOW = 1
    MOMENTUMX = 2
    MOMENTUMY = 3
    MOMENTUMZ = 4
    MASSFLOW_TRACK = 5
    MOMENTUMX_TRACK = 6
    MOMENTUMY_TRACK = 7
    MOMENTUMZ_TRACK = 8


FIELDS = list(Field)


class Mode(enum.IntEnum):
    ORDERED = 0   # particles in sequence, C library rand(): the reference's own order
    PARALLEL = 1  # lock-step particles, fixed-point integer deposits


class _CParams(ctypes.Structure):
    _fields_ = [
        ("max_age", ctypes.c_int),
        ("boundarylayer", ctypes.c_float),
        ("suspension", ctypes.c_float),
        ("gravity", ctypes.c_float),
        ("lrate", ctypes.c_float),
        ("maxdiff", ctypes.c_float),
        ("settling", ctypes.c_float),
        ("mapscale", ctypes.c_float),
        ("pspeed", ctypes.c_float * 3),
        ("frac_bits", ctypes.c_int),
        ("lanes", ctypes.c_int),
    ]


@dataclass
class Params:
    """Mirror of the reference statics; defaults are the reference's values:
    Wind::maxAge/boundarylayer/suspension/gravity (wind.hpp:23-26),
    World::lrate/maxdiff/settling (world.hpp:30-32), quad::mapscale
    (cellpool.h:184), Wind::pspeed (wind.hpp:13). frac_bits is the parallel
    mode's fixed-point resolution; lanes its particles in flight (0: automatic,
    max(1024, cells/256), which keeps the sequential reference's terrain
    statistics: height histogram, spectrum and mean; < 0: all particles of a cycle at once)."""

    max_age: int = 512
    boundarylayer: float = 2.0
    suspension: float = 0.05
    gravity: float = 0.1
    lrate: float = 0.1
    maxdiff: float = 0.005
    settling: float = 1.0
    mapscale: float = 80.0
    pspeed: tuple = (1.0, 0.0, 0.0)
    frac_bits: int = 24
    lanes: int = 0

    def to_c(self) -> _CParams:
        c = _CParams()
        for k in ("max_age", "boundarylayer", "suspension", "gravity", "lrate", "maxdiff", "settling",
                  "mapscale", "frac_bits", "lanes"):
            setattr(c, k, getattr(self, k))
        for i in range(3):
            c.pspeed[i] = float(self.pspeed[i])
        return c


def wind_direction(x: float, y: float, z: float) -> tuple:
    """glm::normalize of a wind vector in float32 arithmetic:
    v * (1/sqrt(dot(v,v))), the prevailing wind the configs quote."""
    v = np.array([x, y, z], dtype=np.float32)
    d = np.float32(np.float32(v[0] * v[0] + v[1] * v[1]) + np.float32(v[2] * v[2]))
    s = np.float32(np.float32(1.0) / np.sqrt(d, dtype=np.float32))
    return tuple(float(np.float32(c * s)) for c in v)


_P = ctypes.c_void_p
_i64p = ctypes.POINTER(ctypes.c_int64)


class _CTerrain(ctypes.Structure):
    _fields_ = [("seed", ctypes.c_uint64), ("octaves", ctypes.c_int), ("base_freq", ctypes.c_float),
                ("lacunarity", ctypes.c_float), ("persistence", ctypes.c_float), ("top", ctypes.c_float),
                ("sediment", ctypes.c_float), ("sediment_jitter", ctypes.c_float), ("npyramids", ctypes.c_int),
                ("pyramids", ctypes.POINTER(ctypes.c_float))]


def _setup(L):
    L.swe_params_default.argtypes = [ctypes.POINTER(_CParams)]
    L.swe_world_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(_CParams), ctypes.c_uint64,
                                   ctypes.POINTER(_P)]
    L.swe_world_destroy.argtypes = [_P]
    L.swe_world_destroy.restype = None
    L.swe_world_set_params.argtypes = [_P, ctypes.POINTER(_CParams)]
    L.swe_world_upload.argtypes = [_P, ctypes.c_int, _P, ctypes.c_size_t]
    L.swe_world_download.argtypes = [_P, ctypes.c_int, _P, ctypes.c_size_t]
    L.swe_world_device_field.argtypes = [_P, ctypes.c_int, ctypes.POINTER(_P)]
    L.swe_world_erode.argtypes = [_P, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    L.swe_world_terrain.argtypes = [_P, ctypes.POINTER(_CTerrain)]
    L.swe_terrain_default.argtypes = [ctypes.POINTER(_CTerrain)]
    L.swe_terrain_default.restype = None
    L.swe_world_get_cycle.argtypes = [_P, ctypes.POINTER(ctypes.c_uint64)]
    L.swe_world_set_cycle.argtypes = [_P, ctypes.c_uint64]
    L.swe_world_set_wait_limit.argtypes = [_P, ctypes.c_uint64]
    L.swe_world_set_form.argtypes = [_P, ctypes.c_int, ctypes.c_int]
    L.swe_world_get_form.argtypes = [_P, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
    L.swe_world_tune.argtypes = [_P, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                 ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
    L.swe_batch_erode.argtypes = [ctypes.POINTER(_P), ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
    L.swe_batch_erode_ordered.argtypes = [ctypes.POINTER(_P), ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
    L.swe_batch_create.argtypes = [ctypes.POINTER(_P), ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.c_int,
                                   ctypes.POINTER(_P)]
    L.swe_batch_run.argtypes = [_P, ctypes.c_int]
    L.swe_batch_shape.argtypes = [_P, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                  ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
    L.swe_batch_set_shape.argtypes = [_P, ctypes.c_int, ctypes.c_int]
    L.swe_batch_destroy.argtypes = [_P]
    L.swe_batch_destroy.restype = None
    L.swe_world_sync.argtypes = [_P]
    L.swe_world_status.argtypes = [_P, ctypes.POINTER(ctypes.c_uint32)]
    L.swe_world_seed_rand.argtypes = [_P, ctypes.c_uint32]
    L.swe_world_set_rand_tape.argtypes = [_P, _P, ctypes.c_size_t]
    L.swe_world_mass_ledger.argtypes = [_P, _i64p, _i64p, _i64p]
    L.swe_world_stats.argtypes = [_P, _i64p, _i64p, _i64p]
    L.swe_trace_particles.argtypes = [_P, _P, ctypes.c_int, ctypes.c_int, _P, _P]
    L.swe_world_fly.argtypes = [_P, ctypes.c_float, ctypes.c_float, ctypes.c_int, _P, _P,
                                ctypes.POINTER(ctypes.c_int)]
    L.swe_world_cascade_at.argtypes = [_P, ctypes.c_int, ctypes.c_int]
    L.swe_world_normals.argtypes = [_P, _P, ctypes.c_size_t]
    L.swe_world_windmap.argtypes = [_P, _P, ctypes.c_size_t]
    L.swe_world_vertices.argtypes = [_P, _P, ctypes.c_size_t]
    L.swe_world_expf_bits.argtypes = [_P, ctypes.c_uint32, ctypes.c_size_t, _P]
    L.swe_world_get_stream.argtypes = [_P, ctypes.POINTER(_P)]
    L.swe_world_set_stream.argtypes = [_P, _P]
    L.swe_world_kernel_times.argtypes = [_P, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
    L.swe_world_phase_times.argtypes = [_P, _P, ctypes.c_int]
    L.swe_world_cascade_stats.argtypes = [_P, _i64p, _i64p, ctypes.POINTER(ctypes.c_int)]
    L.swe_last_error.restype = ctypes.c_char_p
    L.swe_last_error.argtypes = []


class _Lazy:
    """The library, loaded and typed on first attribute access."""

    def __init__(self):
        self._L = None

    def __getattr__(self, name):
        if self._L is None:
            L = _libmod.load()
            _setup(L)
            self._L = L
        return getattr(self._L, name)


lib = _Lazy()


def _check(rc: int):
    if rc != 0:
        raise SweError(rc, lib.swe_last_error().decode(errors="replace"))


def _ptr(a: np.ndarray) -> _P:
    return a.ctypes.data_as(_P)


class World:
    """One erosion world (the reference's `World` statics plus its map)."""

    def __init__(self, nx: int, nz: int | None = None, params: Params | None = None, seed: int = 0):
        self.nx = int(nx)
        self.nz = int(nx if nz is None else nz)
        self.params = params or Params()
        self._h = _P()
        cp = self.params.to_c()
        _check(lib.swe_world_create(self.nx, self.nz, ctypes.byref(cp), ctypes.c_uint64(seed),
                                    ctypes.byref(self._h)))

    # -- lifetime
    def close(self):
        if self._h:
            lib.swe_world_destroy(self._h)
            self._h = _P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def n(self) -> int:
        return self.nx * self.nz

    def set_params(self, params: Params):
        cp = params.to_c()
        _check(lib.swe_world_set_params(self._h, ctypes.byref(cp)))
        self.params = params

    # -- fields
    def upload(self, f: Field, values) -> None:
        a = np.ascontiguousarray(np.asarray(values, dtype=np.float32).reshape(-1))
        _check(lib.swe_world_upload(self._h, int(f), _ptr(a), a.size))

    def download(self, f: Field) -> np.ndarray:
        a = np.empty(self.n, dtype=np.float32)
        _check(lib.swe_world_download(self._h, int(f), _ptr(a), a.size))
        return a.reshape(self.nx, self.nz)

    def device_field(self, f: Field) -> int:
        p = _P()
        _check(lib.swe_world_device_field(self._h, int(f), ctypes.byref(p)))
        return int(p.value or 0)

    @property
    def height(self) -> np.ndarray:
        return self.download(Field.HEIGHT)

    @height.setter
    def height(self, v):
        self.upload(Field.HEIGHT, v)

    # -- simulation (World::erode, world.hpp:36-77)
    def erode(self, particles: int, cycles: int = 1, mode: Mode = Mode.PARALLEL, sync: bool = True) -> None:
        _check(lib.swe_world_erode(self._h, int(cycles), int(particles), int(mode)))
        if sync:
            self.sync()

    def sync(self) -> None:
        _check(lib.swe_world_sync(self._h))

    def status(self) -> int:
        s = ctypes.c_uint32()
        _check(lib.swe_world_status(self._h, ctypes.byref(s)))
        return int(s.value)

    def seed_rand(self, seed: int) -> None:
        _check(lib.swe_world_seed_rand(self._h, ctypes.c_uint32(seed)))

    def set_rand_tape(self, tape) -> None:
        if tape is None:
            _check(lib.swe_world_set_rand_tape(self._h, None, 0))
            return
        a = np.ascontiguousarray(np.asarray(tape, dtype=np.int32).reshape(-1))
        _check(lib.swe_world_set_rand_tape(self._h, _ptr(a), a.size))

    def mass_ledger(self) -> tuple[int, int, int]:
        m, i, e = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        _check(lib.swe_world_mass_ledger(self._h, ctypes.byref(m), ctypes.byref(i), ctypes.byref(e)))
        return m.value, i.value, e.value

    def stats(self) -> tuple[int, int, int]:
        s, p, t = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        _check(lib.swe_world_stats(self._h, ctypes.byref(s), ctypes.byref(p), ctypes.byref(t)))
        return s.value, p.value, t.value

    # -- unit-level entry points
    def trace(self, spawn_xz, steps: int, tape) -> np.ndarray:
        """Frozen-map trajectories; returns (n, steps, 9) records
        (alive, age, pos.xyz, speed.xyz, sediment)."""
        s = np.ascontiguousarray(np.asarray(spawn_xz, dtype=np.float32).reshape(-1, 2))
        n = s.shape[0]
        t = np.ascontiguousarray(np.asarray(tape, dtype=np.int32).reshape(-1))
        if t.size != n * steps * 3:
            raise ValueError("tape must hold 3 values per particle step")
        out = np.empty((n, steps, 9), dtype=np.float32)
        _check(lib.swe_trace_particles(self._h, _ptr(s), n, int(steps), _ptr(t), _ptr(out)))
        return out

    def fly(self, x: float, z: float, steps: int, tape=None) -> tuple[np.ndarray, int]:
        out = np.empty((steps, 9), dtype=np.float32)
        ok = ctypes.c_int()
        tp = None
        if tape is not None:
            tp = np.ascontiguousarray(np.asarray(tape, dtype=np.int32).reshape(-1))
            if tp.size != steps * 3:
                raise ValueError("tape must hold 3 values per step")
        _check(lib.swe_world_fly(self._h, ctypes.c_float(x), ctypes.c_float(z), int(steps),
                                 _ptr(tp) if tp is not None else None, _ptr(out), ctypes.byref(ok)))
        return out, ok.value

    def cascade(self, x: int, z: int) -> None:
        _check(lib.swe_world_cascade_at(self._h, int(x), int(z)))

    # -- streams and timing
    def stream(self) -> int:
        p = _P()
        _check(lib.swe_world_get_stream(self._h, ctypes.byref(p)))
        return int(p.value or 0)

    def set_stream(self, stream: int | None) -> None:
        _check(lib.swe_world_set_stream(self._h, _P(stream) if stream else None))

    def kernel_times(self) -> tuple[float, float]:
        """(fly_ms, cascade_ms) of the parallel mode, summed over the cycles
        of the last erode call."""
        a, b = ctypes.c_double(), ctypes.c_double()
        _check(lib.swe_world_kernel_times(self._h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    PHASES = ["spawn", "fly", "unused"] + [f"colour{k}" for k in range(9)] + ["ema"]

    def cascade_stats(self) -> tuple[int, int, int]:
        """(cascade evaluations, cell-steps with owed cascades, max cascades
        of one cell in one step) of the last parallel erode call."""
        a, b, m = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int()
        _check(lib.swe_world_cascade_stats(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(m)))
        return a.value, b.value, m.value

    def phase_times(self) -> dict:
        """Per-phase time (ms) of the parallel cycle kernel over the last
        erode call."""
        out = np.zeros(13, dtype=np.float64)
        _check(lib.swe_world_phase_times(self._h, _ptr(out), 13))
        return dict(zip(self.PHASES, out.tolist()))

    def upload_ptr(self, f: Field, host_ptr: int, n: int) -> None:
        """Upload from a raw host pointer (e.g. pinned memory)."""
        _check(lib.swe_world_upload(self._h, int(f), _P(host_ptr), n))

    def download_ptr(self, f: Field, host_ptr: int, n: int) -> None:
        _check(lib.swe_world_download(self._h, int(f), _P(host_ptr), n))

    def expf_bits(self, first_bits: int, n: int) -> np.ndarray:
        """The device's reference-compatible expf over n consecutive float bit
        patterns starting at first_bits."""
        out = np.empty(n, dtype=np.float32)
        _check(lib.swe_world_expf_bits(self._h, ctypes.c_uint32(first_bits), n, _ptr(out)))
        return out

    def normals(self) -> np.ndarray:
        out = np.empty(self.n * 3, dtype=np.float32)
        _check(lib.swe_world_normals(self._h, _ptr(out), out.size))
        return out.reshape(self.nx, self.nz, 3)

    @property
    def cycle(self) -> int:
        """PARALLEL-mode cycle counter (keys the random numbers with the seed)."""
        v = ctypes.c_uint64()
        _check(lib.swe_world_get_cycle(self._h, ctypes.byref(v)))
        return int(v.value)

    @cycle.setter
    def cycle(self, value: int) -> None:
        _check(lib.swe_world_set_cycle(self._h, ctypes.c_uint64(int(value))))

    def set_form(self, kind: int, ctas: int = 0) -> None:
        """Launch form of the PARALLEL kernel (0 default, 1 one cluster, 2 a
        grid of `ctas` CTAs, 3 the same with a CTA's lanes spread over four
        warps); changes no result."""
        _check(lib.swe_world_set_form(self._h, int(kind), int(ctas)))

    def form(self) -> tuple[int, int]:
        k, c = ctypes.c_int(), ctypes.c_int()
        _check(lib.swe_world_get_form(self._h, ctypes.byref(k), ctypes.byref(c)))
        return k.value, c.value

    def tune(self, particles: int) -> dict:
        """swe_world_tune: the fastest launch form for `particles` per cycle,
        timed on a scratch copy of this world and kept for it."""
        k, c, b, d = ctypes.c_int(), ctypes.c_int(), ctypes.c_double(), ctypes.c_double()
        _check(lib.swe_world_tune(self._h, int(particles), ctypes.byref(k), ctypes.byref(c), ctypes.byref(b),
                                  ctypes.byref(d)))
        return {"kind": k.value, "ctas": c.value, "best_ms": b.value, "default_ms": d.value}

    def set_wait_limit(self, ns: int) -> None:
        """Deadline (ns) of every wait inside a PARALLEL cycle; 0 restores
        the default 2 s. A wait past it aborts the cycle with
        SWE_STATUS_TIMEOUT (reported by the next sync)."""
        _check(lib.swe_world_set_wait_limit(self._h, ctypes.c_uint64(int(ns))))

    def vertices(self) -> np.ndarray:
        """swe_world_vertices: [nx, nz, 12] floats per cell, the position,
        normal and +x/+z edge vectors updatenode writes for rendering."""
        out = np.empty(self.n * 12, dtype=np.float32)
        _check(lib.swe_world_vertices(self._h, _ptr(out), out.size))
        return out.reshape(self.nx, self.nz, 12)

    def windmap(self) -> np.ndarray:
        """swe_world_windmap: RGBA float texels [nx, nz, 4] of the momentum
        fields, 0.5(1+erf(2 m)) per channel (the reference app's wind map)."""
        out = np.empty(self.n * 4, dtype=np.float32)
        _check(lib.swe_world_windmap(self._h, _ptr(out), out.size))
        return out.reshape(self.nx, self.nz, 4)

    def terrain(self, seed: int = 0, octaves: int = 0, base_freq: float = 1.0 / 64.0, lacunarity: float = 2.0,
                persistence: float = 0.5, top: float = 0.5, sediment: float = 0.0, sediment_jitter: float = 0.0,
                pyramids=()) -> None:
        """swe_world_terrain: build the initial height map on the device
        (octaves 0: the reference's Gaussian bump; else fBm), plus pyramids
        (cx, cz, height, base) and a jittered sediment layer."""
        pyr = np.ascontiguousarray(np.asarray(pyramids, dtype=np.float32).reshape(-1))
        t = _CTerrain(seed & 0xFFFFFFFFFFFFFFFF, octaves, base_freq, lacunarity, persistence, top, sediment,
                      sediment_jitter, len(pyr) // 4,
                      pyr.ctypes.data_as(ctypes.POINTER(ctypes.c_float)) if len(pyr) else None)
        _check(lib.swe_world_terrain(self._h, ctypes.byref(t)))


def batch_erode(worlds, cycles: int, particles, mode: Mode = Mode.PARALLEL) -> None:
    """`cycles` erode cycles of every world of an ensemble, particles[i]
    particles per cycle for worlds[i] (an int applies to all). Each world
    ends as swe_world_erode would leave it. PARALLEL (swe_batch_erode): the
    worlds that fit one 16-CTA cluster run together in one persistent
    launch. ORDERED (swe_batch_erode_ordered): every world bit for bit the
    reference's sequential loop, one GPU thread per world."""
    worlds = list(worlds)
    if isinstance(particles, int):
        particles = [particles] * len(worlds)
    if len(particles) != len(worlds):
        raise ValueError("one particle count per world")
    handles = (_P * len(worlds))(*[w._h for w in worlds])
    counts = (ctypes.c_int * len(worlds))(*[int(p) for p in particles])
    if Mode(mode) == Mode.ORDERED:
        _check(lib.swe_batch_erode_ordered(handles, len(worlds), int(cycles), counts))
    else:
        _check(lib.swe_batch_erode(handles, len(worlds), int(cycles), counts))


class Batch:
    """A prepared PARALLEL ensemble (swe_batch_create): repeated runs in one
    persistent launch each, capturable into a CUDA graph; `tune` picks the
    launch shape by measurement. The worlds must outlive the batch."""

    def __init__(self, worlds, particles, tune: bool = False):
        self.worlds = list(worlds)
        if isinstance(particles, int):
            particles = [particles] * len(self.worlds)
        handles = (_P * len(self.worlds))(*[w._h for w in self.worlds])
        counts = (ctypes.c_int * len(self.worlds))(*[int(p) for p in particles])
        self._h = _P()
        _check(lib.swe_batch_create(handles, len(self.worlds), counts, 1 if tune else 0, ctypes.byref(self._h)))

    def run(self, cycles: int = 1) -> None:
        """Enqueue `cycles` cycles on the first world's stream."""
        _check(lib.swe_batch_run(self._h, int(cycles)))

    def shape(self) -> dict:
        c, t, tm, dm = ctypes.c_int(), ctypes.c_int(), ctypes.c_double(), ctypes.c_double()
        _check(lib.swe_batch_shape(self._h, ctypes.byref(c), ctypes.byref(t), ctypes.byref(tm), ctypes.byref(dm)))
        return {"ctas_per_cluster": c.value, "threads_per_cta": t.value, "tuned_ms": tm.value,
                "default_ms": dm.value}

    def set_shape(self, ctas: int, threads: int) -> None:
        _check(lib.swe_batch_set_shape(self._h, int(ctas), int(threads)))

    def close(self):
        if self._h:
            lib.swe_batch_destroy(self._h)
            self._h = _P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

