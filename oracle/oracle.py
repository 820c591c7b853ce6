"""TEST INFRASTRUCTURE: ctypes access to the CPU oracles.

- `Port`: oracle/swe_oracle.cpp, this project's restatement of the reference's
  World::erode / Wind::fly / World::cascade / quad::_normal
  (source/world.hpp:36-153, source/wind.hpp:28-117, source/cellpool.h:200-223),
  plus the CPU model of the library's parallel fixed-point mode.
- `Reference`: the reference's own headers compiled by oracle/Makefile into
  oracle/_ref/libswe_ref_<N>.so (only where the reference sources exist).

Only tests, the smoke check and the bench's CPU legs import this module; the
product library never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
PORT_LIB = HERE / "_build" / "libswe_oracle.so"
REF_DIR = HERE / "_ref"
# The reference checkout: $SWE_REFERENCE, else a directory named "reference"
# beside this repository.
REFERENCE_SRC = Path(os.environ.get("SWE_REFERENCE", str(HERE.parent.parent / "reference")))

RNG_LIBC, RNG_GLIBC, RNG_TAPE = 0, 1, 2
EXP_LIBM, EXP_CR = 0, 1

_P = ctypes.c_void_p
_i64p = ctypes.POINTER(ctypes.c_int64)


def build_port() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE), "port"], check=True)
    return PORT_LIB


def reference_available() -> bool:
    return (REFERENCE_SRC / "source" / "world.hpp").exists()


def build_reference(sizes=(8, 16, 32, 64, 128, 256)) -> None:
    if not reference_available():
        raise FileNotFoundError(f"reference sources not found under {REFERENCE_SRC}")
    targets = [f"{REF_DIR}/libswe_ref_{n}.so" for n in sizes]
    subprocess.run(["make", "-s", "-C", str(HERE), f"REF={REFERENCE_SRC}", "-j8"] + targets, check=True)


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


_port = None


def port_lib():
    global _port
    if _port is None:
        build_port()
        L = ctypes.CDLL(str(PORT_LIB))
        L.so_params_default.argtypes = [ctypes.POINTER(_CParams)]
        L.so_create.restype = _P
        L.so_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(_CParams)]
        L.so_destroy.argtypes = [_P]
        L.so_set_params.argtypes = [_P, ctypes.POINTER(_CParams)]
        L.so_set_field.argtypes = [_P, ctypes.c_int, _P]
        L.so_get_field.argtypes = [_P, ctypes.c_int, _P]
        L.so_set_rng.argtypes = [_P, ctypes.c_int, ctypes.c_uint32]
        L.so_set_exp.argtypes = [_P, ctypes.c_int]
        L.so_set_tape.argtypes = [_P, _P, ctypes.c_long]
        L.so_tape_pos.restype = ctypes.c_long
        L.so_tape_pos.argtypes = [_P]
        L.so_erode.argtypes = [_P, ctypes.c_int, ctypes.c_int]
        L.so_normal.argtypes = [_P, ctypes.c_int, ctypes.c_int, _P]
        L.so_cascade.argtypes = [_P, ctypes.c_int, ctypes.c_int]
        L.so_trace.argtypes = [_P, ctypes.c_int, _P, ctypes.c_int, _P, _P]
        L.so_fly_live.argtypes = [_P, ctypes.c_float, ctypes.c_float, ctypes.c_int, _P, _P]
        L.so_stats.argtypes = [_P, _i64p, _i64p, _i64p]
        L.so_glibc_rand_sequence.argtypes = [ctypes.c_uint32, ctypes.c_int, _P]
        L.so_par_erode.argtypes = [_P, ctypes.c_int, ctypes.c_int, ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64)]
        L.so_par_set_spawn_mode.argtypes = [_P, ctypes.c_int]
        L.so_par_max_move.argtypes = [_P]
        L.so_par_max_move.restype = ctypes.c_float
        L.so_par_get_heights_q.argtypes = [_P, _P]
        L.so_par_ledger.argtypes = [_P, _i64p, _i64p]
        L.so_philox4x32.argtypes = [ctypes.c_uint32] * 6 + [_P]
        L.so_expf_libm_bits.argtypes = [ctypes.c_uint32, ctypes.c_long, _P]
        L.so_expf_poly.restype = ctypes.c_float
        L.so_expf_poly.argtypes = [ctypes.c_float]
        _port = L
    return _port


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_P)


def params_struct(max_age=512, boundarylayer=2.0, suspension=0.05, gravity=0.1, lrate=0.1, maxdiff=0.005,
                  settling=1.0, mapscale=80.0, pspeed=(1.0, 0.0, 0.0), frac_bits=24, lanes=0) -> _CParams:
    c = _CParams()
    c.max_age = max_age
    c.boundarylayer = boundarylayer
    c.suspension = suspension
    c.gravity = gravity
    c.lrate = lrate
    c.maxdiff = maxdiff
    c.settling = settling
    c.mapscale = mapscale
    for i in range(3):
        c.pspeed[i] = pspeed[i]
    c.frac_bits = frac_bits
    c.lanes = lanes
    return c


class Port:
    """The CPU restatement on an nx*nz map (row-major [x][z])."""

    def __init__(self, nx: int, nz: int | None = None, exp_kind: int = EXP_LIBM, **params):
        self.L = port_lib()
        self.nx, self.nz = nx, (nx if nz is None else nz)
        self._cp = params_struct(**params)
        self.w = self.L.so_create(self.nx, self.nz, ctypes.byref(self._cp))
        self.L.so_set_exp(self.w, exp_kind)
        self.L.so_set_rng(self.w, RNG_GLIBC, 1)
        self._keep = None

    def __del__(self):
        try:
            self.L.so_destroy(self.w)
        except Exception:
            pass

    @property
    def n(self):
        return self.nx * self.nz

    def set_field(self, f: int, a) -> None:
        a = np.ascontiguousarray(np.asarray(a, dtype=np.float32).reshape(-1))
        assert a.size == self.n
        self.L.so_set_field(self.w, f, _ptr(a))

    def get_field(self, f: int) -> np.ndarray:
        a = np.empty(self.n, dtype=np.float32)
        self.L.so_get_field(self.w, f, _ptr(a))
        return a.reshape(self.nx, self.nz)

    def seed(self, seed: int, libc: bool = False) -> None:
        self.L.so_set_rng(self.w, RNG_LIBC if libc else RNG_GLIBC, seed)

    def set_tape(self, tape) -> None:
        self._keep = np.ascontiguousarray(np.asarray(tape, dtype=np.int32).reshape(-1))
        self.L.so_set_tape(self.w, _ptr(self._keep), self._keep.size)

    def erode(self, particles: int, cycles: int = 1) -> None:
        self.L.so_erode(self.w, particles, cycles)

    def stats(self):
        s, p, t = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        self.L.so_stats(self.w, ctypes.byref(s), ctypes.byref(p), ctypes.byref(t))
        return s.value, p.value, t.value

    def normal(self, x: int, z: int) -> np.ndarray:
        o = np.empty(3, dtype=np.float32)
        self.L.so_normal(self.w, x, z, _ptr(o))
        return o

    def normals(self) -> np.ndarray:
        out = np.empty((self.nx, self.nz, 3), dtype=np.float32)
        for x in range(self.nx):
            for z in range(self.nz):
                out[x, z] = self.normal(x, z)
        return out

    def cascade(self, x: int, z: int) -> None:
        self.L.so_cascade(self.w, x, z)

    def trace(self, spawn_xz, steps: int, tape) -> np.ndarray:
        s = np.ascontiguousarray(np.asarray(spawn_xz, dtype=np.float32).reshape(-1, 2))
        t = np.ascontiguousarray(np.asarray(tape, dtype=np.int32).reshape(-1))
        out = np.empty((s.shape[0], steps, 9), dtype=np.float32)
        self.L.so_trace(self.w, s.shape[0], _ptr(s), steps, _ptr(t), _ptr(out))
        return out

    def fly_live(self, x: float, z: float, steps: int, tape=None):
        out = np.empty((steps, 9), dtype=np.float32)
        tp = None if tape is None else np.ascontiguousarray(np.asarray(tape, dtype=np.int32).reshape(-1))
        ok = self.L.so_fly_live(self.w, x, z, steps, _ptr(tp) if tp is not None else None, _ptr(out))
        return out, ok

    # parallel-mode model
    def par_erode(self, particles: int, cycles: int, seed: int, cycle: int = 0) -> int:
        c = ctypes.c_uint64(cycle)
        self.L.so_par_erode(self.w, particles, cycles, ctypes.c_uint64(seed), ctypes.byref(c))
        return c.value

    def par_spawn_mode(self, mode: int) -> None:
        """Which particles fly together in par_erode: 0 the library's rule,
        1 lane-own id sequences, 2 a fixed spawn schedule (so_par_set_spawn_mode)."""
        self.L.so_par_set_spawn_mode(self.w, int(mode))

    def par_max_move(self) -> float:
        """The last par_erode call's largest one-step move along x or z (cells)."""
        return float(self.L.so_par_max_move(self.w))

    def par_heights_q(self) -> np.ndarray:
        a = np.empty(self.n, dtype=np.int32)
        self.L.so_par_get_heights_q(self.w, _ptr(a))
        return a.reshape(self.nx, self.nz)

    def par_ledger(self):
        m, e = ctypes.c_int64(), ctypes.c_int64()
        self.L.so_par_ledger(self.w, ctypes.byref(m), ctypes.byref(e))
        return m.value, e.value


def glibc_rand_sequence(seed: int, n: int) -> np.ndarray:
    out = np.empty(n, dtype=np.int32)
    port_lib().so_glibc_rand_sequence(seed, n, _ptr(out))
    return out


def philox(c0, c1, c2, c3, k0, k1):
    out = np.empty(4, dtype=np.uint32)
    port_lib().so_philox4x32(c0, c1, c2, c3, k0, k1, _ptr(out))
    return out


def expf_libm_bits(first: int, n: int) -> np.ndarray:
    out = np.empty(n, dtype=np.float32)
    port_lib().so_expf_libm_bits(first, n, _ptr(out))
    return out


def expf_poly(x: float) -> float:
    return port_lib().so_expf_poly(ctypes.c_float(x))


class Reference:
    """The reference's own World/Wind code compiled for an N*N map. One map
    per process and library (the reference keeps it in statics)."""

    _libs: dict = {}

    def __init__(self, n: int):
        path = REF_DIR / f"libswe_ref_{n}.so"
        if not path.exists():
            build_reference(sizes=(n,))
        if n not in Reference._libs:
            L = ctypes.CDLL(str(path))
            L.ref_set_field.argtypes = [ctypes.c_int, _P]
            L.ref_get_field.argtypes = [ctypes.c_int, _P]
            L.ref_srand.argtypes = [ctypes.c_uint]
            L.ref_rand_calls.restype = ctypes.c_long
            L.ref_rand_sequence.argtypes = [ctypes.c_int, _P]
            L.ref_erode.argtypes = [ctypes.c_int]
            L.ref_erode_pspeed.argtypes = [ctypes.c_int, ctypes.c_float, ctypes.c_float, ctypes.c_float]
            L.ref_normal.argtypes = [ctypes.c_int, ctypes.c_int, _P]
            L.ref_cascade.argtypes = [ctypes.c_int, ctypes.c_int]
            L.ref_trace.argtypes = [ctypes.c_int, _P, _P, ctypes.c_int, _P, _P]
            L.ref_fly_live.argtypes = [ctypes.c_float, ctypes.c_float, _P, ctypes.c_int, _P, _P]
            L.ref_probe_order.argtypes = [_P]
            L.ref_map_init.argtypes = [ctypes.c_int]
            L.ref_updatenode.argtypes = [_P]
            Reference._libs[n] = L
        self.L = Reference._libs[n]
        self.nx = self.nz = n
        assert self.L.ref_size() == n

    @property
    def n(self):
        return self.nx * self.nz

    def set_field(self, f: int, a) -> None:
        a = np.ascontiguousarray(np.asarray(a, dtype=np.float32).reshape(-1))
        assert a.size == self.n
        self.L.ref_set_field(f, _ptr(a))

    def get_field(self, f: int) -> np.ndarray:
        a = np.empty(self.n, dtype=np.float32)
        self.L.ref_get_field(f, _ptr(a))
        return a.reshape(self.nx, self.nz)

    def reset(self, height) -> None:
        z = np.zeros(self.n, dtype=np.float32)
        for f in range(9):
            self.set_field(f, z)
        self.set_field(0, height)

    def srand(self, seed: int) -> None:
        self.L.ref_srand(seed)

    def erode(self, particles: int, cycles: int = 1, pspeed=None) -> None:
        for _ in range(cycles):
            if pspeed is None:
                self.L.ref_erode(particles)
            else:
                self.L.ref_erode_pspeed(particles, *[ctypes.c_float(v) for v in pspeed])

    def normal(self, x: int, z: int) -> np.ndarray:
        o = np.empty(3, dtype=np.float32)
        self.L.ref_normal(x, z, _ptr(o))
        return o

    def normals(self) -> np.ndarray:
        out = np.empty((self.nx, self.nz, 3), dtype=np.float32)
        for x in range(self.nx):
            for z in range(self.nz):
                out[x, z] = self.normal(x, z)
        return out

    def cascade(self, x: int, z: int) -> None:
        self.L.ref_cascade(x, z)

    def trace(self, spawn_xz, steps: int, tape, pspeed=(1.0, 0.0, 0.0)) -> np.ndarray:
        s = np.ascontiguousarray(np.asarray(spawn_xz, dtype=np.float32).reshape(-1, 2))
        t = np.ascontiguousarray(np.asarray(tape, dtype=np.int32).reshape(-1))
        ps = np.asarray(pspeed, dtype=np.float32)
        out = np.empty((s.shape[0], steps, 9), dtype=np.float32)
        rc = self.L.ref_trace(s.shape[0], _ptr(s), _ptr(ps), steps, _ptr(t), _ptr(out))
        assert rc == 0
        return out

    def fly_live(self, x: float, z: float, steps: int, tape=None, pspeed=(1.0, 0.0, 0.0)):
        ps = np.asarray(pspeed, dtype=np.float32)
        tp = None if tape is None else np.ascontiguousarray(np.asarray(tape, dtype=np.int32).reshape(-1))
        out = np.empty((steps, 9), dtype=np.float32)
        ok = self.L.ref_fly_live(ctypes.c_float(x), ctypes.c_float(z), _ptr(ps), steps,
                                 _ptr(tp) if tp is not None else None, _ptr(out))
        return out, ok

    def map_init(self, seed: int = 0) -> np.ndarray:
        """quad::map::init's own terrain (the bump), returned as heights."""
        self.L.ref_map_init(seed)
        return self.get_field(0)

    def vertices(self) -> np.ndarray:
        """updatenode's vertex data per cell: [n, n, 12] (P, N, T-P, B-P)."""
        out = np.zeros(self.n * 12, dtype=np.float32)
        self.L.ref_updatenode(_ptr(out))
        return out.reshape(self.nx, self.nz, 12)

    def probe_order(self):
        o = np.empty(7, dtype=np.int32)
        self.L.ref_probe_order(_ptr(o))
        return o
