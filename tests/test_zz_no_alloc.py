"""The allocation-free entry point swe_erode_parallel_noalloc, through the C ABI.

It serves callers that may not call cudaMalloc (a frame loop inside an
engine that owns the GPU's memory pool, or code running while another
framework's allocator owns the device memory): they pass their own nine
device fields, and the parallel kernel's scratch comes from a static device
array inside the library. Here the caller's fields are torch tensors, and the
results must equal those of the allocating world API (swe_world_erode in
parallel mode) bit for bit, on two calls in a row (the second call finds the
first call's leftovers in the shared scratch).

This file is collected last on purpose; it also runs alone in a fresh
process.
"""
import ctypes

import numpy as np
import pytest

import simplewinderosion_gb300 as swe
from simplewinderosion_gb300 import terrain
from tests.conftest import WIND_101, bits

pytestmark = pytest.mark.gpu


def _entry():
    L = swe.lib
    f = L.swe_erode_parallel_noalloc
    f.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, ctypes.c_int, ctypes.POINTER(swe._CParams),
                  ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                  ctypes.POINTER(ctypes.c_uint32)]
    return f


def _fields(torch, h):
    dev = torch.device("cuda", 0)
    fields = [torch.zeros(h.size, dtype=torch.float32, device=dev) for _ in range(9)]
    fields[0].copy_(torch.from_numpy(h.reshape(-1)))
    return fields, (ctypes.c_void_p * 9)(*[f.data_ptr() for f in fields])


def _call(entry, ptrs, nx, nz, cp, seed, first_cycle, particles, stream):
    status = ctypes.c_uint32(0)
    rc = entry(ptrs, nx, nz, ctypes.byref(cp), seed, first_cycle, 1, particles, ctypes.c_void_p(stream),
               ctypes.byref(status))
    assert rc == 0, swe.lib.swe_last_error()
    assert status.value == 0


def _same(fields, world, nx, nz, what):
    for k, f in enumerate(swe.FIELDS):
        got = fields[k].cpu().numpy().reshape(nx, nz)
        assert np.array_equal(bits(got), bits(world.download(f))), (what, f)


@pytest.mark.parametrize("lanes,particles,form", [
    (0, 16384, "one 16-CTA cluster (default lanes, 1,024)"),
    (8192, 20000, "one CTA per SM (8,192 lanes)"),
])
def test_noalloc_matches_world_on_two_calls(lanes, particles, form):
    torch = pytest.importorskip("torch")
    n = 160
    params = swe.Params(pspeed=WIND_101, frac_bits=16, lanes=lanes)
    h = (terrain.normalise(terrain.fbm(n, n, 9, 1.0 / 40)) + 0.1).astype(np.float32)
    seed = 31

    world = swe.World(n, params=params, seed=seed)
    world.upload(swe.Field.HEIGHT, h)
    fields, ptrs = _fields(torch, h)
    cp = params.to_c()
    stream = torch.cuda.current_stream(torch.device("cuda", 0)).cuda_stream
    entry = _entry()

    # two calls in a row: the second finds the first call's leftovers in the
    # shared scratch
    for call in range(2):
        _call(entry, ptrs, n, n, cp, seed, call, particles, stream)
        world.erode(particles, 1, mode=swe.Mode.PARALLEL)
        torch.cuda.synchronize()
        _same(fields, world, n, n, (form, call))
    world.close()

    # then another map shape: the scratch's layout (map stride, bitmap and
    # track offsets) changes with nx*nz
    nx, nz = 96, 200
    h2 = (terrain.normalise(terrain.fbm(nx, nz, 4, 1.0 / 32)) + 0.1).astype(np.float32)
    fresh = swe.World(nx, nz, params=params, seed=seed)
    fresh.upload(swe.Field.HEIGHT, h2)
    fields2, ptrs2 = _fields(torch, h2)
    _call(entry, ptrs2, nx, nz, cp, seed, 0, particles, stream)
    fresh.erode(particles, 1, mode=swe.Mode.PARALLEL)
    torch.cuda.synchronize()
    _same(fields2, fresh, nx, nz, (form, "96x200"))
    fresh.close()


def test_noalloc_refuses_sizes_beyond_the_static_scratch():
    torch = pytest.importorskip("torch")
    n = 160
    h = np.zeros((n, n), np.float32)
    fields, ptrs = _fields(torch, h)
    cp = swe.Params(pspeed=WIND_101, frac_bits=16).to_c()
    stream = torch.cuda.current_stream(torch.device("cuda", 0)).cuda_stream
    entry = _entry()
    status = ctypes.c_uint32(0)
    rc = entry(ptrs, 1024, 1024, ctypes.byref(cp), 31, 0, 1, 16384, ctypes.c_void_p(stream), ctypes.byref(status))
    assert rc == -1 and b"SWE_NOALLOC_MAX_CELLS" in swe.lib.swe_last_error()
    rc = entry(ptrs, n, n, ctypes.byref(cp), 31, 0, 1, 1 << 20, ctypes.c_void_p(stream), ctypes.byref(status))
    assert rc == -1 and b"SWE_NOALLOC_MAX_PARTICLES" in swe.lib.swe_last_error()
