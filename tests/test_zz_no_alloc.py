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


def test_noalloc_matches_world_on_two_calls():
    torch = pytest.importorskip("torch")
    n, particles = 160, 16384
    params = swe.Params(pspeed=WIND_101, frac_bits=16)
    h = (terrain.normalise(terrain.fbm(n, n, 9, 1.0 / 40)) + 0.1).astype(np.float32)
    seed = 31

    world = swe.World(n, params=params, seed=seed)
    world.upload(swe.Field.HEIGHT, h)

    dev = torch.device("cuda", 0)
    fields = [torch.zeros(n * n, dtype=torch.float32, device=dev) for _ in range(9)]
    fields[0].copy_(torch.from_numpy(h.reshape(-1)))
    ptrs = (ctypes.c_void_p * 9)(*[f.data_ptr() for f in fields])
    cp = params.to_c()
    stream = torch.cuda.current_stream(dev).cuda_stream
    entry = _entry()

    for call in range(2):
        status = ctypes.c_uint32(0)
        rc = entry(ptrs, n, n, ctypes.byref(cp), seed, call, 1, particles, ctypes.c_void_p(stream),
                   ctypes.byref(status))
        assert rc == 0, swe.lib.swe_last_error()
        assert status.value == 0
        world.erode(particles, 1, mode=swe.Mode.PARALLEL)
        torch.cuda.synchronize()
        for k, f in enumerate(swe.FIELDS):
            got = fields[k].cpu().numpy().reshape(n, n)
            assert np.array_equal(bits(got), bits(world.download(f))), (call, f)

    # sizes beyond the static scratch are refused, not truncated
    status = ctypes.c_uint32(0)
    rc = entry(ptrs, 1024, 1024, ctypes.byref(cp), seed, 0, 1, particles, ctypes.c_void_p(stream),
               ctypes.byref(status))
    assert rc == -1 and b"SWE_NOALLOC_MAX_CELLS" in swe.lib.swe_last_error()
    rc = entry(ptrs, n, n, ctypes.byref(cp), seed, 0, 1, 1 << 20, ctypes.c_void_p(stream), ctypes.byref(status))
    assert rc == -1 and b"SWE_NOALLOC_MAX_PARTICLES" in swe.lib.swe_last_error()
    world.close()
