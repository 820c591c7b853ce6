"""The C ABI without a GPU: the library builds, loads, exports every entry
point include/swe.h declares, reports the reference's default constants, and
rejects bad arguments before touching a device."""
import ctypes
import re
from pathlib import Path

import pytest

import simplewinderosion_gb300 as swe
from tests.conftest import ROOT

HEADER = ROOT / "include" / "swe.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(swe_[a-z_]+)\s*\(", text)))


def test_header_declares_the_path(lib_built):
    names = declared_functions()
    for must in ["swe_world_create", "swe_world_erode", "swe_world_upload", "swe_world_download",
                 "swe_trace_particles", "swe_world_mass_ledger", "swe_world_set_rand_tape", "swe_last_error"]:
        assert must in names


def test_library_exports_every_declared_symbol(lib_built):
    L = ctypes.CDLL(str(lib_built))
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing


def test_params_default_are_reference_statics(lib_built):
    c = swe._CParams()
    swe.lib.swe_params_default(ctypes.byref(c))
    # wind.hpp:23-26, world.hpp:30-32, cellpool.h:184, wind.hpp:13
    assert c.max_age == 512
    assert c.boundarylayer == pytest.approx(2.0)
    assert c.suspension == pytest.approx(0.05)
    assert c.gravity == pytest.approx(0.1)
    assert c.lrate == pytest.approx(0.1)
    assert c.maxdiff == pytest.approx(0.005)
    assert c.settling == pytest.approx(1.0)
    assert c.mapscale == pytest.approx(80.0)
    assert list(c.pspeed) == [1.0, 0.0, 0.0]
    py = swe.Params()
    for k in ("max_age", "boundarylayer", "suspension", "gravity", "lrate", "maxdiff", "settling", "mapscale",
              "frac_bits"):
        assert getattr(c, k) == pytest.approx(getattr(py, k))


@pytest.mark.parametrize("nx,nz", [(0, 4), (4, 0), (-3, 3), (70000, 70000)])
def test_create_rejects_bad_sizes(lib_built, nx, nz):
    with pytest.raises(swe.SweError) as e:
        swe.World(nx, nz)
    assert e.value.code == -1


def test_create_rejects_bad_params(lib_built):
    with pytest.raises(swe.SweError) as e:
        swe.World(8, params=swe.Params(frac_bits=40))
    assert e.value.code == -1
    with pytest.raises(swe.SweError):
        swe.World(8, params=swe.Params(boundarylayer=0.0))


def test_null_handles_are_rejected(lib_built):
    L = swe.lib
    assert L.swe_world_erode(None, 1, 1, 1) == -1
    assert L.swe_world_sync(None) == -1
    assert b"NULL" in L.swe_last_error()


def test_wind_direction_is_glm_normalize():
    x, y, z = swe.wind_direction(1, 0, 1)
    assert (x, y, z) == (0.70710677, 0.0, 0.70710677) or abs(x - 0.70710677) < 1e-7


def test_batch_rejects_bad_arguments(lib_built):
    L = swe.lib
    assert L.swe_batch_erode(None, -1, 1, None) == -1
    assert L.swe_batch_erode(None, 2, 1, None) == -1
    assert L.swe_batch_erode(None, 0, 1, None) == 0
    assert L.swe_batch_erode_ordered(None, -1, 1, None) == -1
    assert L.swe_batch_erode_ordered(None, 2, 1, None) == -1
    assert L.swe_batch_erode_ordered(None, 0, 1, None) == 0


def test_surrogate_entry_points_reject_bad_arguments(lib_built):
    # argument checks run before any device work, so no GPU is needed
    import ctypes
    L = swe.lib
    P = ctypes.c_void_p
    fake = P(0x1000)  # never dereferenced: every call below fails its checks first
    odd = P(0x1002)
    L.swe_nn_conv3x3.argtypes = [P, P, P, P] + [ctypes.c_int] * 5 + [P]
    assert L.swe_nn_conv3x3(None, fake, None, fake, 1, 8, 8, 16, 16, None) == -1      # NULL input
    assert L.swe_nn_conv3x3(fake, fake, None, fake, 1, 8, 8, 12, 16, None) == -1      # cin % 16
    assert L.swe_nn_conv3x3(fake, fake, None, fake, 1, 8, 8, 16, 12, None) == -1      # cout % 8
    assert L.swe_nn_conv3x3(odd, fake, None, fake, 1, 8, 8, 16, 16, None) == -1       # alignment
    L.swe_nn_conv3x3_wgrad.argtypes = [P, P, P, P] + [ctypes.c_int] * 5 + [P]
    assert L.swe_nn_conv3x3_wgrad(fake, fake, fake, None, 1, 8, 8, 16, 264, None) == -1  # cout > 256
    L.swe_nn_pool2.argtypes = [P, P] + [ctypes.c_int] * 5 + [P]
    assert L.swe_nn_pool2(fake, fake, 1, 7, 8, 16, 0, None) == -1                     # odd height
    assert L.swe_nn_pool2(fake, fake, 1, 8, 8, 12, 0, None) == -1                     # c % 8
    L.swe_nn_gelu.argtypes = [P, P, ctypes.c_int64, P]
    assert L.swe_nn_gelu(fake, fake, 12, None) == -1                                  # count % 8
    assert L.swe_nn_gelu(fake, fake, 0, None) == 0                                    # nothing to do
    L.swe_nn_adam.argtypes = [P, P, P, P, P, ctypes.c_int64] + [ctypes.c_float] * 4 + [ctypes.c_int, P]
    assert L.swe_nn_adam(fake, fake, fake, fake, None, 8, 1e-3, 0.9, 0.999, 1e-8, 0, None) == -1  # step 0
    assert b"adam" in L.swe_last_error()
    L.swe_nn_pack_input_centered.argtypes = [P, P, P, P] + [ctypes.c_int] * 3 + [ctypes.c_float, P]
    assert L.swe_nn_pack_input_centered(fake, fake, None, fake, 1, 8, 8, 0.35, None) == -1   # NULL means
    assert L.swe_nn_pack_input_centered(fake, fake, fake, fake, 0, 8, 8, 0.35, None) == -1   # no maps
    assert L.swe_nn_pack_input_centered(fake, fake, fake, fake, 1, 8, 8, float("nan"), None) == -1  # NaN ref
    assert b"pack_input_centered" in L.swe_last_error()
    L.swe_nn_conv3x3_tc.argtypes = [P, P, P, P, P] + [ctypes.c_int] * 5 + [P]
    assert L.swe_nn_conv3x3_tc(fake, fake, None, fake, None, 1, 8, 8, 12, 16, None) == -1     # cin % 16
    L.swe_nn_conv3x3_wgrad_tc.argtypes = [P, P, P, P] + [ctypes.c_int] * 5 + [P]
    assert L.swe_nn_conv3x3_wgrad_tc(fake, fake, fake, None, 1, 8, 8, 16, 144, None) == -1  # cout > 128


def test_surrogate_flop_count():
    from simplewinderosion_gb300 import surrogate
    fwd = surrogate.conv_flops(1, 8, 8)
    # by hand: 2 * cin * cout * 9 * pixels of each layer's resolution
    want = 2 * 9 * (16 * 32 * 64 + 32 * 32 * 64 + 32 * 64 * 16 + 64 * 96 * 4 + 96 * 128 * 1 + 128 * 128 * 1
                    + 128 * 96 * 4 + 96 * 64 * 16 + 64 * 32 * 64 + 32 * 16 * 64)
    assert fwd == want
    # a training step adds the input gradients (all but the first layer) and the weight gradients
    assert surrogate.conv_flops(1, 8, 8, backward=True) == 3 * want - 2 * 9 * 16 * 32 * 64
