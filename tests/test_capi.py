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
