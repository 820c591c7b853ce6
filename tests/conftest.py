"""Test configuration: the `gpu` marker and shared fixtures.

Tests marked `gpu` need a CUDA device and call the library through its C ABI
(include/swe.h); everything else runs on the CPU: the oracles against the
reference and the golden fixtures, the host logic, and the library's exported
symbols.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"
WIND_101 = (0.70710677, 0.0, 0.70710677)  # glm::normalize(vec3(1,0,1)) in float


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); calls the C ABI")


def golden(name: str) -> dict:
    with np.load(GOLDEN / f"{name}.npz") as z:
        return {k: z[k] for k in z.files}


def bits(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32)).view(np.int32)


@pytest.fixture(scope="session")
def lib_built():
    """The CUDA library, built if needed (nvcc cross-compiles without a GPU)."""
    from simplewinderosion_gb300 import build as b
    return b.build()
