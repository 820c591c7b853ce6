"""Loads libswe_gb300.so, the package's CUDA library. There is no fallback:
if the library has not been built, the first use fails with a message naming
the build step."""
from __future__ import annotations

import ctypes
from pathlib import Path

lib_path = Path(__file__).resolve().parent / "_build" / "libswe_gb300.so"

_lib = None


def load() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not lib_path.exists():
            raise ImportError(
                f"{lib_path} is missing: build the CUDA library first "
                "(python -c 'import __graft_entry__ as g; g.build()' or python simplewinderosion_gb300/build.py)"
            )
        _lib = ctypes.CDLL(str(lib_path))
    return _lib
