"""Build recipe of the CUDA library libswe_gb300.so (sm_103a only).

Each .cu file is compiled on its own (in parallel) and the objects are linked
into one shared library with the CUDA runtime linked statically. All
translation units use -fmad=false: the kernels round every float multiply and
add separately, like the reference built with g++ -O2, and write fused
multiply-adds out explicitly where they want them.

One build step is host-side: gen_libm_expf lists the arguments where this
machine's C library expf differs from the correctly rounded value, and
swe_libm_table.cpp embeds that list, so the exact-semantics kernels reproduce
the reference's std::exp(float) (source/wind.hpp:50) bit for bit. The list is
regenerated per machine and C library.
"""
from __future__ import annotations

import os
import platform
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT_DIR = PKG / "_build"
LIB = OUT_DIR / "libswe_gb300.so"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3",
    "-lineinfo",
    "-std=c++17",
    "-fmad=false",
    "-Xcompiler",
    "-fPIC",
    "-I",
    str(INCLUDE),
]


def nvcc() -> str:
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libswe_gb300.so")


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def libm_tag() -> str:
    libc = "-".join(x for x in platform.libc_ver() if x) or "libc"
    return f"{platform.machine()}-{libc}".replace("/", "_")


def build_libm_table(force: bool = False) -> Path:
    """Generate (if needed) the expf exception list of this machine's libm."""
    gen_dir = OUT_DIR / "gen"
    gen_dir.mkdir(parents=True, exist_ok=True)
    out = gen_dir / f"libm_expf_{libm_tag()}.bin"
    src = CSRC / "gen_libm_expf.cpp"
    exe = gen_dir / f"gen_libm_expf_{platform.machine()}"
    if force or _stale(exe, [src]):
        cmd = [shutil.which("g++") or "g++", "-O2", "-std=c++17", "-pthread", "-o", str(exe), str(src)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"g++ failed on {src.name}:\n{r.stdout}\n{r.stderr}")
    if force or _stale(out, [exe]):
        r = subprocess.run([str(exe), str(out)], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"{exe.name} failed:\n{r.stdout}\n{r.stderr}")
    return out


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile the library if any source is newer than it; return its path."""
    srcs = sources()
    headers = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))
    obj_dir = OUT_DIR / "obj"
    obj_dir.mkdir(parents=True, exist_ok=True)
    exe = nvcc()

    def compile_one(src: Path) -> Path:
        obj = obj_dir / (src.stem + ".o")
        if force or _stale(obj, [src] + headers):
            cmd = [exe] + NVCC_FLAGS + ["-c", str(src), "-o", str(obj)]
            if verbose:
                print(" ".join(cmd), file=sys.stderr)
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}")
        return obj

    table = build_libm_table(force)

    def compile_table() -> Path:
        src = CSRC / "swe_libm_table.cpp"
        obj = obj_dir / f"swe_libm_table_{libm_tag()}.o"
        if force or _stale(obj, [src, table]):
            cmd = [shutil.which("g++") or "g++", "-c", "-fPIC", f"-DSWE_LIBM_EXPF_BIN={table}", str(src),
                   "-o", str(obj)]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"g++ failed on {src.name}:\n{r.stdout}\n{r.stderr}")
        return obj

    with ThreadPoolExecutor(max_workers=min(8, len(srcs) + 1)) as ex:
        fut = ex.submit(compile_table)
        objs = list(ex.map(compile_one, srcs))
        objs.append(fut.result())
    if force or _stale(LIB, objs):
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [exe] + ARCH + ["-shared", "-o", str(tmp)] + [str(o) for o in objs] + ["-cudart", "static"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
