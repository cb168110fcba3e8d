"""Builds the CUDA library (sm_103a) in-tree: simpimc_gb300/lib/libsimpimc_gb300.so.

Translation units compile in parallel with nvcc; the result links the CUDA runtime statically so
the shared object only needs the CUDA driver library (libcuda) at load time.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
SRC = PKG / "src"
BUILD = PKG / "_build"
LIB_DIR = PKG / "lib"
LIB = LIB_DIR / "libsimpimc_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "--extended-lambda", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-Wall", "-Xptxas", "-O3", "-diag-suppress", "177"]

SOURCES = [
    SRC / "capi.cu",
    SRC / "framework" / "setup.cu",
    SRC / "framework" / "output.cu",
    SRC / "kernels" / "estimators.cu",
    SRC / "kernels" / "sweep.cu",
    SRC / "kernels" / "batch.cu",
    SRC / "kernels" / "adjoint.cu",
    SRC / "kernels" / "perm.cu",
    SRC / "noalloc.cu",
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _deps_newer(obj: Path) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    for p in list(SRC.rglob("*")) + [PKG.parent / "include" / "simpimc_gb300.h", Path(__file__)]:
        if p.is_file() and p.stat().st_mtime > t:
            return True
    return False


def _compile(src: Path, extra: list[str]) -> Path:
    obj = BUILD / (src.stem + ".o")
    if _deps_newer(obj):
        cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-c", str(src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")
        if r.stderr.strip():
            sys.stderr.write(r.stderr)
    return obj


def build(verbose: bool = False, ptxas_info: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    LIB_DIR.mkdir(exist_ok=True)
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), SOURCES))
    if not LIB.exists() or any(o.stat().st_mtime > LIB.stat().st_mtime for o in objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True, ptxas_info="-v" in sys.argv)
