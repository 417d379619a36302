"""In-tree build of libhdbscan_gb300.so for sm_103a (nvcc, no cmake).

Each translation unit under csrc/ compiles in parallel to an object file in
hdbscan_gb300/_build/, then nvcc links the shared library next to this file.
Arithmetic-bearing code is compiled with --fmad=false so that no multiply-add
can be contracted (the kernels also use explicit _rn intrinsics).
"""

from __future__ import annotations

import concurrent.futures
import fcntl
import os
import shutil
import subprocess
from pathlib import Path

PACKAGE = Path(__file__).resolve().parent
CSRC = PACKAGE / "csrc"
BUILD = PACKAGE / "_build"
LIBRARY = PACKAGE / "libhdbscan_gb300.so"
INCLUDE = PACKAGE.parent / "include"
SOURCES = ("hdb_capi.cu", "hdb_kernels_f32.cu", "hdb_kernels_f64.cu", "hdb_cluster_f32.cu", "hdb_cluster_f64.cu",
           "hdb_noalloc.cu")
ARCH = ("-gencode", "arch=compute_103a,code=sm_103a")
FLAGS = ("-O3", "-std=c++17", "--fmad=false", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2")


def nvcc() -> str:
    found = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(found).exists():
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build hdbscan_gb300")
    return found


def _inputs():
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + sorted(
        INCLUDE.glob("*.h"))


def up_to_date() -> bool:
    if not LIBRARY.exists():
        return False
    built = LIBRARY.stat().st_mtime
    return all(p.stat().st_mtime <= built for p in _inputs())


def _compile(source: str) -> Path:
    obj = BUILD / (Path(source).stem + ".o")
    cmd = [nvcc(), *ARCH, *FLAGS, "-I", str(INCLUDE), "-c", str(CSRC / source), "-o", str(obj)]
    result = subprocess.run(cmd, capture_output=True, text=True)
    if result.returncode:
        raise RuntimeError(f"nvcc failed on {source}:\n{result.stdout}\n{result.stderr}")
    return obj


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile (if stale) and return the path of libhdbscan_gb300.so."""
    if not force and up_to_date():
        return LIBRARY
    BUILD.mkdir(exist_ok=True)
    with open(BUILD / ".lock", "w") as lock:
        fcntl.flock(lock, fcntl.LOCK_EX)  # concurrent builders (test subprocesses) wait here
        if not force and up_to_date():
            return LIBRARY
        return _build_locked(verbose)


def _build_locked(verbose: bool) -> Path:
    workers = min(len(SOURCES), os.cpu_count() or 1)
    with concurrent.futures.ThreadPoolExecutor(workers) as pool:
        objects = list(pool.map(_compile, SOURCES))
    tmp = LIBRARY.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objects), "-lcudart"]
    result = subprocess.run(cmd, capture_output=True, text=True)
    if result.returncode:
        raise RuntimeError(f"nvcc link failed:\n{result.stdout}\n{result.stderr}")
    os.replace(tmp, LIBRARY)
    if verbose:
        print(f"built {LIBRARY}")
    return LIBRARY


if __name__ == "__main__":
    build(force=True, verbose=True)
