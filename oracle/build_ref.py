"""Compile the reference's own CUDA-C kernel bodies for the CPU into oracle/_ref/.

Test infrastructure only.  The reference (CosineAI/hdbscan) keeps its CUDA
kernels as C source strings in hdbscan_gpu/_kernels.py and JIT-compiles them
with NVRTC through CuPy (hdbscan_gpu/_cuda.py:18-42).  Their serial branch
(no PARALLEL_PRIM) is plain C, so with a small CPU macro header
(oracle/ref_cpu_header.inc) and a host driver (oracle/ref_driver.inc) it builds
with g++ and runs here without CuPy or a GPU.

This script reads the strings from the reference checkout where it lies
($HDB_REFERENCE, a path given on the command line, or else a checkout named
"reference" beside this repository), writes the generated translation units
ONLY into oracle/_ref/ (git-ignored, never committed) and compiles
oracle/_ref/libhdb_ref.so.  When the reference checkout is absent but the
generated sources are present (a copy of this tree on another machine), it
compiles those.  Uses: validating the oracle restatement, generating the
golden vectors, and the reference arm of bench.py.
"""

from __future__ import annotations

import importlib.util
import json
import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
LIBRARY = OUT / "libhdb_ref.so"
DEFAULT_REFERENCE = Path(os.environ["HDB_REFERENCE"]) if os.environ.get("HDB_REFERENCE") else \
    HERE.parent.parent / "reference"


def _load_kernels(reference: Path):
    path = reference / "hdbscan_gpu" / "_kernels.py"
    spec = importlib.util.spec_from_file_location("_hdb_reference_kernels", path)
    module = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(module)  # pure string constants; imports nothing
    return module


def generate(reference: Path = DEFAULT_REFERENCE) -> bool:
    """Write oracle/_ref/ref_kernels.cpp from the reference strings; False if the checkout is absent."""
    if not (reference / "hdbscan_gpu" / "_kernels.py").exists():
        return False
    kernels = _load_kernels(reference)
    OUT.mkdir(exist_ok=True)
    parts = ['#include "../ref_cpu_header.inc"\n']
    for suffix, real, maximum in (("f32", "float", "3.4028234663852886e+38F"),
                                  ("f64", "double", "1.7976931348623157e+308")):
        parts.append(f"namespace ref_{suffix} {{\ntypedef {real} Real;\n#define REAL_MAX {maximum}\n")
        parts.append("static void distances_one(int hdb_gid, const Real* x, const int* params, Real* distances) {\n")
        parts.append(kernels.DISTANCE_SOURCE)
        parts.append("\n}\n")
        parts.append("static void clusters_one(int hdb_gid, const Real* distances, const Real* core, const int* params, "
                     "const Real* options, int* labels, int* integers, Real* reals) {\n")
        parts.append(kernels.CLUSTER_SOURCE)
        parts.append("\n}\n")
        # Linkage-only prefix (Prim + sort + union-find), as the reference's own
        # kernel tests build it: the full body reuses left/right/sizes later.
        parts.append("static void linkage_one(int hdb_gid, const Real* distances, const Real* core, const int* params, "
                     "const Real* options, int* labels, int* integers, Real* reals) {\n")
        parts.append(kernels.CLUSTER_SOURCE.split(kernels.CONDENSE_SOURCE)[0])
        parts.append("\n}\n")
        parts.append(f'#define HDB_REF_SUFFIX {suffix}\n#include "../ref_driver.inc"\n#undef HDB_REF_SUFFIX\n')
        parts.append("#undef REAL_MAX\n}\n")
    text = "".join(parts)
    target = OUT / "ref_kernels.cpp"
    if not target.exists() or target.read_text() != text:  # keep the mtime when nothing changed
        target.write_text(text)
    layout = {
        "INTEGER_ARRAYS": list(kernels.INTEGER_ARRAYS),
        "REAL_ARRAYS": list(kernels.REAL_ARRAYS),
        "INTEGER_WORKSPACE": kernels.INTEGER_WORKSPACE,
        "REAL_WORKSPACE": kernels.REAL_WORKSPACE,
    }
    (OUT / "layout.json").write_text(json.dumps(layout, indent=1))
    # The CUDA-C strings as the reference's NVRTC path assembles them
    # (hdbscan_gpu/_cuda.py:18-42), for oracle/ref_cuda.py on a GPU.
    cuda = {
        "header": {p: kernels.header("cuda", p) for p in ("float32", "float64")},
        "distance": kernels.DISTANCE_SOURCE,
        "cluster": kernels.CLUSTER_SOURCE,
        "cluster_threads": kernels.CLUSTER_THREADS,
        "integer_workspace": kernels.INTEGER_WORKSPACE,
        "real_workspace": kernels.REAL_WORKSPACE,
    }
    target = OUT / "ref_cuda_source.json"
    text = json.dumps(cuda)
    if not target.exists() or target.read_text() != text:
        target.write_text(text)
    return True


def build(reference: Path = DEFAULT_REFERENCE) -> Path | None:
    """Generate (when the checkout is present) and compile; None when nothing can be built."""
    generate(reference)
    source = OUT / "ref_kernels.cpp"
    if not source.exists():
        return None
    deps = [source, HERE / "ref_cpu_header.inc", HERE / "ref_driver.inc"]
    if LIBRARY.exists() and LIBRARY.stat().st_mtime >= max(p.stat().st_mtime for p in deps):
        return LIBRARY
    subprocess.run(
        ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
         "-w", "-o", str(LIBRARY), str(source), "-lpthread"],
        check=True,
    )
    return LIBRARY


if __name__ == "__main__":
    path = build(Path(sys.argv[1]) if len(sys.argv) > 1 else DEFAULT_REFERENCE)
    print(path if path else "reference checkout and generated sources absent; nothing built")
