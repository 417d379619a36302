"""ctypes front end of the CPU oracle (test infrastructure only).

This module is the checker for the CUDA path: tests/, __graft_entry__.smoke()
and the CPU-baseline leg of bench.py import it.  The product package
(hdbscan_gb300) never imports it and has no CPU fallback.

The oracle restates the reference CUDA path of CosineAI/hdbscan
(hdbscan_gpu/_kernels.py + hdbscan_gpu/_cuda.py:91-128) in serial C; see
hdb_oracle_body.h for the stage-by-stage citations.  Parity of the
restatement is pinned by tests/test_oracle.py against golden vectors made by
tests/golden/make_golden.py from scikit-learn and from the reference kernels
compiled for the CPU (oracle/build_ref.py).
"""

from __future__ import annotations

import ctypes
import os
import subprocess
import threading
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIBRARY = HERE / "libhdb_oracle.so"
_lock = threading.Lock()
_lib = None

_P = ctypes.c_void_p


def build(force: bool = False) -> Path:
    """Compile oracle/libhdb_oracle.so with the committed Makefile."""
    if force or not LIBRARY.exists() or LIBRARY.stat().st_mtime < max(
        (HERE / "hdb_oracle.c").stat().st_mtime, (HERE / "hdb_oracle_body.h").stat().st_mtime
    ):
        subprocess.run(["make", "-s", "-B" if force else "libhdb_oracle.so"], cwd=HERE, check=True)
    return LIBRARY


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            handle = ctypes.CDLL(str(LIBRARY))
            for suffix in ("f32", "f64"):
                fn = getattr(handle, f"hdb_oracle_cluster_{suffix}")
                fn.restype = ctypes.c_int
                fn.argtypes = [_P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                               ctypes.POINTER(_Out)]
                fn = getattr(handle, f"hdb_oracle_cluster_ex_{suffix}")
                fn.restype = ctypes.c_int
                fn.argtypes = [_P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                               ctypes.c_int, ctypes.c_int, ctypes.POINTER(_Out)]
                fn = getattr(handle, f"hdb_oracle_graph_{suffix}")
                fn.restype = None
                fn.argtypes = [_P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.POINTER(_Out)]
                fn = getattr(handle, f"hdb_oracle_batch_{suffix}")
                fn.restype = ctypes.c_int
                fn.argtypes = [_P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                               _P, _P, ctypes.c_int]
                fn = getattr(handle, f"hdb_oracle_batch_ex_{suffix}")
                fn.restype = ctypes.c_int
                fn.argtypes = [_P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                               ctypes.POINTER(_Out), _P, ctypes.c_int]
                fn = getattr(handle, f"hdb_oracle_distances_{suffix}")
                fn.restype = None
                fn.argtypes = [_P, ctypes.c_int, ctypes.c_int, _P]
                fn = getattr(handle, f"hdb_oracle_argsort_{suffix}")
                fn.restype = None
                fn.argtypes = [_P, ctypes.c_int, _P, ctypes.c_int, ctypes.c_int]
            _lib = handle
    return _lib


def _dtype(precision):
    if precision not in ("float32", "float64"):
        raise ValueError("precision must be 'float32' or 'float64'")
    return (np.float32, "f32") if precision == "float32" else (np.float64, "f64")


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def distances(x, precision="float64"):
    dtype, suffix = _dtype(precision)
    x = np.ascontiguousarray(x, dtype=dtype)
    n, d = x.shape
    out = np.empty((n, n), dtype=dtype)
    getattr(lib(), f"hdb_oracle_distances_{suffix}")(_ptr(x), n, d, _ptr(out))
    return out


def argsort(weights, precision=None, depth=None):
    """NumPy-2.3.5 scalar quicksort order of `weights` (optionally forcing the depth limit)."""
    weights = np.asarray(weights)
    precision = precision or ("float32" if weights.dtype == np.float32 else "float64")
    dtype, suffix = _dtype(precision)
    w = np.ascontiguousarray(weights, dtype=dtype)
    order = np.empty(len(w), dtype=np.int32)
    getattr(lib(), f"hdb_oracle_argsort_{suffix}")(_ptr(w), len(w), _ptr(order), int(depth or 0), depth is not None)
    return order


_FIELDS = ("labels", "edges_uv", "edge_w", "order", "link_lr", "link_w", "link_size", "n_clusters",
           "cl_parent", "cl_birth", "cl_stability", "cl_selected", "cl_size", "point_parent", "point_lambda",
           "core", "core_nbr", "probabilities")
METHODS = {"eom": 0, "leaf": 1}


class _Out(ctypes.Structure):
    _fields_ = [(name, ctypes.c_void_p) for name in _FIELDS]


def _outputs(n, dtype):
    m = max(n - 1, 1)
    out = {
        "labels": np.empty(n, np.int32),
        "edges_uv": np.empty((m, 2), np.int32),
        "edge_w": np.empty(m, dtype),
        "order": np.empty(m, np.int32),
        "link_lr": np.empty((m, 2), np.int32),
        "link_w": np.empty(m, dtype),
        "link_size": np.empty(m, np.int32),
        "n_clusters": np.zeros(1, np.int32),
        "cl_parent": np.empty(n, np.int32),
        "cl_birth": np.empty(n, dtype),
        "cl_stability": np.empty(n, dtype),
        "cl_selected": np.empty(n, np.uint8),
        "cl_size": np.empty(n, np.int32),
        "point_parent": np.empty(n, np.int32),
        "point_lambda": np.empty(n, dtype),
        "core": np.empty(n, dtype),
        "core_nbr": np.empty(n, np.int32),
        "probabilities": np.empty(n, dtype),
    }
    struct = _Out(*[out[name].ctypes.data for name in _FIELDS])
    return out, struct


def _trim(out, n):
    k = int(out["n_clusters"][0])
    for key in ("cl_parent", "cl_birth", "cl_stability", "cl_selected", "cl_size"):
        out[key] = out[key][:k]
    for key in ("edges_uv", "edge_w", "order", "link_lr", "link_w", "link_size"):
        out[key] = out[key][: n - 1]
    return out


def cluster(x, min_cluster_size, min_samples=None, epsilon=0.0, precision="float64", method="eom",
            allow_single_cluster=False):
    """Run the whole reference pipeline on one window and return every stage's state.

    method "leaf" and allow_single_cluster=True are the scikit-learn selection
    options beyond the reference's fixed contract (eom, no single cluster)."""
    dtype, suffix = _dtype(precision)
    x = np.ascontiguousarray(x, dtype=dtype)
    if x.ndim != 2:
        raise ValueError("oracle.cluster takes one [N, D] window")
    n, d = x.shape
    ms = min_cluster_size if min_samples is None else min_samples
    out, struct = _outputs(n, dtype)
    status = getattr(lib(), f"hdb_oracle_cluster_ex_{suffix}")(
        _ptr(x), n, d, int(min_cluster_size), int(ms), float(epsilon), METHODS[method],
        int(bool(allow_single_cluster)), ctypes.byref(struct))
    out["status"] = int(status)
    return _trim(out, n)


def normalize_rows(x, precision="float32"):
    """The producer stage's L2 normalisation, restated: s = sum of x_k*x_k in
    coordinate order, x_k / sqrt(s), every operation rounded to nearest in the
    precision (NumPy scalar-type arithmetic, no fused multiply-add); zero
    vectors unchanged."""
    dtype, _ = _dtype(precision)
    x = np.asarray(x, dtype=dtype)
    s = np.zeros(x.shape[0], dtype)
    for k in range(x.shape[1]):
        s = s + x[:, k] * x[:, k]
    r = np.sqrt(s)
    out = x.copy()
    nz = r > 0
    out[nz] = x[nz] / r[nz, None]
    return out


def graph(distances, core, min_cluster_size, epsilon=0.0, precision=None):
    """Hierarchy and labels from a caller-supplied distance matrix; core None = unit core."""
    distances = np.asarray(distances)
    precision = precision or ("float32" if distances.dtype == np.float32 else "float64")
    dtype, suffix = _dtype(precision)
    dist = np.ascontiguousarray(distances, dtype=dtype)
    n = dist.shape[0]
    core_arr = None if core is None else np.ascontiguousarray(core, dtype=dtype)
    out, struct = _outputs(n, dtype)
    getattr(lib(), f"hdb_oracle_graph_{suffix}")(
        _ptr(dist), _ptr(core_arr), n, int(min_cluster_size), float(epsilon), ctypes.byref(struct))
    out["status"] = 0
    out["core"] = core_arr
    return _trim(out, n)


def batch(packed, offsets, min_cluster_size, min_samples=None, epsilon=0.0, precision="float64", threads=None):
    """Labels for a ragged batch: packed [sum N, D] rows, offsets [B+1]; host threads over windows."""
    dtype, suffix = _dtype(precision)
    packed = np.ascontiguousarray(packed, dtype=dtype)
    offsets = np.ascontiguousarray(offsets, dtype=np.int64)
    windows = len(offsets) - 1
    ms = min_cluster_size if min_samples is None else min_samples
    labels = np.empty(int(offsets[-1]), np.int32)
    status = np.zeros(windows, np.int32)
    threads = threads or len(os.sched_getaffinity(0))
    getattr(lib(), f"hdb_oracle_batch_{suffix}")(
        _ptr(packed), _ptr(offsets), windows, packed.shape[1], int(min_cluster_size), int(ms), float(epsilon),
        _ptr(labels), _ptr(status), int(threads),
    )
    return labels, status


def batch_ex(packed, offsets, min_cluster_size, min_samples=None, epsilon=0.0, precision="float64", threads=None):
    """Every stage's state for a ragged batch, packed as the GPU exports are:
    edge rows of window w at offsets[w] - w, point and cluster rows at
    offsets[w], n_clusters[w].  Windows run on host threads."""
    dtype, suffix = _dtype(precision)
    packed = np.ascontiguousarray(packed, dtype=dtype)
    offsets = np.ascontiguousarray(offsets, dtype=np.int64)
    windows = len(offsets) - 1
    T = int(offsets[-1])
    E = max(T - windows, 1)
    ms = min_cluster_size if min_samples is None else min_samples
    out = {
        "labels": np.empty(T, np.int32),
        "edges_uv": np.empty((E, 2), np.int32),
        "edge_w": np.empty(E, dtype),
        "order": np.empty(E, np.int32),
        "link_lr": np.empty((E, 2), np.int32),
        "link_w": np.empty(E, dtype),
        "link_size": np.empty(E, np.int32),
        "n_clusters": np.zeros(windows, np.int32),
        "cl_parent": np.zeros(T, np.int32),
        "cl_birth": np.zeros(T, dtype),
        "cl_stability": np.zeros(T, dtype),
        "cl_selected": np.zeros(T, np.uint8),
        "cl_size": np.zeros(T, np.int32),
        "point_parent": np.empty(T, np.int32),
        "point_lambda": np.empty(T, dtype),
        "core": np.empty(T, dtype),
        "core_nbr": np.empty(T, np.int32),
        "probabilities": np.empty(T, dtype),
    }
    struct = _Out(*[out[name].ctypes.data for name in _FIELDS])
    status = np.zeros(windows, np.int32)
    threads = threads or len(os.sched_getaffinity(0))
    getattr(lib(), f"hdb_oracle_batch_ex_{suffix}")(
        _ptr(packed), _ptr(offsets), windows, packed.shape[1], int(min_cluster_size), int(ms), float(epsilon),
        ctypes.byref(struct), _ptr(status), int(threads))
    out["status"] = status
    return out
