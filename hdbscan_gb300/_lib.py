"""ctypes binding of libhdbscan_gb300.so (the C ABI of include/hdbscan_gb300.h).

There is no fallback: if the library cannot be built or loaded, every call
raises.  The library is compiled in-tree by hdbscan_gb300/_build.py.
"""

from __future__ import annotations

import ctypes
import threading

from . import _build

HDB_F32 = 0
HDB_F64 = 1
HDB_FLAG_FORCE_MATRIX = 1
HDB_FLAG_NO_GRAPH_STREAMS = 2
HDB_FLAG_ONE_PERSISTENT = 4
HDB_FLAG_LEAF = 8
HDB_FLAG_ALLOW_SINGLE = 16
HDB_FLAG_INPUT_BF16 = 32
HDB_FLAG_INPUT_F16 = 64
HDB_FLAG_L2_NORMALIZE = 128
HDB_FLAG_TEST_STALL = 256
STATUS_OVERFLOW = 1
STATUS_NONFINITE = 2
STATUS_INTERNAL = 4
PHASES = ("prepare", "distance", "core", "forward")

_P = ctypes.c_void_p
_lock = threading.Lock()
_lib = None

EXPORT_FIELDS = ("edges_uv", "edge_w", "order", "link_lr", "link_w", "link_size", "n_clusters", "cl_parent",
                 "cl_birth", "cl_stability", "cl_selected", "point_parent", "core", "core_nbr", "stage_ns",
                 "probabilities", "cl_size", "point_lambda")


class Exports(ctypes.Structure):
    """hdb_exports_t: optional device output pointers of a forward call."""

    _fields_ = [(name, ctypes.c_void_p) for name in EXPORT_FIELDS]


class HDBError(RuntimeError):
    """A C-ABI call returned a nonzero code."""


def _declare(handle):
    sig = {
        "hdb_version": (ctypes.c_int, []),
        "hdb_last_error": (ctypes.c_char_p, []),
        "hdb_set_tuning": (ctypes.c_int, [_P, ctypes.c_int]),
        "hdb_get_tuning": (ctypes.c_int, [_P, ctypes.c_int]),
        "hdb_list_variants": (ctypes.c_int, [ctypes.c_int, _P, ctypes.c_int]),
        "hdb_plan_create": (ctypes.c_int, [ctypes.POINTER(_P), ctypes.c_int, ctypes.c_int, _P, ctypes.c_int,
                                           ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_uint]),
        "hdb_plan_destroy": (ctypes.c_int, [_P]),
        "hdb_plan_workspace_bytes": (ctypes.c_size_t, [_P]),
        "hdb_plan_describe": (ctypes.c_int, [_P, ctypes.c_char_p, ctypes.c_size_t]),
        "hdb_plan_forward": (ctypes.c_int, [_P, _P, _P, _P, ctypes.c_size_t, _P, ctypes.POINTER(Exports), _P]),
        "hdb_plan_capture": (ctypes.c_int, [_P, _P, _P, _P, ctypes.c_size_t, _P, ctypes.POINTER(Exports), _P]),
        "hdb_plan_replay": (ctypes.c_int, [_P, _P]),
        "hdb_plan_profile": (ctypes.c_int, [_P, _P, _P, _P, ctypes.c_size_t, _P, ctypes.POINTER(Exports), _P, _P,
                                            _P]),
        "hdb_plan_backward": (ctypes.c_int, [_P, _P, ctypes.POINTER(Exports), _P, _P, _P, ctypes.c_size_t, _P]),
        "hdb_cluster_workspace_bytes": (ctypes.c_size_t, [ctypes.c_int] * 6),
        "hdb_cluster_f32": (ctypes.c_int, [_P] + [ctypes.c_int] * 5 + [ctypes.c_double, _P, _P, ctypes.c_size_t,
                                                                        _P, _P]),
        "hdb_cluster_f64": (ctypes.c_int, [_P] + [ctypes.c_int] * 5 + [ctypes.c_double, _P, _P, ctypes.c_size_t,
                                                                        _P, _P]),
        "hdb_cluster_noalloc": (ctypes.c_int, [ctypes.c_int, _P] + [ctypes.c_int] * 5 + [ctypes.c_double, _P, _P,
                                                                                          _P]),
    }
    for name, (restype, argtypes) in sig.items():
        fn = getattr(handle, name)
        fn.restype = restype
        fn.argtypes = argtypes
    return sig


# Every symbol include/hdbscan_gb300.h declares.
SYMBOLS = ("hdb_version", "hdb_last_error", "hdb_set_tuning", "hdb_get_tuning", "hdb_list_variants",
           "hdb_plan_create", "hdb_plan_destroy", "hdb_plan_workspace_bytes",
           "hdb_plan_describe", "hdb_plan_forward", "hdb_plan_profile", "hdb_plan_capture", "hdb_plan_replay",
           "hdb_plan_backward",
           "hdb_cluster_workspace_bytes", "hdb_cluster_f32", "hdb_cluster_f64", "hdb_cluster_noalloc")


def lib():
    """Build (if stale) and load the library; raises if that is impossible."""
    global _lib
    with _lock:
        if _lib is None:
            path = _build.build()
            handle = ctypes.CDLL(str(path))
            _declare(handle)
            _lib = handle
            from . import autotune

            autotune.apply_table(handle)
    return _lib


def check(rc: int, what: str) -> None:
    if rc != 0:
        message = lib().hdb_last_error().decode(errors="replace")
        if rc == -1:
            raise ValueError(message or what)
        raise HDBError(f"{what} failed ({rc}): {message}")
