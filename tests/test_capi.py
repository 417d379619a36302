"""The C ABI: every declared entry point is exported and argument checks work without a GPU."""

import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "hdbscan_gb300.h"


def declared_functions():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(hdb_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from hdbscan_gb300 import _lib

    return _lib.lib()


def test_library_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 10
    for name in names:
        assert hasattr(lib, name), f"{name} declared in include/hdbscan_gb300.h but not exported"


def test_python_binding_covers_the_header(lib):
    from hdbscan_gb300 import _lib

    assert set(_lib.SYMBOLS) == set(declared_functions())


def test_version_and_error_message(lib):
    assert lib.hdb_version() == 1
    assert isinstance(lib.hdb_last_error(), bytes)


@pytest.mark.parametrize("kwargs,message", [
    (dict(precision=7), "precision"),
    (dict(mcs=1), "min_cluster_size"),
    (dict(ms=0), "min_samples"),
    (dict(ms=9), "min_samples must not exceed"),
    (dict(eps=-1.0), "epsilon"),
    (dict(eps=float("nan")), "epsilon"),
    (dict(eps=1e39), "representable"),
    (dict(offsets=[0, 1]), "at least 2"),
    (dict(offsets=[0, 5000]), "4096"),
    (dict(offsets=[3, 8]), "start at 0"),
])
def test_plan_argument_validation_needs_no_gpu(lib, kwargs, message):
    import numpy as np

    offsets = np.asarray(kwargs.get("offsets", [0, 8]), dtype=np.int64)
    handle = ctypes.c_void_p()
    rc = lib.hdb_plan_create(ctypes.byref(handle), kwargs.get("precision", 0), len(offsets) - 1,
                             offsets.ctypes.data_as(ctypes.c_void_p), 3, kwargs.get("mcs", 2), kwargs.get("ms", 2),
                             kwargs.get("eps", 0.0), 0)
    assert rc == -1
    assert message in lib.hdb_last_error().decode()
    assert not handle.value


def test_noalloc_rejects_oversized_batches_before_touching_the_device(lib):
    rc = lib.hdb_cluster_noalloc(0, ctypes.c_void_p(16), 65, 4096, 8, 5, 5, 0.0, ctypes.c_void_p(16), None, None)
    assert rc == -1
    assert "no-allocation limit" in lib.hdb_last_error().decode()


def test_committed_tuning_table_names_compiled_variants(lib):
    """Every rule of the committed autotune table names a compiled forward
    variant that can hold its bucket, and the library accepts the table."""
    import json

    from hdbscan_gb300 import _lib, autotune

    table = json.loads(autotune.TABLE.read_text())
    assert table["fields"] == ["precision", "unit_core", "n_max", "d_max", "threads", "slots", "dims", "cluster",
                               "per_sm"]
    compiled = {code: set(autotune.variants(lib, code)) for code in (_lib.HDB_F32, _lib.HDB_F64)}
    assert table["rules"]
    for entry in table["rules"]:
        precision, unit, n_max, d_max, threads, slots, dims, cluster, per_sm = entry["rule"]
        assert (threads, slots, dims, cluster, per_sm) in compiled[precision], entry["rule"]
        assert threads * slots * cluster >= n_max, entry["rule"]
        assert dims == 0 or d_max <= dims, entry["rule"]
        assert unit in (0, 1)
    assert autotune.apply_table(lib) == len(table["rules"])
