"""Validation of the public entry point (no GPU needed).

Mirrors the reference's behaviour contract (tests/test_api.py:15-83 there):
the same ValueError substrings, checked before any backend import.  The
deliberate differences of this build are tested too: "cuda" is the only
backend ("mlx" names Metal), and there is no 512 MiB dense-buffer cap.
"""

import builtins

import numpy as np
import pytest

from hdbscan_gb300 import MAX_SAMPLES, hdbscan

VALUES = np.array([[0], [0.01], [0.02], [3], [3.01], [3.02]], np.float32)


@pytest.mark.parametrize("parameters,match", [
    ({"backend": "cpu"}, "backend"),
    ({"backend": "auto"}, "backend"),
    ({"backend": "CUDA"}, "backend"),
    ({"backend": None}, "backend"),
    ({"precision": "float16"}, "precision"),
    ({"precision": np.float32}, "precision"),
    ({"precision": "float64", "backend": "mlx"}, "Metal"),
    ({"backend": "mlx"}, "Metal"),
    ({"min_cluster_size": 1}, "min_cluster_size"),
    ({"min_cluster_size": 2.0}, "min_cluster_size"),
    ({"min_cluster_size": True}, "min_cluster_size"),
    ({"min_cluster_size": np.bool_(True)}, "min_cluster_size"),
    ({"min_cluster_size": None}, "min_cluster_size"),
    ({"min_cluster_size": 2**31, "min_samples": 1}, "int32"),
    ({"min_samples": 0}, "min_samples"),
    ({"min_samples": -1}, "min_samples"),
    ({"min_samples": 2.0}, "min_samples"),
    ({"min_samples": True}, "min_samples"),
    ({"min_samples": np.bool_(True)}, "min_samples"),
    ({"min_samples": 7}, "min_samples"),
    ({"cluster_selection_epsilon": -0.1}, "epsilon"),
    ({"cluster_selection_epsilon": float("nan")}, "epsilon"),
    ({"cluster_selection_epsilon": float("inf")}, "epsilon"),
    ({"cluster_selection_epsilon": True}, "epsilon"),
    ({"cluster_selection_epsilon": "0.1"}, "epsilon"),
    ({"cluster_selection_epsilon": 1e40}, "representable"),
])
def test_parameter_validation_without_backend_import(monkeypatch, parameters, match):
    original_import = builtins.__import__

    def no_backend_import(name, *args, **kwargs):
        if name in ("torch", "hdbscan_gb300._cuda", "_cuda") or (name == "" and "_cuda" in str(args)):
            raise AssertionError(f"invalid parameters reached the backend: {name}")
        return original_import(name, *args, **kwargs)

    monkeypatch.setattr(builtins, "__import__", no_backend_import)
    with pytest.raises(ValueError, match=match):
        hdbscan(VALUES, **parameters)


@pytest.mark.parametrize("values,match", [
    (np.zeros(6), "rank"),
    (np.array(0), "rank"),
    (np.zeros((1, 2, 3, 4)), "rank"),
    (np.zeros((0, 2)), "at least 2"),
    (np.zeros((1, 2)), "at least 2"),
    (np.zeros((2, 0)), "nonempty"),
    (np.zeros((0, 6, 2)), "nonempty"),
    (np.zeros((6, 2), dtype=bool), "real numeric"),
    (np.ones((6, 2), dtype=complex), "real numeric"),
    (np.full((6, 2), "1"), "real numeric"),
    (np.full((6, 2), object(), dtype=object), "real numeric"),
    (np.full((6, 2), np.nan), "finite"),
    (np.full((6, 2), np.inf), "finite"),
    (np.full((6, 2), -np.inf), "finite"),
    (np.zeros((MAX_SAMPLES + 1, 1), np.float32), "4096"),
])
def test_host_input_validation(values, match):
    with pytest.raises(ValueError, match=match):
        hdbscan(values, min_cluster_size=2, min_samples=1)


def test_no_dense_buffer_cap_in_validation(monkeypatch):
    # The reference rejects [5, 4096, 1] with "512 MiB" (its dense [B,N,N]
    # buffers); this build never allocates them, so validation lets it through
    # to the backend.
    import hdbscan_gb300._api as api

    reached = {}

    def fake_cluster(x, mcs, ms, eps, precision):
        reached["shape"] = np.shape(x)
        return "backend reached"

    import types

    fake = types.ModuleType("hdbscan_gb300._cuda")
    fake.cluster = fake_cluster
    monkeypatch.setitem(__import__("sys").modules, "hdbscan_gb300._cuda", fake)
    values = np.broadcast_to(np.float32(0), (5, 4096, 1))
    assert api.hdbscan(values, min_cluster_size=2, min_samples=1) == "backend reached"
    assert reached["shape"] == (5, 4096, 1)


def test_default_min_samples_is_min_cluster_size(monkeypatch):
    import sys
    import types

    calls = {}
    fake = types.ModuleType("hdbscan_gb300._cuda")
    fake.cluster = lambda x, mcs, ms, eps, precision: calls.setdefault("args", (mcs, ms, eps, precision))
    monkeypatch.setitem(sys.modules, "hdbscan_gb300._cuda", fake)
    hdbscan(VALUES, min_cluster_size=4, backend="cuda", precision="float64", cluster_selection_epsilon=np.float64(0))
    assert calls["args"] == (4, 4, 0.0, "float64")


@pytest.mark.parametrize("kwargs,match", [
    (dict(cluster_selection_method="dbscan"), "cluster_selection_method"),
    (dict(allow_single_cluster=1), "allow_single_cluster"),
])
def test_selection_option_validation(kwargs, match):
    from hdbscan_gb300 import _api as api

    with pytest.raises(ValueError, match=match):
        api.hdbscan(np.zeros((4, 2)), min_cluster_size=2, **kwargs)


def test_selection_options_reach_the_backend_only_when_set(monkeypatch):
    from hdbscan_gb300 import _api as api
    from hdbscan_gb300 import _cuda

    seen = []
    monkeypatch.setattr(_cuda, "cluster", lambda *args, **kwargs: seen.append(kwargs) or "ok")
    x = np.arange(12, dtype=float).reshape(6, 2)
    api.hdbscan(x, min_cluster_size=2)
    api.hdbscan(x, min_cluster_size=2, cluster_selection_method="leaf", allow_single_cluster=True,
                return_probabilities=True)
    assert seen == [{}, {"method": "leaf", "allow_single_cluster": True, "return_probabilities": True}]
