"""Behaviour contract of the public API on the GPU (the reference's tests/test_api.py:86-287 there)."""

import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle
from tests.conftest import partition_equal

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]
VALUES = np.array([[0], [0.01], [0.02], [3], [3.01], [3.02]], np.float32)
PRECISIONS = ["float32", "float64"]


def _oracle_labels(values, precision, mcs=2, ms=1, eps=0.0):
    return oracle.cluster(np.asarray(values, dtype=np.float64), mcs, ms, eps, precision)["labels"]


def _check_device_labels(labels, shape):
    import torch

    assert isinstance(labels, torch.Tensor) and labels.is_cuda
    assert labels.dtype == torch.int32 and tuple(labels.shape) == shape
    assert (labels >= -1).all()


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("dtype", [np.float16, np.float32, np.float64, np.int32, np.uint32])
def test_host_numeric_dtypes_and_no_mutation(cuda, precision, dtype):
    from hdbscan_gb300 import hdbscan

    values = (VALUES * 100).astype(dtype)
    before = values.copy()
    values.flags.writeable = False
    labels = hdbscan(values, backend="cuda", precision=precision, min_cluster_size=2, min_samples=1)
    _check_device_labels(labels, (6,))
    assert partition_equal(labels.cpu().numpy(), _oracle_labels(values, precision))
    np.testing.assert_array_equal(values, before)


@pytest.mark.parametrize("layout", ["reversed", "column-strided", "fortran", "list"])
def test_host_strides_lists_and_numpy_scalar_parameters(cuda, layout):
    from hdbscan_gb300 import hdbscan

    values = np.concatenate([VALUES, VALUES + 1, VALUES + 2, VALUES + 3], axis=1)
    if layout == "reversed":
        values = values[::-1, ::-1]
    elif layout == "column-strided":
        values = values[:, ::2]
    elif layout == "fortran":
        values = np.asfortranarray(values)
    expected = _oracle_labels(values, "float32")
    result = hdbscan(values.tolist() if layout == "list" else values, backend="cuda",
                     min_cluster_size=np.int64(2), min_samples=np.int32(1), cluster_selection_epsilon=np.float64(0))
    _check_device_labels(result, (6,))
    assert partition_equal(result.cpu().numpy(), expected)


def test_native_strided_views_and_no_mutation(cuda):
    import torch

    from hdbscan_gb300 import hdbscan

    host = np.arange(48, dtype=np.float32).reshape(8, 6)
    native = torch.as_tensor(host, device=cuda)
    views = [native[:, ::2], native.flip(0).flip(1)[:, ::2], native.T, torch.as_tensor(np.stack([host, host + 100]),
                                                                                 device=cuda)[1:]]
    for view in views:
        before = view.cpu().numpy().copy()
        labels = hdbscan(view, backend="cuda", min_cluster_size=2, min_samples=1)
        _check_device_labels(labels, before.shape[:-1])
        np.testing.assert_array_equal(view.cpu().numpy(), before)
        got = labels.cpu().numpy()
        if before.ndim == 2:
            assert partition_equal(got, _oracle_labels(before, "float32"))
        else:
            assert partition_equal(got[0], _oracle_labels(before[0], "float32"))
    np.testing.assert_array_equal(native.cpu().numpy(), host)


@pytest.mark.parametrize("value", [float("nan"), float("inf"), -float("inf")])
def test_native_nonfinite_rejected(cuda, value):
    import torch

    from hdbscan_gb300 import hdbscan

    with pytest.raises(ValueError, match="finite"):
        hdbscan(torch.full((6, 2), value, device=cuda), backend="cuda")


@pytest.mark.parametrize("dtype", ["bool", "complex64"])
def test_native_nonnumeric_rejected(cuda, dtype):
    import torch

    from hdbscan_gb300 import hdbscan

    values = torch.as_tensor(VALUES, device=cuda).to(getattr(torch, dtype))
    with pytest.raises(ValueError, match="real numeric"):
        hdbscan(values, backend="cuda")


@pytest.mark.parametrize("precision", PRECISIONS)
def test_overflow_rejected(cuda, precision):
    from hdbscan_gb300 import hdbscan

    largest = np.finfo(precision).max / 4
    values = np.array([[-largest], [-largest], [largest], [largest]])
    with pytest.raises(ValueError, match="overflow"):
        hdbscan(values, backend="cuda", precision=precision, min_cluster_size=2)


@pytest.mark.parametrize("precision", PRECISIONS)
def test_input_error_outranks_overflow_in_a_later_window(cuda, precision):
    import torch

    from hdbscan_gb300 import hdbscan

    values = np.zeros((3, 33, 1), dtype=precision)
    values[-1, -1, 0] = np.finfo(precision).max
    with pytest.raises(ValueError, match="overflow"):
        hdbscan(torch.as_tensor(values, device=cuda), backend="cuda", precision=precision, min_cluster_size=2)
    values[0, 0, 0] = np.finfo(precision).max
    values[-1, -1, 0] = np.nan
    with pytest.raises(ValueError, match="only finite"):
        hdbscan(torch.as_tensor(values, device=cuda), backend="cuda", precision=precision, min_cluster_size=2)


def test_requested_precision_conversion_rejects_nonfinite(cuda):
    from hdbscan_gb300 import hdbscan

    with pytest.raises(ValueError, match="finite"):
        hdbscan(np.full((6, 1), 1e40, dtype=np.float64), backend="cuda", precision="float32")


def test_nondefault_stream_is_honoured(cuda):
    import torch

    from hdbscan_gb300 import hdbscan

    stream = torch.cuda.Stream(cuda)
    with torch.cuda.stream(stream):
        result = hdbscan(VALUES, backend="cuda", min_cluster_size=2, min_samples=1)
        assert torch.cuda.current_stream(cuda) == stream
    stream.synchronize()
    _check_device_labels(result, (6,))
    assert partition_equal(result.cpu().numpy(), _oracle_labels(VALUES, "float32"))


@pytest.mark.parametrize("precision", PRECISIONS)
def test_batch_individual_and_position_invariance(cuda, precision):
    from hdbscan_gb300 import hdbscan

    rng = np.random.default_rng(31415)
    windows = np.stack([rng.normal(size=(32, 3)), rng.integers(-4, 5, (32, 3)) / 2, np.zeros((32, 3))])
    params = dict(min_cluster_size=3, min_samples=2, cluster_selection_epsilon=0.1, backend="cuda",
                  precision=precision)
    individual = [hdbscan(w, **params).cpu().numpy() for w in windows]
    for order in ([0, 1, 2], [2, 0, 1], [1, 2, 0], [0, 0, 2]):
        result = hdbscan(windows[order], **params).cpu().numpy()
        for position, labels in enumerate(result):
            np.testing.assert_array_equal(labels, individual[order[position]])


def test_graph_replay_and_ragged_api_match_plain_forward(cuda):
    import torch

    from hdbscan_gb300 import Plan, hdbscan_ragged

    rng = np.random.default_rng(9)
    windows = [rng.normal(size=(n, 5)) for n in (40, 700, 129, 2)]
    labels, offsets = hdbscan_ragged(windows, min_cluster_size=3, min_samples=2, precision="float64")
    plan = Plan(offsets, 5, min_cluster_size=3, min_samples=2, precision="float64")
    packed = torch.as_tensor(np.concatenate(windows), device=cuda)
    g_labels, status = plan.capture(packed)
    for _ in range(3):
        plan.replay()
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    np.testing.assert_array_equal(g_labels.cpu().numpy(), labels.cpu().numpy())
    for w, x in enumerate(windows):
        lo, hi = offsets[w], offsets[w + 1]
        np.testing.assert_array_equal(labels.cpu().numpy()[lo:hi], oracle.cluster(x, 3, 2, 0.0, "float64")["labels"])


def test_production_call_imports_no_cpu_clustering_and_keeps_input_on_device(cuda):
    script = r"""
import importlib.abc, sys
import numpy as np
class NoCpuClustering(importlib.abc.MetaPathFinder):
    def find_spec(self, fullname, path=None, target=None):
        if fullname.split(".")[0] in {"sklearn", "hdbscan", "oracle"}:
            raise AssertionError("production imported CPU clustering: " + fullname)
sys.meta_path.insert(0, NoCpuClustering())
import torch
from hdbscan_gb300 import hdbscan
values = torch.tensor([[0], [.01], [.02], [3], [3.01], [3.02]], dtype=torch.float32, device="cuda")
def forbidden(*args, **kwargs):
    raise AssertionError("native device input transferred to the host")
torch.Tensor.cpu = forbidden
torch.Tensor.numpy = forbidden
labels = hdbscan(values, backend="cuda", min_cluster_size=2, min_samples=1)
assert labels.is_cuda and labels.dtype == torch.int32
actual = labels.to("cuda").tolist()
assert len(set(actual[:3])) == len(set(actual[3:])) == 1 and actual[0] != actual[3] and min(actual) >= 0
assert not any(name.split(".")[0] in {"sklearn", "hdbscan", "oracle"} for name in sys.modules)
print("device-only production call passed")
"""
    env = dict(os.environ, PYTHONPATH=str(ROOT))
    result = subprocess.run([sys.executable, "-c", script], cwd=ROOT, env=env, text=True, capture_output=True,
                            timeout=300)
    assert result.returncode == 0, result.stdout + result.stderr
    assert "device-only production call passed" in result.stdout
