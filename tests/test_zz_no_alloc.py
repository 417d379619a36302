"""hdb_cluster_noalloc: clustering for callers that cannot allocate device memory.

Some callers may not call cudaMalloc where they cluster -- their device
memory belongs to a pool reserved at start-up, or to the allocator of a host
framework they run inside -- so they cannot supply the workspace the planned
entry points take.  hdb_cluster_noalloc keeps its scratch in a fixed array
inside the library instead.  These tests call it through the C ABI and check
that its labels equal those of the planned entry point (hdb_cluster_f32/_f64)
exactly, on two calls in a row: the second call must rebuild, not trust, the
scratch the first call left behind.  The file runs last so that a failure here
stops a `-x` run only after every other test has run.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bind(lib):
    fn = lib.hdb_cluster_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                   ctypes.c_int, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    return fn


def _windows(seed, batch, n, dims):
    rng = np.random.default_rng(seed)
    centres = rng.uniform(-4, 4, (5, dims))
    x = centres[rng.integers(0, 5, (batch, n))] + rng.normal(0, 0.4, (batch, n, dims))
    return x


def _compare_with_planned(cuda, precision, min_samples, shapes, seed=100):
    """Labels of hdb_cluster_noalloc equal hdb_cluster_f32/_f64's, one call per shape, in order."""
    import torch

    from hdbscan_gb300 import _lib

    lib = _lib.lib()
    noalloc = _bind(lib)
    code = _lib.HDB_F32 if precision == "float32" else _lib.HDB_F64
    planned = lib.hdb_cluster_f32 if precision == "float32" else lib.hdb_cluster_f64
    dtype = torch.float32 if precision == "float32" else torch.float64
    stream = torch.cuda.current_stream(cuda).cuda_stream
    mcs, eps = 5, 0.1
    for call, (batch, n, dims) in enumerate(shapes):
        X = torch.as_tensor(_windows(seed + call, batch, n, dims), dtype=dtype, device=cuda).contiguous()
        ws_bytes = lib.hdb_cluster_workspace_bytes(code, batch, n, dims, mcs, min_samples)
        assert ws_bytes > 0, lib.hdb_last_error()
        workspace = torch.empty(ws_bytes, dtype=torch.uint8, device=cuda)
        want = torch.empty((batch, n), dtype=torch.int32, device=cuda)
        want_status = torch.empty(1, dtype=torch.int32, device=cuda)
        rc = planned(X.data_ptr(), batch, n, dims, mcs, min_samples, eps, want.data_ptr(), workspace.data_ptr(),
                     ws_bytes, want_status.data_ptr(), stream)
        assert rc == 0, lib.hdb_last_error()
        got = torch.full((batch, n), -7, dtype=torch.int32, device=cuda)
        got_status = torch.full((1,), -7, dtype=torch.int32, device=cuda)
        rc = noalloc(code, X.data_ptr(), batch, n, dims, mcs, min_samples, eps, got.data_ptr(),
                     got_status.data_ptr(), stream)
        assert rc == 0, lib.hdb_last_error()
        torch.cuda.synchronize()
        assert int(want_status.item()) == 0 and int(got_status.item()) == 0
        assert torch.equal(got, want), f"call {call} {(batch, n, dims)}: labels differ from the planned entry point"


@pytest.mark.parametrize("precision,min_samples", [("float32", 2), ("float32", 5), ("float64", 4)])
def test_noalloc_labels_equal_planned_entry_on_two_calls(cuda, precision, min_samples):
    _compare_with_planned(cuda, precision, min_samples, [(6, 300, 8), (4, 520, 12)])


@pytest.mark.parametrize("precision,min_samples,shapes", [
    # 80 > 64 nearest neighbours: the core distances come from the select kernel.
    ("float32", 80, [(3, 300, 6), (2, 400, 6)]),
    ("float64", 80, [(3, 300, 6), (2, 400, 6)]),
    # Windows of 1025-2048 points (4 slots per Prim thread) and above 2048 (8 slots).
    ("float32", 5, [(4, 1500, 12), (2, 3000, 8)]),
    ("float64", 4, [(4, 1500, 8), (3, 1100, 8)]),
])
def test_noalloc_select_kernel_and_large_windows(cuda, precision, min_samples, shapes):
    _compare_with_planned(cuda, precision, min_samples, shapes, seed=200)


def _refusal(cuda, precision, batch, n, dims, epsilon=0.0):
    import torch

    from hdbscan_gb300 import _lib

    lib = _lib.lib()
    noalloc = _bind(lib)
    X = torch.zeros(8, dtype=torch.float32, device=cuda)
    labels = torch.zeros(8, dtype=torch.int32, device=cuda)
    code = _lib.HDB_F32 if precision == "float32" else _lib.HDB_F64
    rc = noalloc(code, X.data_ptr(), batch, n, dims, 5, 5, epsilon, labels.data_ptr(), None,
                 torch.cuda.current_stream(cuda).cuda_stream)
    return rc, lib.hdb_last_error().decode()


def test_noalloc_rejects_batches_beyond_its_scratch(cuda):
    rc, message = _refusal(cuda, "float32", 65, 4096, 8)
    assert rc == -1
    assert "no-allocation limit" in message


@pytest.mark.parametrize("precision,n,dims,limit", [
    ("float32", 1500, 17, "at most 16 dims"),
    ("float32", 3000, 9, "at most 8 dims"),
    ("float32", 1000, 33, "at most 32 dims"),
    ("float64", 1500, 9, "at most 8 dims"),
    ("float64", 3000, 4, "not supported"),
])
def test_noalloc_rejects_dims_beyond_its_limit(cuda, precision, n, dims, limit):
    rc, message = _refusal(cuda, precision, 1, n, dims)
    assert rc == -1
    assert "no-allocation limit" in message and limit in message, message


def test_noalloc_rejects_epsilon_beyond_float32(cuda):
    rc, message = _refusal(cuda, "float32", 1, 100, 4, epsilon=1e39)
    assert rc == -1
    assert "representable" in message
