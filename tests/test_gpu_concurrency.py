"""The dense C-ABI entry points under concurrent use.

hdb_cluster_f32/_f64 keep a cache of plans per shape.  Two host threads on two
streams call the same shape while a third thread cycles through more shapes
than the cache holds, so plans are evicted while others are in use.  Every
call's labels must equal those of a serial run: a call must join its own
forward, and eviction must never free a plan another thread still uses.
"""

import ctypes
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _windows(seed, batch, n, dims):
    rng = np.random.default_rng(seed)
    centres = rng.uniform(-4, 4, (6, dims))
    return centres[rng.integers(0, 6, (batch, n))] + rng.normal(0, 0.4, (batch, n, dims))


def test_two_threads_two_streams_with_cache_churn(cuda):
    import torch

    from hdbscan_gb300 import _lib

    lib = _lib.lib()
    batch, n, dims, mcs, ms, eps = 24, 700, 8, 5, 4, 0.05
    calls = 50
    X = torch.as_tensor(_windows(1, batch, n, dims), dtype=torch.float32, device=cuda).contiguous()
    ws_bytes = lib.hdb_cluster_workspace_bytes(_lib.HDB_F32, batch, n, dims, mcs, ms)
    assert ws_bytes > 0, lib.hdb_last_error()

    def run(stream, out, workspace, status):
        rc = lib.hdb_cluster_f32(X.data_ptr(), batch, n, dims, mcs, ms, eps, out.data_ptr(), workspace.data_ptr(),
                                 ws_bytes, status.data_ptr(), stream.cuda_stream)
        return rc

    serial = torch.empty((batch, n), dtype=torch.int32, device=cuda)
    ws0 = torch.empty(ws_bytes, dtype=torch.uint8, device=cuda)
    st0 = torch.empty(1, dtype=torch.int32, device=cuda)
    assert run(torch.cuda.current_stream(cuda), serial, ws0, st0) == 0, lib.hdb_last_error()
    torch.cuda.synchronize()
    assert int(st0.item()) == 0
    expected = serial.cpu()

    errors = []
    results = {0: [], 1: []}
    streams = [torch.cuda.Stream(cuda), torch.cuda.Stream(cuda)]
    # Every buffer a worker touches is made here, before the threads start.
    buffers = [[(torch.empty((batch, n), dtype=torch.int32, device=cuda),
                 torch.empty(ws_bytes, dtype=torch.uint8, device=cuda),
                 torch.empty(1, dtype=torch.int32, device=cuda)) for _ in range(2)] for _ in range(2)]
    churn_shapes = [(1, 40 + 3 * i, 4) for i in range(20)]
    churn_inputs = [torch.as_tensor(_windows(100 + i, *shape), dtype=torch.float32, device=cuda).contiguous()
                    for i, shape in enumerate(churn_shapes)]
    churn_ws = []
    for shape in churn_shapes:
        size = lib.hdb_cluster_workspace_bytes(_lib.HDB_F32, shape[0], shape[1], shape[2], 5, 4)
        churn_ws.append(torch.empty(max(size, 256), dtype=torch.uint8, device=cuda))
    churn_stream = torch.cuda.Stream(cuda)
    torch.cuda.synchronize()
    stop = threading.Event()

    def worker(index):
        try:
            torch.cuda.set_device(cuda)
            stream = streams[index]
            for call in range(calls):
                out, workspace, status = buffers[index][call % 2]
                # The previous use of this buffer pair was read back below, so
                # nothing on the GPU still touches it.
                rc = run(stream, out, workspace, status)
                if rc:
                    errors.append(lib.hdb_last_error().decode())
                    return
                stream.synchronize()
                results[index].append((int(status.item()), torch.equal(out.cpu(), expected)))
        except Exception as error:  # reported by the main thread
            errors.append(repr(error))

    def churn():
        try:
            torch.cuda.set_device(cuda)
            i = 0
            while not stop.is_set():
                k = i % len(churn_shapes)
                b, m, d = churn_shapes[k]
                labels = torch.empty((b, m), dtype=torch.int32, device=cuda)
                status = torch.empty(1, dtype=torch.int32, device=cuda)
                rc = lib.hdb_cluster_f32(churn_inputs[k].data_ptr(), b, m, d, 5, 4, 0.0, labels.data_ptr(),
                                         churn_ws[k].data_ptr(), churn_ws[k].numel(), status.data_ptr(),
                                         churn_stream.cuda_stream)
                if rc:
                    errors.append(lib.hdb_last_error().decode())
                    return
                churn_stream.synchronize()
                i += 1
        except Exception as error:
            errors.append(repr(error))

    threads = [threading.Thread(target=worker, args=(i,)) for i in range(2)]
    churner = threading.Thread(target=churn)
    churner.start()
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=600)
    stop.set()
    churner.join(timeout=600)
    torch.cuda.synchronize()
    assert not errors, errors
    for index in (0, 1):
        assert len(results[index]) == calls
        assert all(status == 0 for status, _ in results[index])
        assert all(same for _, same in results[index]), f"thread {index}: labels differ from the serial run"
