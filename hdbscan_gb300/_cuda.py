"""CUDA backend: torch tensors in, the C ABI of libhdbscan_gb300.so underneath.

`cluster()` is the seam the reference calls `cluster(x, min_cluster_size,
min_samples, epsilon, precision)` (hdbscan_gpu/_cuda.py:91-128).  `Plan` is
the ragged/persistent/graph-captured interface the reference lacks: a batch of
windows of different sizes, packed row-wise with offsets, launched as one
CUDA graph of persistent kernels.  torch provides device memory, streams and
DLPack import only; every computation runs in the library's kernels.
"""

from __future__ import annotations

import ctypes
import threading
from collections import OrderedDict

import numpy as np
import torch

from . import _lib

_DTYPES = {"float32": (torch.float32, np.float32, _lib.HDB_F32), "float64": (torch.float64, np.float64, _lib.HDB_F64)}
# Encoder outputs the producer stage converts on the device (exactly).
_HALF_INPUTS = {torch.bfloat16: _lib.HDB_FLAG_INPUT_BF16, torch.float16: _lib.HDB_FLAG_INPUT_F16}


def _stream_handle(device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def _require_gpu():
    if not torch.cuda.is_available() or torch.cuda.device_count() < 1:
        raise RuntimeError("the CUDA backend requires a CUDA GPU")


def raise_for_status(status: int) -> None:
    """Map the device status word to the reference's exceptions (_cuda.py:98-113)."""
    if status & _lib.STATUS_NONFINITE:
        raise ValueError("X must contain only finite values in the requested precision")
    if status & _lib.STATUS_OVERFLOW:
        raise ValueError("pairwise distances overflow the requested precision")
    if status & _lib.STATUS_INTERNAL:
        raise RuntimeError("hdbscan_gb300 device consistency check failed")


class Plan:
    """A compiled batch description: window sizes, dims and parameters.

    Windows are rows offsets[w]..offsets[w+1]-1 of a packed [T, dims] tensor.
    The plan picks kernel variants per window size, sorts windows into
    persistent work queues and owns its device tables' pinned host image.
    """

    def __init__(self, offsets, dims, *, min_cluster_size=5, min_samples=None, cluster_selection_epsilon=0.0,
                 precision="float32", force_matrix=False, one_persistent=False, cluster_selection_method="eom",
                 allow_single_cluster=False, input_dtype=None, normalize=False, device=None, test_flags=0):
        if precision not in _DTYPES:
            raise ValueError("precision must be 'float32' or 'float64'")
        _require_gpu()
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None else
                                   torch.device(device).index or 0)
        self.offsets = np.ascontiguousarray(np.asarray(offsets, dtype=np.int64))
        if self.offsets.ndim != 1 or len(self.offsets) < 2:
            raise ValueError("offsets must be a 1-D array of B+1 row offsets")
        self.windows = len(self.offsets) - 1
        self.points = int(self.offsets[-1])
        self.edges = self.points - self.windows
        self.dims = int(dims)
        self.min_cluster_size = int(min_cluster_size)
        self.min_samples = int(min_cluster_size if min_samples is None else min_samples)
        self.epsilon = float(cluster_selection_epsilon)
        self.precision = precision
        self.torch_dtype, self.numpy_dtype, code = _DTYPES[precision]
        if cluster_selection_method not in ("eom", "leaf"):
            raise ValueError("cluster_selection_method must be 'eom' or 'leaf'")
        self.flags = (_lib.HDB_FLAG_FORCE_MATRIX if force_matrix else 0) | (
            _lib.HDB_FLAG_ONE_PERSISTENT if one_persistent else 0) | (
            _lib.HDB_FLAG_LEAF if cluster_selection_method == "leaf" else 0) | (
            _lib.HDB_FLAG_ALLOW_SINGLE if allow_single_cluster else 0) | (
            _HALF_INPUTS.get(input_dtype, 0)) | (_lib.HDB_FLAG_L2_NORMALIZE if normalize else 0) | int(test_flags)
        if input_dtype is not None and input_dtype not in _HALF_INPUTS and input_dtype != self.torch_dtype:
            raise ValueError("input_dtype must be torch.bfloat16, torch.float16 or the compute precision")
        self.input_dtype = self.torch_dtype if input_dtype is None else input_dtype
        lib = _lib.lib()
        handle = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(lib.hdb_plan_create(ctypes.byref(handle), code, self.windows,
                                           self.offsets.ctypes.data_as(ctypes.c_void_p), self.dims,
                                           self.min_cluster_size, self.min_samples, self.epsilon, self.flags),
                       "hdb_plan_create")
        self._handle = handle
        self.workspace_bytes = int(lib.hdb_plan_workspace_bytes(handle))
        self._graph_keys = None
        self._graph_refs = None

    def __del__(self):
        handle = getattr(self, "_handle", None)
        if handle is not None and handle.value:
            try:
                _lib.lib().hdb_plan_destroy(handle)
            except Exception:
                pass
            self._handle = None

    def describe(self) -> str:
        buf = ctypes.create_string_buffer(1 << 16)
        _lib.check(_lib.lib().hdb_plan_describe(self._handle, buf, len(buf)), "hdb_plan_describe")
        return buf.value.decode()

    # -- buffers -------------------------------------------------------------
    def workspace(self) -> torch.Tensor:
        return torch.empty(max(self.workspace_bytes, 256), dtype=torch.uint8, device=self.device)

    def export_buffers(self, hierarchy=True, gradients=False, probabilities=False) -> dict:
        """Device tensors for hdb_exports_t (edges, linkage, condensed tree, cores, probabilities)."""
        dev, dt = self.device, self.torch_dtype
        E, T, B = max(self.edges, 1), max(self.points, 1), self.windows
        out = {}
        if probabilities:
            out["probabilities"] = torch.empty(T, dtype=dt, device=dev)
        if hierarchy or gradients:
            out.update(
                edges_uv=torch.empty((E, 2), dtype=torch.int32, device=dev),
                edge_w=torch.empty(E, dtype=dt, device=dev),
                order=torch.empty(E, dtype=torch.int32, device=dev),
                link_lr=torch.empty((E, 2), dtype=torch.int32, device=dev),
                link_w=torch.empty(E, dtype=dt, device=dev),
                link_size=torch.empty(E, dtype=torch.int32, device=dev),
            )
        if hierarchy:
            out.update(
                n_clusters=torch.empty(B, dtype=torch.int32, device=dev),
                cl_parent=torch.empty(T, dtype=torch.int32, device=dev),
                cl_birth=torch.empty(T, dtype=dt, device=dev),
                cl_stability=torch.empty(T, dtype=dt, device=dev),
                cl_selected=torch.empty(T, dtype=torch.uint8, device=dev),
                point_parent=torch.empty(T, dtype=torch.int32, device=dev),
                cl_size=torch.empty(T, dtype=torch.int32, device=dev),
                point_lambda=torch.empty(T, dtype=dt, device=dev),
            )
        if self.min_samples > 2:
            out.update(core=torch.empty(T, dtype=dt, device=dev),
                       core_nbr=torch.empty(T, dtype=torch.int32, device=dev))
        return out

    @staticmethod
    def _exports_struct(buffers):
        if not buffers:
            return None
        return _lib.Exports(*[buffers[name].data_ptr() if name in buffers else None for name in _lib.EXPORT_FIELDS])

    def _check_x(self, X: torch.Tensor) -> torch.Tensor:
        if not isinstance(X, torch.Tensor) or X.device != self.device:
            raise ValueError(f"X must be a torch tensor on {self.device}")
        if tuple(X.shape) != (self.points, self.dims):
            raise ValueError(f"X must have shape [{self.points}, {self.dims}]")
        if X.dtype != self.input_dtype or not X.is_contiguous():
            X = X.to(self.input_dtype).contiguous()
        return X

    # -- forward ---------------------------------------------------------------
    def forward(self, X, labels=None, workspace=None, status=None, exports=None):
        """Enqueue the forward on the current stream; returns (labels, status) device tensors."""
        X = self._check_x(X)
        labels = torch.empty(self.points, dtype=torch.int32, device=self.device) if labels is None else labels
        workspace = self.workspace() if workspace is None else workspace
        status = torch.empty(1, dtype=torch.int32, device=self.device) if status is None else status
        ex = self._exports_struct(exports)
        with torch.cuda.device(self.device):
            _lib.check(_lib.lib().hdb_plan_forward(
                self._handle, X.data_ptr(), labels.data_ptr(), workspace.data_ptr(), workspace.numel(),
                status.data_ptr(), ctypes.byref(ex) if ex is not None else None, _stream_handle(self.device)),
                "hdb_plan_forward")
        return labels, status

    def profile(self, X, labels=None, workspace=None, status=None, exports=None):
        """The forward with every launch serialized and timed by CUDA events (synchronizes).
        Returns {phase: (milliseconds, launches)} for prepare/distance/core/forward."""
        X = self._check_x(X)
        labels = torch.empty(self.points, dtype=torch.int32, device=self.device) if labels is None else labels
        workspace = self.workspace() if workspace is None else workspace
        status = torch.empty(1, dtype=torch.int32, device=self.device) if status is None else status
        ex = self._exports_struct(exports)
        ms = (ctypes.c_double * len(_lib.PHASES))()
        launches = (ctypes.c_int32 * len(_lib.PHASES))()
        with torch.cuda.device(self.device):
            _lib.check(_lib.lib().hdb_plan_profile(
                self._handle, X.data_ptr(), labels.data_ptr(), workspace.data_ptr(), workspace.numel(),
                status.data_ptr(), ctypes.byref(ex) if ex is not None else None, _stream_handle(self.device),
                ctypes.cast(ms, ctypes.c_void_p), ctypes.cast(launches, ctypes.c_void_p)), "hdb_plan_profile")
        return {name: (float(ms[i]), int(launches[i])) for i, name in enumerate(_lib.PHASES)}

    def capture(self, X, labels=None, workspace=None, status=None, exports=None):
        """Capture the forward for these buffers into a CUDA graph; returns (labels, status)."""
        X = self._check_x(X)
        labels = torch.empty(self.points, dtype=torch.int32, device=self.device) if labels is None else labels
        workspace = self.workspace() if workspace is None else workspace
        status = torch.empty(1, dtype=torch.int32, device=self.device) if status is None else status
        ex = self._exports_struct(exports)
        stream = torch.cuda.Stream(self.device)
        stream.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.device(self.device):
            _lib.check(_lib.lib().hdb_plan_capture(
                self._handle, X.data_ptr(), labels.data_ptr(), workspace.data_ptr(), workspace.numel(),
                status.data_ptr(), ctypes.byref(ex) if ex is not None else None, stream.cuda_stream),
                "hdb_plan_capture")
        torch.cuda.current_stream(self.device).wait_stream(stream)
        # Keep every captured buffer alive as long as the graph exists.
        self._graph_refs = (X, labels, workspace, status, exports, ex)
        return labels, status

    def replay(self):
        """Launch the captured graph on the current stream."""
        if self._graph_refs is None:
            raise RuntimeError("capture() must be called before replay()")
        with torch.cuda.device(self.device):
            _lib.check(_lib.lib().hdb_plan_replay(self._handle, _stream_handle(self.device)), "hdb_plan_replay")
        return self._graph_refs[1], self._graph_refs[3]

    def backward(self, X, exports, grad, dX=None, workspace=None):
        """dX += d(sum grad * merge_weights)/dX with the forward's structure held fixed."""
        X = self._check_x(X)
        dX = torch.zeros_like(X) if dX is None else dX
        workspace = self.workspace() if workspace is None else workspace
        grad = grad.to(self.torch_dtype).contiguous()
        ex = self._exports_struct(exports)
        with torch.cuda.device(self.device):
            _lib.check(_lib.lib().hdb_plan_backward(
                self._handle, X.data_ptr(), ctypes.byref(ex), grad.data_ptr(), dX.data_ptr(),
                workspace.data_ptr(), workspace.numel(), _stream_handle(self.device)), "hdb_plan_backward")
        return dX


_plan_lock = threading.Lock()
_plans: "OrderedDict[tuple, Plan]" = OrderedDict()


def plan_for(offsets, dims, min_cluster_size, min_samples, epsilon, precision, force_matrix=False, method="eom",
             allow_single_cluster=False, input_dtype=None, normalize=False) -> Plan:
    """Cached Plan for these window sizes and parameters on the current device."""
    offsets = np.asarray(offsets, dtype=np.int64)
    key = (torch.cuda.current_device(), offsets.tobytes(), int(dims), int(min_cluster_size), int(min_samples),
           float(epsilon), precision, bool(force_matrix), method, bool(allow_single_cluster), str(input_dtype),
           bool(normalize))
    with _plan_lock:
        plan = _plans.get(key)
        if plan is None:
            plan = Plan(offsets, dims, min_cluster_size=min_cluster_size, min_samples=min_samples,
                        cluster_selection_epsilon=epsilon, precision=precision, force_matrix=force_matrix,
                        cluster_selection_method=method, allow_single_cluster=allow_single_cluster,
                        input_dtype=input_dtype, normalize=normalize)
            _plans[key] = plan
            if len(_plans) > 32:
                _plans.popitem(last=False)
        else:
            _plans.move_to_end(key)
    return plan


def to_device_tensor(X, precision, keep_half=False) -> torch.Tensor:
    """Native CUDA input stays on the device (cast/contiguous copy only); host input is uploaded.
    keep_half: bfloat16/float16 tensors stay as they are (the producer stage converts them)."""
    torch_dtype, numpy_dtype, _ = _DTYPES[precision]
    if isinstance(X, torch.Tensor):
        if X.device.type != "cuda":
            X = X.to("cuda")
        if keep_half and X.dtype in _HALF_INPUTS:
            return X.contiguous()
        return X.to(torch_dtype).contiguous()
    if hasattr(X, "__dlpack__") and not isinstance(X, np.ndarray):
        return torch.from_dlpack(X).to(torch_dtype).contiguous()
    host = np.ascontiguousarray(np.asarray(X, dtype=numpy_dtype))
    return torch.from_numpy(host).to(device="cuda")


def cluster(x, min_cluster_size, min_samples, epsilon, precision, method="eom", allow_single_cluster=False,
            return_probabilities=False, normalize=False):
    """Labels for [N, D] or [B, N, D] input (the reference's backend seam)."""
    _require_gpu()
    X = to_device_tensor(x, precision, keep_half=True)
    input_dtype = X.dtype if X.dtype in _HALF_INPUTS else None
    with torch.cuda.device(X.device):
        unbatched = X.ndim == 2
        if unbatched:
            X = X[None]
        batch, n, dims = X.shape
        offsets = np.arange(batch + 1, dtype=np.int64) * n
        plan = plan_for(offsets, dims, min_cluster_size, min_samples, epsilon, precision, method=method,
                        allow_single_cluster=allow_single_cluster, input_dtype=input_dtype, normalize=normalize)
        exports = plan.export_buffers(hierarchy=False, probabilities=True) if return_probabilities else None
        labels, status = plan.forward(X.reshape(batch * n, dims), exports=exports)
        raise_for_status(int(status.item()))
        labels = labels.view(batch, n)
        labels = labels[0] if unbatched else labels
        if not return_probabilities:
            return labels
        probs = exports["probabilities"].view(batch, n)
        return labels, (probs[0] if unbatched else probs)


def pack(windows, precision="float32", keep_half=False):
    """Pack a list of [N_i, D] arrays/tensors into (packed [sum N, D] CUDA tensor, offsets int64)."""
    tensors = [to_device_tensor(w, precision, keep_half) for w in windows]
    if not tensors:
        raise ValueError("X requires nonempty batches/features and at least 2 samples")
    dims = {t.shape[-1] for t in tensors}
    if len(dims) != 1 or any(t.ndim != 2 for t in tensors):
        raise ValueError("every window must be [N_i, D] with the same D")
    offsets = np.zeros(len(tensors) + 1, dtype=np.int64)
    offsets[1:] = np.cumsum([t.shape[0] for t in tensors])
    return torch.cat(tensors, 0).contiguous(), offsets


def cluster_ragged(packed, offsets, min_cluster_size, min_samples, epsilon, precision, exports=False,
                   check=True, force_matrix=False, method="eom", allow_single_cluster=False, normalize=False):
    """Labels [sum N] for a ragged batch; optionally the hierarchy exports (with probabilities) too."""
    _require_gpu()
    X = to_device_tensor(packed, precision, keep_half=True)
    input_dtype = X.dtype if X.dtype in _HALF_INPUTS else None
    with torch.cuda.device(X.device):
        plan = plan_for(offsets, X.shape[1], min_cluster_size, min_samples, epsilon, precision, force_matrix,
                        method=method, allow_single_cluster=allow_single_cluster, input_dtype=input_dtype,
                        normalize=normalize)
        buffers = plan.export_buffers(hierarchy=True, gradients=True, probabilities=True) if exports else None
        labels, status = plan.forward(X, exports=buffers)
        if check:
            raise_for_status(int(status.item()))
        return (labels, buffers) if exports else labels
