"""Public entry point, a drop-in for hdbscan_gpu.hdbscan(..., backend="cuda").

Validation order and messages follow the reference's hdbscan_gpu/_api.py:11-102
so callers and their tests see the same errors.  Differences, all deliberate:
  * backend "cuda" is the default and the only backend; "mlx" (Apple Metal) is
    rejected with a message naming Metal (the reference's "Metal" error);
  * native device input is a torch CUDA tensor (or any DLPack CUDA producer)
    instead of a CuPy array;
  * there is no 512 MiB dense-distance cap: the fused path never materializes
    the [B, N, N] buffer the reference needed (hdbscan_gpu/_api.py:81-83).
Nothing here imports torch or the CUDA library before validation passes.
"""

from __future__ import annotations

import math
from numbers import Integral, Real

import numpy as np

MAX_SAMPLES = 4096


def _is_native(X) -> bool:
    module = type(X).__module__.split(".")[0]
    if module == "torch":
        return X.device.type == "cuda"
    return hasattr(X, "__dlpack_device__") and not isinstance(X, np.ndarray) and module not in ("numpy",)


def _native_is_numeric(X) -> bool:
    module = type(X).__module__.split(".")[0]
    if module == "torch":
        return not (X.dtype.is_complex or X.dtype == _torch_bool())
    dtype = getattr(X, "dtype", None)
    kind = getattr(dtype, "kind", None)
    return kind is None or kind in "fiu"


def _torch_bool():
    import torch

    return torch.bool


def validate_selection(cluster_selection_method, allow_single_cluster):
    """Checks of the selection options beyond the reference's fixed contract."""
    if cluster_selection_method not in ("eom", "leaf"):
        raise ValueError("cluster_selection_method must be 'eom' or 'leaf'")
    if not isinstance(allow_single_cluster, (bool, np.bool_)):
        raise ValueError("allow_single_cluster must be a bool")
    return cluster_selection_method, bool(allow_single_cluster)


def validate_parameters(min_cluster_size, min_samples, cluster_selection_epsilon, backend, precision):
    """Parameter checks of hdbscan_gpu/_api.py:32-56; returns (mcs, ms, eps)."""
    if backend not in ("mlx", "cuda"):
        raise ValueError("backend must be 'mlx' or 'cuda'")
    if precision not in ("float32", "float64"):
        raise ValueError("precision must be 'float32' or 'float64'")
    if backend == "mlx":
        raise ValueError("the Metal backend (backend='mlx') is not available in hdbscan_gb300; use backend='cuda'")
    for name, value, lower in (
        ("min_cluster_size", min_cluster_size, 2),
        ("min_samples", min_samples, 1),
    ):
        if value is None and name == "min_samples":
            continue
        if isinstance(value, (bool, np.bool_)) or not isinstance(value, Integral):
            raise ValueError(f"{name} must be an integer")
        if value < lower:
            raise ValueError(f"{name} must be >= {lower}")
    if (
        isinstance(cluster_selection_epsilon, (bool, np.bool_))
        or not isinstance(cluster_selection_epsilon, Real)
        or not math.isfinite(cluster_selection_epsilon)
        or cluster_selection_epsilon < 0
    ):
        raise ValueError("cluster_selection_epsilon must be finite and >= 0")
    if min_samples is None:
        min_samples = min_cluster_size
    return min_cluster_size, min_samples, cluster_selection_epsilon


def validate_limits(n, min_cluster_size, min_samples, cluster_selection_epsilon, precision):
    """Limit checks of hdbscan_gpu/_api.py:77-87 (minus the dense-buffer cap)."""
    if n > MAX_SAMPLES:
        raise ValueError(f"at most {MAX_SAMPLES} samples per window are supported")
    if min_samples > n:
        raise ValueError("min_samples must not exceed the number of samples")
    if min_cluster_size > np.iinfo(np.int32).max:
        raise ValueError("min_cluster_size must fit in int32")
    if float(cluster_selection_epsilon) > float(np.finfo(precision).max):
        raise ValueError("cluster_selection_epsilon is not representable in the requested precision")


def hdbscan(
    X,
    *,
    min_cluster_size=5,
    min_samples=None,
    cluster_selection_epsilon=0.0,
    backend="cuda",
    precision="float32",
    cluster_selection_method="eom",
    allow_single_cluster=False,
    return_probabilities=False,
    normalize=False,
):
    """Return device labels for Euclidean EOM HDBSCAN, excluding the root.

    Accepts [N, D] or [B, N, D]; min_samples includes the point itself.
    Host arrays (NumPy, lists, CPU tensors) are explicitly transferred; torch
    CUDA tensors are never copied to the host.  One 4-byte device status read
    validates finite inputs and distances and synchronizes the stream.
    Labels are a new torch.int32 CUDA tensor ([N] or [B, N], -1 noise)
    produced on the caller's current stream.  Windows hold at most 4096
    points.  Float32 rounding can change near-tied hierarchies relative to
    scikit-learn's float64 calculation, exactly as in the reference.

    Beyond the reference's fixed contract (its defaults): cluster_selection_method
    "leaf", allow_single_cluster=True, and return_probabilities=True, which
    returns (labels, probabilities) with scikit-learn's membership strengths
    (a tensor of the requested precision).  normalize=True L2-normalises every
    point first (exact order: sum of squares in coordinate order, correctly
    rounded sqrt and division; zero vectors unchanged), and torch bfloat16 /
    float16 tensors are converted on the device by the same producer stage.
    """
    min_cluster_size, min_samples, cluster_selection_epsilon = validate_parameters(
        min_cluster_size, min_samples, cluster_selection_epsilon, backend, precision)
    cluster_selection_method, allow_single_cluster = validate_selection(cluster_selection_method,
                                                                        allow_single_cluster)

    if _is_native(X):
        if not _native_is_numeric(X):
            raise ValueError("X must contain real numeric values")
    else:
        if type(X).__module__.split(".")[0] == "torch":
            X = X.detach().numpy()  # CPU tensor: a host array
        elif hasattr(X, "__cuda_array_interface__"):
            raise TypeError("use a torch CUDA tensor (or a DLPack CUDA array) or a NumPy host array")
        X = np.asarray(X)
        if X.dtype.kind not in "fiu":
            raise ValueError("X must contain real numeric values")
        if not np.isfinite(X).all():
            raise ValueError("X must contain only finite values")

    if X.ndim not in (2, 3):
        raise ValueError("X must have rank 2 [N,D] or rank 3 [B,N,D]")
    n, dimensions = X.shape[-2:]
    batch = X.shape[0] if X.ndim == 3 else 1
    if batch < 1 or dimensions < 1 or n < 2:
        raise ValueError("X requires nonempty batches/features and at least 2 samples")
    validate_limits(n, min_cluster_size, min_samples, cluster_selection_epsilon, precision)

    from ._cuda import cluster

    # The seam keeps the reference's signature (hdbscan_gpu/_api.py:92-102); the
    # extensions travel as keywords only when they differ from its contract.
    extras = {}
    if cluster_selection_method != "eom":
        extras["method"] = cluster_selection_method
    if allow_single_cluster:
        extras["allow_single_cluster"] = True
    if return_probabilities:
        extras["return_probabilities"] = True
    if not isinstance(normalize, (bool, np.bool_)):
        raise ValueError("normalize must be a bool")
    if normalize:
        extras["normalize"] = True
    return cluster(X, int(min_cluster_size), int(min_samples), float(cluster_selection_epsilon), precision, **extras)
