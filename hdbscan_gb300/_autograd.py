"""Differentiable merge weights (0-dimensional persistence of the mutual-reachability graph).

No reference counterpart: the reference documents "no gradients".  The
forward runs the clustering kernels with exports; the backward kernel
(csrc/hdb_backward.cuh) holds the discrete structure fixed (MST edges, sort
order, core neighbours) and routes each merge weight's gradient through the
distance that attains max(core_u, core_v, d_uv), recomputing that distance
instead of keeping an N^2 buffer.
"""

from __future__ import annotations

import numpy as np
import torch

from ._api import validate_limits, validate_parameters
from ._cuda import plan_for, raise_for_status


class _MergeWeights(torch.autograd.Function):
    @staticmethod
    def forward(ctx, X, plan):
        buffers = plan.export_buffers(hierarchy=False, gradients=True)
        labels, status = plan.forward(X.detach(), exports=buffers)
        raise_for_status(int(status.item()))
        ctx.plan = plan
        ctx.buffers = buffers
        ctx.save_for_backward(X)
        ctx.mark_non_differentiable(labels)
        return buffers["link_w"].clone(), labels

    @staticmethod
    def backward(ctx, grad_w, grad_labels):
        (X,) = ctx.saved_tensors
        if grad_w is None:
            return None, None
        dX = ctx.plan.backward(X.detach(), ctx.buffers, grad_w.contiguous())
        return dX, None


def merge_weights(X, offsets=None, *, min_cluster_size=5, min_samples=None, cluster_selection_epsilon=0.0,
                  precision=None, force_matrix=False):
    """Merge weights (single-linkage 'value' column, linkage order) and labels, differentiable in X.

    X is a CUDA tensor [N, D], [B, N, D] or packed [T, D] with `offsets`.
    Returns (weights, labels): weights [B, N-1] / [N-1] / [T-B] follow the
    input layout; gradients flow from weights to X.
    """
    if not isinstance(X, torch.Tensor) or X.device.type != "cuda":
        raise TypeError("merge_weights needs a torch CUDA tensor")
    precision = precision or ("float64" if X.dtype == torch.float64 else "float32")
    min_cluster_size, min_samples, cluster_selection_epsilon = validate_parameters(
        min_cluster_size, min_samples, cluster_selection_epsilon, "cuda", precision)
    shape = X.shape
    if offsets is None:
        if X.ndim not in (2, 3):
            raise ValueError("X must have rank 2 [N,D] or rank 3 [B,N,D]")
        batch, n = (1, shape[0]) if X.ndim == 2 else (shape[0], shape[1])
        offsets = np.arange(batch + 1, dtype=np.int64) * n
        packed = X.reshape(batch * n, shape[-1])
    else:
        if X.ndim != 2:
            raise ValueError("with offsets, X must be the packed [T, D] windows")
        offsets = np.asarray(offsets, dtype=np.int64)
        packed = X
    sizes = np.diff(offsets)
    validate_limits(int(sizes.max()), min_cluster_size, min_samples, cluster_selection_epsilon, precision)
    if min_samples > int(sizes.min()):
        raise ValueError("min_samples must not exceed the number of samples")
    dtype = torch.float32 if precision == "float32" else torch.float64
    packed = packed.to(dtype)
    with torch.cuda.device(X.device):
        plan = plan_for(offsets, packed.shape[1], min_cluster_size, min_samples, cluster_selection_epsilon,
                        precision, force_matrix)
        weights, labels = _MergeWeights.apply(packed.contiguous(), plan)
    if X.ndim == 3:  # dense [B, N, D]: one row of merge weights / labels per window
        return weights.view(shape[0], shape[1] - 1), labels.view(shape[0], shape[1])
    return weights, labels
