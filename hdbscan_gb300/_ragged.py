"""Ragged batches: windows of different sizes in one persistent launch."""

from __future__ import annotations

import numpy as np

from ._api import validate_limits, validate_parameters, validate_selection


def hdbscan_ragged(windows=None, *, packed=None, offsets=None, min_cluster_size=5, min_samples=None,
                   cluster_selection_epsilon=0.0, precision="float32", return_hierarchy=False,
                   force_matrix=False, cluster_selection_method="eom", allow_single_cluster=False,
                   normalize=False):
    """Cluster a ragged batch in one launch.

    Give either `windows` (a list of [N_i, D] arrays/tensors) or `packed`
    ([sum N_i, D]) with `offsets` ([B+1] row offsets).  Returns
    (labels [sum N_i] int32 CUDA tensor, offsets) and, with
    return_hierarchy=True, a dict of device exports (Prim edges, sort order,
    single-linkage rows, condensed clusters, cores, membership probabilities).
    """
    min_cluster_size, min_samples, cluster_selection_epsilon = validate_parameters(
        min_cluster_size, min_samples, cluster_selection_epsilon, "cuda", precision)
    cluster_selection_method, allow_single_cluster = validate_selection(cluster_selection_method,
                                                                        allow_single_cluster)
    from ._cuda import cluster_ragged, pack, to_device_tensor

    if windows is not None:
        if packed is not None or offsets is not None:
            raise ValueError("give either windows or packed+offsets")
        packed, offsets = pack(windows, precision, keep_half=True)
    else:
        if packed is None or offsets is None:
            raise ValueError("give either windows or packed+offsets")
        packed = to_device_tensor(packed, precision, keep_half=True)
        offsets = np.asarray(offsets, dtype=np.int64)
    if packed.ndim != 2 or packed.shape[1] < 1:
        raise ValueError("X requires nonempty batches/features and at least 2 samples")
    sizes = np.diff(offsets)
    if len(sizes) < 1 or offsets[0] != 0 or offsets[-1] != packed.shape[0] or sizes.min() < 2:
        raise ValueError("X requires nonempty batches/features and at least 2 samples")
    validate_limits(int(sizes.max()), min_cluster_size, min_samples, cluster_selection_epsilon, precision)
    if min_samples > int(sizes.min()):
        raise ValueError("min_samples must not exceed the number of samples")
    result = cluster_ragged(packed, offsets, int(min_cluster_size), int(min_samples),
                            float(cluster_selection_epsilon), precision, exports=return_hierarchy,
                            force_matrix=force_matrix, method=cluster_selection_method,
                            allow_single_cluster=allow_single_cluster, normalize=bool(normalize))
    if return_hierarchy:
        labels, exports = result
        return labels, offsets, exports
    return result, offsets


def condensed_tree(hierarchy, offsets):
    """Per-window condensed trees in scikit-learn's ``condensed_tree_`` columns.

    `hierarchy` is the dict hdbscan_ragged(..., return_hierarchy=True) returns.
    For each window, a dict of device tensors ``parent``, ``child``,
    ``lambda_val`` and ``child_size`` (sklearn/cluster/_hdbscan/_tree.pyx:
    122-237): one row per point (child = point index, size 1) followed by one
    row per condensed cluster except the root (child = cluster id >= n + 1),
    ordered by child.  Only the per-window cluster counts are read back.
    """
    import torch

    offsets = np.asarray(offsets, dtype=np.int64)
    counts = hierarchy["n_clusters"].cpu().numpy()
    device = hierarchy["point_parent"].device
    trees = []
    for w in range(len(offsets) - 1):
        lo, hi = int(offsets[w]), int(offsets[w + 1])
        n, k = hi - lo, int(counts[w])
        clusters = slice(lo + 1, lo + k)  # row c - n of cluster c; the root (c = n) has no row
        trees.append({
            "parent": torch.cat([hierarchy["point_parent"][lo:hi], hierarchy["cl_parent"][clusters]]),
            "child": torch.arange(n + k, dtype=torch.int32, device=device)[torch.arange(n + k, device=device) != n],
            "lambda_val": torch.cat([hierarchy["point_lambda"][lo:hi], hierarchy["cl_birth"][clusters]]),
            "child_size": torch.cat([torch.ones(n, dtype=torch.int32, device=device),
                                     hierarchy["cl_size"][clusters]]),
        })
    return trees
