"""Batched, device-resident HDBSCAN for one NVIDIA GB300 (sm_103a).

Drop-in for the CUDA path of CosineAI/hdbscan's ``hdbscan_gpu.hdbscan``:
the same keyword arguments, validation messages and int32 labels, computed by
hand-written CUDA kernels behind a C ABI (include/hdbscan_gb300.h).
Additions: ragged batches (``hdbscan_ragged``/``Plan``), CUDA-graph replay,
hierarchy exports and differentiable merge weights (``merge_weights``).
"""

from ._api import MAX_SAMPLES, hdbscan

__all__ = ["hdbscan", "hdbscan_ragged", "condensed_tree", "Plan", "merge_weights", "MAX_SAMPLES"]


def __getattr__(name):
    # torch-dependent parts load lazily so that validation imports nothing heavy.
    if name == "Plan":
        from ._cuda import Plan

        return Plan
    if name == "hdbscan_ragged":
        from ._ragged import hdbscan_ragged

        return hdbscan_ragged
    if name == "condensed_tree":
        from ._ragged import condensed_tree

        return condensed_tree
    if name == "merge_weights":
        from ._autograd import merge_weights

        return merge_weights
    raise AttributeError(name)
