"""CUDA path vs the CPU oracle, bit-exact on every exported stage.

The oracle (oracle/hdb_oracle_body.h) restates the reference kernels
(hdbscan_gpu/_kernels.py); it is pinned to the reference and scikit-learn by
tests/test_oracle.py.  Here every intermediate the reference's kernel tests
inspect (tests/test_kernels.py:301-380 of the reference) is compared exactly:
Prim edges and weights, sort order, linkage rows, condensed clusters, labels.
"""

import numpy as np
import pytest

from oracle import oracle

pytestmark = pytest.mark.gpu


def _windows(seed, count, n_range, dims):
    rng = np.random.default_rng(seed)
    out = []
    for w in range(count):
        n = int(rng.integers(*n_range))
        kind = w % 4
        if kind == 0:
            x = rng.integers(-3, 4, (n, dims)) / 2.0
        elif kind == 1:
            x = rng.normal(size=(n, dims))
        elif kind == 2:
            centers = rng.normal(0, 4, (4, dims))
            x = centers[np.arange(n) % 4] + rng.normal(0, 0.2, (n, dims))
        else:
            x = np.repeat(rng.normal(size=(max(n // 3, 1), dims)), 3, axis=0)[:n]
            if len(x) < n:
                x = np.concatenate([x, rng.normal(size=(n - len(x), dims))])
        out.append(x)
    return out


def _run(windows, mcs, ms, eps, precision, force_matrix=False):
    import torch

    from hdbscan_gb300._cuda import cluster_ragged, pack

    packed, offsets = pack([np.asarray(w) for w in windows], precision)
    labels, ex = cluster_ragged(packed, offsets, mcs, ms, eps, precision, exports=True,
                                force_matrix=force_matrix)
    torch.cuda.synchronize()
    host = {k: v.cpu().numpy() for k, v in ex.items()}
    return labels.cpu().numpy(), host, offsets


def _compare(windows, mcs, ms, eps, precision, force_matrix=False):
    labels, ex, offsets = _run(windows, mcs, ms, eps, precision, force_matrix)
    dtype = np.float32 if precision == "float32" else np.float64
    for w, x in enumerate(windows):
        o = oracle.cluster(np.asarray(x, dtype=dtype), mcs, ms, eps, precision)
        lo, hi = offsets[w], offsets[w + 1]
        n = hi - lo
        e0, e1 = lo - w, hi - w - 1
        ctx = f"window {w} n={n} mcs={mcs} ms={ms} eps={eps} {precision} matrix={force_matrix}"
        np.testing.assert_array_equal(ex["edges_uv"][e0:e1], o["edges_uv"], err_msg=ctx)
        np.testing.assert_array_equal(ex["edge_w"][e0:e1].view(np.uint8), o["edge_w"].view(np.uint8), err_msg=ctx)
        np.testing.assert_array_equal(ex["order"][e0:e1], o["order"], err_msg=ctx)
        np.testing.assert_array_equal(ex["link_lr"][e0:e1], o["link_lr"], err_msg=ctx)
        np.testing.assert_array_equal(ex["link_w"][e0:e1].view(np.uint8), o["link_w"].view(np.uint8), err_msg=ctx)
        np.testing.assert_array_equal(ex["link_size"][e0:e1], o["link_size"], err_msg=ctx)
        k = int(ex["n_clusters"][w])
        assert k == len(o["cl_parent"]), ctx
        np.testing.assert_array_equal(ex["cl_parent"][lo:lo + k], o["cl_parent"], err_msg=ctx)
        np.testing.assert_array_equal(ex["cl_birth"][lo:lo + k].view(np.uint8), o["cl_birth"].view(np.uint8),
                                      err_msg=ctx)
        np.testing.assert_array_equal(ex["cl_stability"][lo:lo + k].view(np.uint8),
                                      o["cl_stability"].view(np.uint8), err_msg=ctx)
        np.testing.assert_array_equal(ex["cl_selected"][lo:lo + k], o["cl_selected"], err_msg=ctx)
        np.testing.assert_array_equal(ex["point_parent"][lo:hi], o["point_parent"], err_msg=ctx)
        if ms > 2:
            np.testing.assert_array_equal(ex["core"][lo:hi].view(np.uint8), o["core"].view(np.uint8), err_msg=ctx)
        np.testing.assert_array_equal(labels[lo:hi], o["labels"], err_msg=ctx)


@pytest.mark.parametrize("precision", ["float32", "float64"])
@pytest.mark.parametrize("mcs,ms,eps", [(2, 1, 0.0), (2, 2, 0.1), (5, 5, 0.0), (7, 3, 0.5), (3, 10, 0.1)])
def test_small_ragged_batch_matches_oracle(cuda, precision, mcs, ms, eps):
    _compare(_windows(11, 12, (12, 300), 3), mcs, ms, eps, precision)


@pytest.mark.parametrize("precision", ["float32", "float64"])
@pytest.mark.parametrize("force_matrix", [False, True])
def test_size_classes_match_oracle(cuda, precision, force_matrix):
    # One window per size class boundary (128/256/512/1024/2048/4096).
    rng = np.random.default_rng(7)
    sizes = [4, 5, 128, 129, 256, 257, 512, 513, 1024, 1025, 2048, 2049]
    windows = [rng.normal(size=(n, 5)) for n in sizes]
    _compare(windows, 5, 4, 0.1, precision, force_matrix)


@pytest.mark.parametrize("precision", ["float32", "float64"])
@pytest.mark.parametrize("ms", [1, 2])
def test_two_and_three_point_windows(cuda, precision, ms):
    rng = np.random.default_rng(ms)
    windows = [rng.normal(size=(n, 2)) for n in (2, 3, 2, 3, 4)]
    _compare(windows, 2, ms, 0.1, precision)


@pytest.mark.parametrize("precision", ["float32", "float64"])
@pytest.mark.parametrize("dims", [1, 8, 9, 16, 17, 32, 33, 64])
def test_dimension_variants_match_oracle(cuda, precision, dims):
    _compare(_windows(dims, 6, (40, 700), dims), 4, 3, 0.05, precision)


@pytest.mark.parametrize("precision", ["float32", "float64"])
def test_large_min_samples_select_kernel(cuda, precision):
    _compare(_windows(3, 4, (100, 400), 4), 10, 70, 0.0, precision)


@pytest.mark.parametrize("precision", ["float32", "float64"])
def test_max_window_4096(cuda, precision):
    rng = np.random.default_rng(4096)
    centers = rng.normal(0, 3, (6, 8))
    x = centers[np.arange(4096) % 6] + rng.normal(0, 0.3, (4096, 8))
    _compare([x], 16, 8, 0.0, precision)


@pytest.mark.parametrize("precision", ["float32", "float64"])
@pytest.mark.parametrize("ms", [20, 40])
def test_long_core_lists_match_oracle(cuda, precision, ms):
    # 32- and 64-entry k-nearest lists over materialized blocks: float32 scans
    # split into column ranges, float64 scans on integer keys; duplicated
    # points give tied core distances.
    _compare(_windows(ms, 6, (ms + 10, 900), 6), 8, ms, 0.0, precision, force_matrix=True)


def _nested_pairs(pairs, seed):
    """Tight pairs of points on a line with growing gaps: every merge up the
    dendrogram joins a pair (two points) to everything below it, so with
    min_cluster_size 2 each split's large child splits again - clusters nested
    `pairs` levels deep."""
    rng = np.random.default_rng(seed)
    centres = np.cumsum(1.0 + 0.05 * np.arange(pairs)) * 10.0
    x = np.repeat(centres, 2)[:, None] + rng.normal(0, 0.01, (2 * pairs, 1))
    return np.concatenate([x, rng.normal(0, 0.01, (2 * pairs, 2))], axis=1)


@pytest.mark.parametrize("precision", ["float32", "float64"])
@pytest.mark.parametrize("pairs", [40, 90])
def test_deeply_nested_clusters_match_oracle(cuda, precision, pairs):
    # Cluster trees 40 and 90 splits deep: the breadth-first condensation runs
    # one long queue level per split with exactly two nodes in it.
    _compare([_nested_pairs(pairs, pairs), _nested_pairs(pairs, pairs + 1)[::-1].copy()], 2, 1, 0.0, precision)
