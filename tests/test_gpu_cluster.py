"""Thread-block-cluster Prim (windows above 1024 points) vs the CPU oracle.

Each compiled cluster variant (CTAs per window x register dimensions or the
matrix variant) is forced through a one-rule autotune table, and every
exported stage is compared bit for bit with the oracle, as in
test_gpu_parity.py: Prim edges and weights, sort order, linkage rows,
condensed clusters, cores and labels.  Windows mix integer lattices (many
equal weights, so tie rules across CTAs matter), duplicated points and
Gaussian clusters.
"""

import ctypes
import json
import zlib

import numpy as np
import pytest

from oracle import oracle

pytestmark = pytest.mark.gpu


def _lattice(rng, n, dims):
    return rng.integers(-4, 5, (n, dims)) / 2.0


def _duplicates(rng, n, dims):
    x = np.repeat(rng.normal(size=(n // 4 + 1, dims)), 4, axis=0)[:n]
    return x[rng.permutation(n)]


def _mixture(rng, n, dims):
    centres = rng.normal(0, 4, (6, dims))
    return centres[rng.integers(0, 6, n)] + rng.normal(0, 0.3, (n, dims))


def _batch(seed, sizes, dims):
    rng = np.random.default_rng(seed)
    makers = (_lattice, _duplicates, _mixture)
    return [makers[i % 3](rng, n, dims) for i, n in enumerate(sizes)]


class forced_variant:
    """Context manager: a tuning table sending windows above 1024 points (or,
    with small=True, every window) to the variant (threads, slots, dims,
    cluster); smaller windows go to the single-CTA matrix variant."""

    def __init__(self, precision, threads, slots, dims, cluster, small=False):
        from hdbscan_gb300 import _lib

        code = _lib.HDB_F32 if precision == "float32" else _lib.HDB_F64
        rules = [] if small else [[code, -1, 1024, 1 << 20, 512, 2, 0, 1, 1]]
        rules.append([code, -1, 4096, 1 << 20, threads, slots, dims, cluster, 1])
        self.rules = np.array(rules, dtype=np.int32)

    def __enter__(self):
        from hdbscan_gb300 import _lib

        lib = _lib.lib()
        _lib.check(lib.hdb_set_tuning(self.rules.ctypes.data_as(ctypes.c_void_p), len(self.rules)),
                   "hdb_set_tuning")
        return self

    def __exit__(self, *exc):
        from hdbscan_gb300 import _lib, autotune

        lib = _lib.lib()
        lib.hdb_set_tuning(None, 0)
        autotune.apply_table(lib)
        return False


def _run_plan(windows, mcs, ms, eps, precision, expect_cluster, threshold=1024, one_persistent=False):
    import torch

    from hdbscan_gb300._cuda import Plan, pack

    packed, offsets = pack([np.asarray(w) for w in windows], precision)
    plan = Plan(offsets, packed.shape[1], min_cluster_size=mcs, min_samples=ms, cluster_selection_epsilon=eps,
                precision=precision, one_persistent=one_persistent)
    classes = json.loads(plan.describe())["classes"]
    big = [c for c in classes if c["nmax"] > threshold]
    assert big and all(c["cluster"] == expect_cluster for c in big), classes
    exports = plan.export_buffers(hierarchy=True, gradients=True)
    labels, status = plan.forward(packed, exports=exports)
    torch.cuda.synchronize()
    host = {k: v.cpu().numpy() for k, v in exports.items()}
    return labels.cpu().numpy(), int(status.item()), host, offsets


def _compare(windows, mcs, ms, eps, precision, expect_cluster, threshold=1024, one_persistent=False):
    labels, status, ex, offsets = _run_plan(windows, mcs, ms, eps, precision, expect_cluster, threshold,
                                            one_persistent)
    assert status == 0
    dtype = np.float32 if precision == "float32" else np.float64
    for w, x in enumerate(windows):
        o = oracle.cluster(np.asarray(x, dtype=dtype), mcs, ms, eps, precision)
        lo, hi = offsets[w], offsets[w + 1]
        n = hi - lo
        e0, e1 = lo - w, hi - w - 1
        ctx = f"window {w} n={n} mcs={mcs} ms={ms} eps={eps} {precision} cluster={expect_cluster}"
        np.testing.assert_array_equal(ex["edges_uv"][e0:e1], o["edges_uv"], err_msg=ctx)
        np.testing.assert_array_equal(ex["edge_w"][e0:e1].view(np.uint8), o["edge_w"].view(np.uint8), err_msg=ctx)
        np.testing.assert_array_equal(ex["order"][e0:e1], o["order"], err_msg=ctx)
        np.testing.assert_array_equal(ex["link_lr"][e0:e1], o["link_lr"], err_msg=ctx)
        np.testing.assert_array_equal(ex["link_w"][e0:e1].view(np.uint8), o["link_w"].view(np.uint8), err_msg=ctx)
        np.testing.assert_array_equal(ex["link_size"][e0:e1], o["link_size"], err_msg=ctx)
        k = int(ex["n_clusters"][w])
        assert k == len(o["cl_parent"]), ctx
        np.testing.assert_array_equal(ex["cl_parent"][lo:lo + k], o["cl_parent"], err_msg=ctx)
        np.testing.assert_array_equal(ex["cl_stability"][lo:lo + k].view(np.uint8),
                                      o["cl_stability"].view(np.uint8), err_msg=ctx)
        np.testing.assert_array_equal(ex["point_parent"][lo:hi], o["point_parent"], err_msg=ctx)
        if ms > 2:
            np.testing.assert_array_equal(ex["core"][lo:hi].view(np.uint8), o["core"].view(np.uint8), err_msg=ctx)
        np.testing.assert_array_equal(labels[lo:hi], o["labels"], err_msg=ctx)


# (precision, register dims, D): every compiled cluster variant.
VARIANTS = [("float32", 8, 5), ("float32", 16, 16), ("float32", 32, 17), ("float32", 0, 40),
            ("float64", 8, 8), ("float64", 16, 11), ("float64", 0, 24)]
PARAMS = [(2, 2, 0.0), (10, 10, 0.05), (5, 3, 0.0)]


@pytest.mark.parametrize("precision,dp,dims", VARIANTS)
@pytest.mark.parametrize("cluster", [2, 4])
@pytest.mark.parametrize("params", PARAMS, ids=lambda p: f"mcs{p[0]}-ms{p[1]}-eps{p[2]}")
def test_cluster_variant_matches_oracle(cuda, precision, dp, dims, cluster, params):
    mcs, ms, eps = params
    top = 1024 * cluster
    sizes = [1025, top, (1025 + top) // 2] if cluster == 2 else [1030, 2049, 3001, top]
    with forced_variant(precision, 512, 2, dp, cluster):
        seed = zlib.crc32(repr((precision, dp, cluster, params)).encode())
        _compare(_batch(seed, sizes, dims), mcs, ms, eps, precision, cluster)


@pytest.mark.parametrize("precision", ["float32", "float64"])
@pytest.mark.parametrize("cluster", [2, 4])
def test_cluster_kernel_on_tiny_windows(cuda, precision, cluster):
    # Windows of 2..40 points on the cluster kernel: CTAs whose vertex range is
    # empty only send sentinel records, and the home CTA still records every edge.
    rng = np.random.default_rng(cluster)
    windows = [_lattice(rng, n, 3) for n in (2, 3, 4, 5, 7, 40)]
    with forced_variant(precision, 512, 2, 8, cluster, small=True):
        _compare(windows, 2, 1, 0.0, precision, cluster, threshold=0)
        _compare(windows, 2, 2, 0.25, precision, cluster, threshold=0)


@pytest.mark.parametrize("precision", ["float32", "float64"])
@pytest.mark.parametrize("cluster", [2, 4])
def test_one_persistent_cluster_serves_every_window(cuda, precision, cluster):
    # One persistent cluster takes the whole queue, so every CTA is the home
    # of several windows (hierarchy overlapping later Prim loops), and one
    # single-CTA kernel takes the small windows of the same plan.
    rng = np.random.default_rng(99 + cluster)
    sizes = [int(s) for s in rng.integers(1025, 1024 * cluster + 1, 9)] + [5, 40, 700, 150]
    with forced_variant(precision, 512, 2, 8, cluster):
        _compare(_batch(5, sizes, 6), 4, 4, 0.1, precision, cluster, one_persistent=True)
        _compare(_batch(6, sizes, 6), 3, 1, 0.0, precision, cluster, one_persistent=True)


@pytest.mark.parametrize("precision", ["float32", "float64"])
def test_cluster_nonfinite_window_is_flagged(cuda, precision):
    import torch

    from hdbscan_gb300 import _lib
    from hdbscan_gb300._cuda import Plan, pack

    windows = _batch(3, [1500, 1100, 2000], 8)
    windows[1] = windows[1].copy()
    windows[1][700, 3] = np.nan
    with forced_variant(precision, 512, 2, 8, 2):
        packed, offsets = pack(windows, precision)
        plan = Plan(offsets, 8, min_cluster_size=5, min_samples=5, precision=precision)
        labels, status = plan.forward(packed)
        torch.cuda.synchronize()
    assert int(status.item()) & _lib.STATUS_NONFINITE
    labels = labels.cpu().numpy()
    assert (labels[offsets[1]:offsets[2]] == -1).all()
    dtype = np.float32 if precision == "float32" else np.float64
    for w in (0, 2):
        o = oracle.cluster(windows[w].astype(dtype), 5, 5, 0.0, precision)
        np.testing.assert_array_equal(labels[offsets[w]:offsets[w + 1]], o["labels"])


@pytest.mark.parametrize("precision", ["float32", "float64"])
def test_cluster_graph_replay_is_stable(cuda, precision):
    import torch

    from hdbscan_gb300._cuda import Plan, pack

    windows = _batch(8, [1200, 2500, 4096, 1800], 8)
    with forced_variant(precision, 512, 2, 8, 4):
        packed, offsets = pack(windows, precision)
        plan = Plan(offsets, 8, min_cluster_size=10, min_samples=10, cluster_selection_epsilon=0.05,
                    precision=precision)
        first, status = plan.forward(packed)
        first = first.clone()
        plan.capture(packed)
        for _ in range(3):
            labels, status = plan.replay()
        torch.cuda.synchronize()
    assert int(status.item()) == 0
    assert torch.equal(first, labels)


def test_cluster_rule_holds_one_wave(cuda):
    """A cluster rule applies while the batch fits one wave of SMs; beyond it
    the smallest clustered windows run on one CTA each (largest keep CS SMs)."""
    import torch

    from hdbscan_gb300._cuda import Plan

    sms = torch.cuda.get_device_properties(0).multi_processor_count
    rng = np.random.default_rng(11)
    with forced_variant("float32", 512, 2, 8, 4):
        few = np.concatenate([[0], np.cumsum(rng.integers(1100, 4000, max(sms // 8, 1)))]).astype(np.int64)
        classes = json.loads(Plan(few, 8, min_cluster_size=5, min_samples=4).describe())["classes"]
        assert all(c["cluster"] == 4 for c in classes), classes
        sizes = np.sort(rng.integers(1100, 4000, sms // 2 + 10))[::-1]
        many = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
        classes = json.loads(Plan(many, 8, min_cluster_size=5, min_samples=4).describe())["classes"]
        clustered = [c for c in classes if c["cluster"] > 1]
        single = [c for c in classes if c["cluster"] == 1]
        assert clustered and single, classes
        assert sum(c["cluster"] * c["windows"] for c in classes) <= sms, classes
        assert sum(c["windows"] for c in classes) == len(sizes)
        n_clustered = sum(c["windows"] for c in clustered)
        assert min(c["nmax"] for c in clustered) >= sizes[n_clustered - 1]  # the largest windows keep the cluster
        assert max(c["nmax"] for c in single) <= sizes[n_clustered]


def test_cluster_waits_give_up_and_report_internal_status(cuda):
    """A ticket that is never broadcast (test switch HDB_FLAG_TEST_STALL): every
    CTA's bounded mbarrier wait runs out after 1 ms, the kernel ends with the
    internal-error status and writes no labels, and the context stays usable.
    Nothing is in flight when the waits give up (no record was sent)."""
    import time

    import torch

    from hdbscan_gb300 import _lib
    from hdbscan_gb300._cuda import Plan, pack, raise_for_status

    rng = np.random.default_rng(17)
    windows = [_mixture(rng, 1500, 8), _mixture(rng, 1300, 8), _mixture(rng, 1100, 8)]
    packed, offsets = pack(windows, "float32")
    with forced_variant("float32", 512, 2, 8, 2):
        stalled = Plan(offsets, 8, min_cluster_size=5, min_samples=2, precision="float32",
                       test_flags=_lib.HDB_FLAG_TEST_STALL)
        normal = Plan(offsets, 8, min_cluster_size=5, min_samples=2, precision="float32")
    assert all(c["cluster"] == 2 for c in json.loads(stalled.describe())["classes"])
    labels = torch.full((stalled.points,), -7, dtype=torch.int32, device=cuda)
    t0 = time.perf_counter()
    _, status = stalled.forward(packed, labels=labels)
    torch.cuda.synchronize()
    elapsed = time.perf_counter() - t0
    assert int(status.item()) == _lib.STATUS_INTERNAL
    assert bool((labels == -7).all()), "a stalled kernel must not write labels"
    assert elapsed < 5.0
    with pytest.raises(RuntimeError, match="consistency"):
        raise_for_status(int(status.item()))
    # The same windows without the switch: the context still works and the
    # labels equal the oracle's.
    got, status = normal.forward(packed)
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    got = got.cpu().numpy()
    for w, x in enumerate(windows):
        want = oracle.cluster(np.asarray(x, np.float32), 5, 2, 0.0, "float32")["labels"]
        np.testing.assert_array_equal(got[offsets[w]:offsets[w + 1]], want)
