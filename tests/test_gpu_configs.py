"""The benchmark configurations at full size, every window, against the oracle.

Each seeded configuration (hdbscan_gb300/synthetic.py) runs as one ragged plan
-- the same plan the benchmark times, with its size classes, chunked matrix
classes, 128x128 distance tiles, clustered windows and two-CTA classes -- and
every window is compared with the CPU oracle (oracle/hdb_oracle_body.h, pinned
to the reference's kernels and scikit-learn by tests/test_oracle.py) bit for
bit: Prim edges and weights, sort order, linkage rows, weights and sizes, core
distances, the condensed tree (parents, births, stabilities, selection, child
sizes, the lambda each point leaves at) and labels.

Also here: the single float64 window of the first configuration against the
scikit-learn outputs stored in tests/golden (labels, single-linkage tree,
condensed tree), and the float32 configurations against the float64 oracle on
the same (float32-rounded) inputs: the share of windows whose partitions agree
exactly and the largest relative error of the merge weights, the statement the
reference documents for its float32 path (tests/test_parity.py:244-263 there).
"""

import numpy as np
import pytest

from oracle import oracle
from tests.conftest import partition_equal
from tests.golden import golden

pytestmark = pytest.mark.gpu

CONFIGS = [("c1", None), ("c2", None), ("c3", "float32"), ("c3", "float64"), ("c4", None), ("c5", None)]


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint8)


def _run_plan(packed, offsets, params, precision):
    import torch

    from hdbscan_gb300._cuda import Plan

    dtype = torch.float32 if precision == "float32" else torch.float64
    plan = Plan(offsets, packed.shape[1], min_cluster_size=params["min_cluster_size"],
                min_samples=params["min_samples"], cluster_selection_epsilon=params["cluster_selection_epsilon"],
                precision=precision)
    X = torch.as_tensor(packed, dtype=dtype, device="cuda")
    buffers = plan.export_buffers(hierarchy=True, gradients=True, probabilities=True)
    labels, status = plan.forward(X, exports=buffers)
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    host = {k: v.cpu().numpy() for k, v in buffers.items()}
    host["labels"] = labels.cpu().numpy()
    return host, plan.describe()


def _first_bad_window(offsets, mask_rows):
    """Window of the first False entry of a per-row mask laid out at row offsets."""
    bad = int(np.flatnonzero(~mask_rows)[0])
    return int(np.searchsorted(offsets, bad, side="right") - 1), bad


def _compare(got, want, offsets, ms, context):
    B = len(offsets) - 1
    sizes = np.diff(offsets)
    E = int(offsets[-1]) - B
    edge_offsets = offsets - np.arange(B + 1)

    def check(name, a, b, rows_offsets):
        a, b = np.asarray(a), np.asarray(b)
        same = np.all(a == b, axis=1) if a.ndim == 2 else a == b
        if not np.all(same):
            w, row = _first_bad_window(rows_offsets, np.asarray(same))
            raise AssertionError(f"{context}: {name} differs first in window {w} (n={sizes[w]}), row {row}")

    check("labels", got["labels"], want["labels"], offsets)
    check("edges_uv", got["edges_uv"][:E], want["edges_uv"][:E], edge_offsets)
    check("edge_w bits", got["edge_w"][:E].view(_int_of(got["edge_w"])), want["edge_w"][:E].view(
        _int_of(want["edge_w"])), edge_offsets)
    check("order", got["order"][:E], want["order"][:E], edge_offsets)
    check("link_lr", got["link_lr"][:E], want["link_lr"][:E], edge_offsets)
    check("link_w bits", got["link_w"][:E].view(_int_of(got["link_w"])),
          want["link_w"][:E].view(_int_of(want["link_w"])), edge_offsets)
    check("link_size", got["link_size"][:E], want["link_size"][:E], edge_offsets)
    if ms > 2:
        check("core bits", got["core"].view(_int_of(got["core"])), want["core"].view(_int_of(want["core"])),
              offsets)
    np.testing.assert_array_equal(got["n_clusters"], want["n_clusters"], err_msg=f"{context}: n_clusters")
    rows = np.concatenate([np.arange(offsets[w], offsets[w] + want["n_clusters"][w]) for w in range(B)])
    # Cluster rows packed densely, with their own offsets, for the error message.
    cluster_offsets = np.concatenate([[0], np.cumsum(want["n_clusters"])])
    for name in ("cl_parent", "cl_selected", "cl_size"):
        check(name, got[name][rows], want[name][rows], cluster_offsets)
    for name in ("cl_birth", "cl_stability"):
        check(name + " bits", got[name][rows].view(_int_of(got[name])), want[name][rows].view(_int_of(want[name])),
              cluster_offsets)
    check("point_parent", got["point_parent"], want["point_parent"], offsets)
    check("point_lambda bits", got["point_lambda"].view(_int_of(got["point_lambda"])),
          want["point_lambda"].view(_int_of(want["point_lambda"])), offsets)
    check("probabilities bits", got["probabilities"].view(_int_of(got["probabilities"])),
          want["probabilities"].view(_int_of(want["probabilities"])), offsets)


def _int_of(a):
    return np.int32 if a.dtype == np.float32 else np.int64


@pytest.mark.parametrize("config,precision", CONFIGS, ids=[f"{c}-{p or 'default'}" for c, p in CONFIGS])
def test_full_config_matches_oracle(cuda, config, precision):
    from hdbscan_gb300 import synthetic

    packed, offsets, params = synthetic.make(config)
    precision = precision or params["precision"]
    got, describe = _run_plan(packed, offsets, params, precision)
    dtype = np.float32 if precision == "float32" else np.float64
    want = oracle.batch_ex(packed.astype(dtype), offsets, params["min_cluster_size"], params["min_samples"],
                           params["cluster_selection_epsilon"], precision)
    assert not want["status"].any()
    _compare(got, want, offsets, params["min_samples"], f"{config} {precision} plan={describe}")


def test_c1_window_matches_sklearn_goldens(cuda):
    """The float64 window of the first configuration against scikit-learn (stored outputs)."""
    import torch

    from hdbscan_gb300 import condensed_tree, hdbscan_ragged

    case = golden.load("configs")["c1"]
    x = case["x"]
    mcs, ms, eps = (int(case["params"][0]), int(case["params"][1]), float(case["params"][2]))
    labels, offsets, hierarchy = hdbscan_ragged([torch.as_tensor(x, device="cuda")], min_cluster_size=mcs,
                                                min_samples=ms, cluster_selection_epsilon=eps, precision="float64",
                                                return_hierarchy=True)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(labels.cpu().numpy(), case["sk_labels"])
    np.testing.assert_array_equal(hierarchy["link_lr"].cpu().numpy(), case["sk_link_lr"])
    np.testing.assert_array_equal(hierarchy["link_size"].cpu().numpy(), case["sk_link_size"])
    np.testing.assert_array_equal(_bits(hierarchy["link_w"].cpu().numpy()), _bits(case["sk_link_w"]))
    tree = {k: v.cpu().numpy() for k, v in condensed_tree(hierarchy, offsets)[0].items()}
    want = sorted(zip(case["sk_ct_parent"].tolist(), case["sk_ct_child"].tolist(), case["sk_ct_lambda"].tolist(),
                      case["sk_ct_size"].tolist()), key=lambda r: r[1])
    got = list(zip(tree["parent"].tolist(), tree["child"].tolist(), tree["lambda_val"].tolist(),
                   tree["child_size"].tolist()))
    assert got == want


@pytest.mark.parametrize("config", ["c2", "c3"])
def test_float32_agreement_with_float64_oracle(cuda, config):
    """float32 labels and merge weights of the full configuration against the float64 oracle."""
    from hdbscan_gb300 import synthetic

    packed, offsets, params = synthetic.make(config)
    x32 = packed.astype(np.float32)
    got, _ = _run_plan(x32, offsets, params, "float32")
    mcs, ms, eps = params["min_cluster_size"], params["min_samples"], params["cluster_selection_epsilon"]
    want = oracle.batch_ex(x32.astype(np.float64), offsets, mcs, ms, eps, "float64")
    exact, worst = 0, 0.0
    for w in range(len(offsets) - 1):
        lo, hi = offsets[w], offsets[w + 1]
        exact += partition_equal(got["labels"][lo:hi], want["labels"][lo:hi])
        a = np.sort(got["link_w"][lo - w:hi - w - 1].astype(np.float64))
        b = np.sort(want["link_w"][lo - w:hi - w - 1])
        worst = max(worst, float(np.max(np.abs(a - b) / np.maximum(np.abs(b), np.finfo(np.float64).tiny))))
    rate = exact / (len(offsets) - 1)
    print(f"{config}: float32 vs float64 oracle: exact partitions {exact}/{len(offsets) - 1}, "
          f"max relative merge-weight error {worst:.3e}")
    # Measured values for these seeded inputs (also in the design notes): every
    # partition agrees; merge weights differ by a few float32 roundings.
    assert rate == 1.0
    assert worst <= 1e-6
