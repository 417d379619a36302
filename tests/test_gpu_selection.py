"""Cluster selection options beyond the reference contract (leaf,
allow_single_cluster) and membership probabilities on the CUDA path.

float64 results equal scikit-learn's (labels with the same ids,
probabilities bit for bit) on the golden cases of tests/golden/make_golden.py
(family "selection"); both precisions equal the oracle on larger seeded
windows, in the single-CTA and the thread-block-cluster kernels.
"""

import numpy as np
import pytest

from oracle import oracle
from tests.golden import golden

pytestmark = pytest.mark.gpu

METHODS = {0: "eom", 1: "leaf"}


def _run(windows, mcs, ms, eps, precision, method, allow):
    import torch

    from hdbscan_gb300._cuda import Plan, pack

    packed, offsets = pack([np.asarray(w) for w in windows], precision)
    plan = Plan(offsets, packed.shape[1], min_cluster_size=mcs, min_samples=ms, cluster_selection_epsilon=eps,
                precision=precision, cluster_selection_method=method, allow_single_cluster=allow)
    exports = plan.export_buffers(hierarchy=False, probabilities=True)
    labels, status = plan.forward(packed, exports=exports)
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    return labels.cpu().numpy(), exports["probabilities"].cpu().numpy(), offsets


def test_selection_goldens_match_sklearn_float64(cuda):
    cases = golden.load("selection")
    groups = {}
    for name, case in cases.items():
        if "sk_failed" in case:
            continue
        mcs, ms, eps = case["params"]
        method, allow = (int(v) for v in case["options"])
        key = (int(mcs), int(ms), float(eps), method, allow, case["x"].shape[1])
        groups.setdefault(key, []).append(name)
    checked = 0
    for (mcs, ms, eps, method, allow, _), names in groups.items():
        windows = [cases[nm]["x"] for nm in names]
        labels, probs, offsets = _run(windows, mcs, ms, eps, "float64", METHODS[method], bool(allow))
        for w, nm in enumerate(names):
            lo, hi = offsets[w], offsets[w + 1]
            np.testing.assert_array_equal(labels[lo:hi], cases[nm]["sk_labels"], err_msg=nm)
            np.testing.assert_array_equal(probs[lo:hi].view(np.uint64), cases[nm]["sk_probabilities"].view(np.uint64),
                                          err_msg=nm)
            checked += 1
    assert checked > 300


def _windows(seed, sizes, dims):
    rng = np.random.default_rng(seed)
    out = []
    for i, n in enumerate(sizes):
        if i % 3 == 0:
            out.append(rng.integers(-4, 5, (n, dims)) / 2.0)
        else:
            k = 2 + i % 5
            centres = rng.normal(0, 3, (k, dims))
            out.append(centres[rng.integers(0, k, n)] + rng.normal(0, 0.3 + 0.1 * (i % 4), (n, dims)))
    return out


@pytest.mark.parametrize("precision", ["float32", "float64"])
@pytest.mark.parametrize("method,allow", [("eom", False), ("eom", True), ("leaf", False), ("leaf", True)])
@pytest.mark.parametrize("eps", [0.0, 0.3])
def test_options_match_oracle(cuda, precision, method, allow, eps):
    windows = _windows(17, [40, 300, 1024, 700, 2048, 3000], 5)
    labels, probs, offsets = _run(windows, 8, 4, eps, precision, method, allow)
    dtype = np.float32 if precision == "float32" else np.float64
    for w, x in enumerate(windows):
        o = oracle.cluster(x.astype(dtype), 8, 4, eps, precision, method=method, allow_single_cluster=allow)
        lo, hi = offsets[w], offsets[w + 1]
        ctx = f"window {w} n={hi - lo} {precision} {method} allow={allow} eps={eps}"
        np.testing.assert_array_equal(labels[lo:hi], o["labels"], err_msg=ctx)
        np.testing.assert_array_equal(probs[lo:hi].view(np.uint8), o["probabilities"].view(np.uint8), err_msg=ctx)


def test_public_api_probabilities(cuda):
    from hdbscan_gb300 import hdbscan

    x = _windows(3, [500], 4)[0]
    labels, probs = hdbscan(x, min_cluster_size=6, min_samples=3, precision="float64", return_probabilities=True)
    o = oracle.cluster(x, 6, 3, 0.0, "float64")
    np.testing.assert_array_equal(labels.cpu().numpy(), o["labels"])
    np.testing.assert_array_equal(probs.cpu().numpy(), o["probabilities"])
    labels_leaf = hdbscan(x, min_cluster_size=6, min_samples=3, precision="float64", cluster_selection_method="leaf")
    np.testing.assert_array_equal(labels_leaf.cpu().numpy(),
                                  oracle.cluster(x, 6, 3, 0.0, "float64", method="leaf")["labels"])
