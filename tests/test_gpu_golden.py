"""CUDA path against the golden vectors: bit-exact with the reference's kernels.

Every golden case (tests/golden/) runs through the ragged C-ABI forward, cases
with equal parameters packed into one batch, in both the on-chip recompute
variant and the materialized-distance (matrix) variant.  Labels, Prim edges
and weights, sort order and single-linkage rows must equal the reference
kernels' outputs bit for bit; sort fixtures must reproduce NumPy's quicksort
tie order.
"""

from collections import defaultdict

import numpy as np
import pytest

from tests.golden import golden

pytestmark = pytest.mark.gpu


def _groups(family):
    groups = defaultdict(list)
    for name, case in golden.load(family).items():
        mcs, ms, eps = case["params"]
        groups[(int(mcs), int(ms), float(eps), case["x"].shape[1])].append((name, case))
    return groups


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint8)


@pytest.mark.parametrize("force_matrix", [False, True])
@pytest.mark.parametrize("precision", ["float32", "float64"])
@pytest.mark.parametrize("family", ["known", "corpus", "exhaustive", "sweep", "sort", "configs"])
def test_golden_family(cuda, family, precision, force_matrix):
    import torch

    from hdbscan_gb300._cuda import cluster_ragged, pack

    checked = 0
    for (mcs, ms, eps, _dims), items in _groups(family).items():
        items = [(n, c) for n, c in items if int(np.ravel(c[f"{precision}/ref_status"])[0]) == 0]
        if not items:
            continue
        packed, offsets = pack([c["x"] for _, c in items], precision)
        labels, ex = cluster_ragged(packed, offsets, mcs, ms, eps, precision, exports=True,
                                    force_matrix=force_matrix)
        torch.cuda.synchronize()
        labels = labels.cpu().numpy()
        host = {k: v.cpu().numpy() for k, v in ex.items()}
        for w, (name, case) in enumerate(items):
            lo, hi = offsets[w], offsets[w + 1]
            e0, e1 = lo - w, hi - w - 1
            ref = lambda key: case[f"{precision}/ref_{key}"]  # noqa: E731
            msg = f"{family}/{name} {precision} matrix={force_matrix}"
            np.testing.assert_array_equal(labels[lo:hi], ref("labels"), err_msg=msg)
            np.testing.assert_array_equal(host["edges_uv"][e0:e1], ref("edges_uv"), err_msg=msg)
            np.testing.assert_array_equal(_bits(host["edge_w"][e0:e1]), _bits(ref("edge_w")), err_msg=msg)
            np.testing.assert_array_equal(host["order"][e0:e1], ref("order"), err_msg=msg)
            np.testing.assert_array_equal(host["link_lr"][e0:e1], ref("link_lr"), err_msg=msg)
            np.testing.assert_array_equal(host["link_size"][e0:e1], ref("link_size"), err_msg=msg)
            np.testing.assert_array_equal(_bits(host["link_w"][e0:e1]), _bits(ref("link_w")), err_msg=msg)
            if family == "sort":
                np.testing.assert_array_equal(host["order"][e0:e1], case["argsort"], err_msg=msg)
            checked += 1
    assert checked > 0
