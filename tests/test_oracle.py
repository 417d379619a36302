"""The CPU oracle against the golden vectors (the pin of every parity claim).

Golden vectors (tests/golden/make_golden.py) hold, per case, the outputs of the
reference's own kernel bodies compiled for the CPU and of scikit-learn.  The
oracle must reproduce the reference's outputs bit for bit in both precisions
(labels, Prim edges and weights, sort order, single-linkage rows) and, in
float64, scikit-learn's labels, single-linkage tree and condensed tree.
Known-answer cases of the reference's own tests are asserted explicitly.
"""

import numpy as np
import pytest

from oracle import oracle
from tests.conftest import partition_equal
from tests.golden import golden

PRECISIONS = ("float32", "float64")


def _cases(family):
    return [pytest.param(family, name, id=f"{family}-{name}") for name in golden.load(family)]


def _run(case, precision):
    x = case["x"]
    mcs, ms, eps = case["params"]
    return oracle.cluster(x, int(mcs), int(ms), float(eps), precision)


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint8)


def _check_reference(case, precision, out):
    ref = {k[len(precision) + 5:]: v for k, v in case.items() if k.startswith(f"{precision}/ref_")}
    assert out["status"] == int(ref["status"][0] if np.ndim(ref["status"]) else ref["status"])
    if out["status"]:
        return
    np.testing.assert_array_equal(out["labels"], ref["labels"])
    np.testing.assert_array_equal(out["edges_uv"], ref["edges_uv"])
    np.testing.assert_array_equal(_bits(out["edge_w"]), _bits(ref["edge_w"].astype(out["edge_w"].dtype)))
    np.testing.assert_array_equal(out["order"], ref["order"])
    np.testing.assert_array_equal(out["link_lr"], ref["link_lr"])
    np.testing.assert_array_equal(out["link_size"], ref["link_size"])
    np.testing.assert_array_equal(_bits(out["link_w"]), _bits(ref["link_w"].astype(out["link_w"].dtype)))


def _condensed_rows(out, n):
    rows = []
    for c in range(1, len(out["cl_parent"])):
        rows.append((int(out["cl_parent"][c]), n + c, float(out["cl_birth"][c]), int(out["cl_size"][c])))
    for i in range(n):
        rows.append((int(out["point_parent"][i]), i, float(out["point_lambda"][i]), 1))
    return sorted(rows, key=lambda r: r[1])


def _check_sklearn(case, out, tag):
    if f"{tag}_link_lr" not in case:
        return
    n = len(case["x"])
    np.testing.assert_array_equal(out["link_lr"], case[f"{tag}_link_lr"])
    np.testing.assert_array_equal(out["link_size"], case[f"{tag}_link_size"])
    np.testing.assert_array_equal(_bits(out["link_w"]), _bits(case[f"{tag}_link_w"]))
    expected = sorted(zip(case[f"{tag}_ct_parent"].tolist(), case[f"{tag}_ct_child"].tolist(),
                          case[f"{tag}_ct_lambda"].tolist(), case[f"{tag}_ct_size"].tolist()), key=lambda r: r[1])
    assert _condensed_rows(out, n) == [(p, c, l, s) for p, c, l, s in expected]
    if f"{tag}_labels" in case:
        assert partition_equal(out["labels"], case[f"{tag}_labels"])
        np.testing.assert_array_equal(out["labels"], case[f"{tag}_labels"])


@pytest.mark.parametrize("family,name", _cases("known") + _cases("corpus") + _cases("exhaustive") +
                         _cases("sweep") + _cases("configs"))
def test_oracle_matches_reference_kernels_and_sklearn(family, name):
    case = golden.load(family)[name]
    for precision in PRECISIONS:
        out = _run(case, precision)
        _check_reference(case, precision, out)
        if precision == "float64":
            _check_sklearn(case, out, "sk")


@pytest.mark.parametrize("family,name", _cases("sort"))
def test_oracle_sort_matches_numpy_quicksort_tie_order(family, name):
    case = golden.load(family)[name]
    w = np.diff(case["x"][:, 0])
    np.testing.assert_array_equal(oracle.argsort(w), case["argsort"])
    for precision in PRECISIONS:
        out = _run(case, precision)
        _check_reference(case, precision, out)
        np.testing.assert_array_equal(out["edge_w"].astype(np.float64), w)
        np.testing.assert_array_equal(out["order"], case["argsort"])


# ---------------------------------------------------------------------------
# Known answers of the reference's tests (tests/test_parity.py:63-91,
# tests/test_float64.py:7-41 there).
# ---------------------------------------------------------------------------
BOUNDARY_COUNTS = {0.0: 4, 0.1: 4, float(np.nextafter(np.float32(0.125), np.float32(0))): 4, 0.125: 4,
                   float(np.nextafter(np.float32(0.125), np.float32(1))): 2}


@pytest.mark.parametrize("eps,clusters", list(BOUNDARY_COUNTS.items()))
def test_epsilon_boundary_known_answer(eps, clusters):
    case = golden.load("known")[f"boundary_eps{eps!r}"]
    for precision in PRECISIONS:
        labels = _run(case, precision)["labels"]
        assert partition_equal(labels, np.repeat(np.arange(clusters), 8 // clusters))


def test_documented_float32_epsilon_resolution_limit():
    # The next float64 above 1/8 merges the duplicate pairs in float64 but
    # rounds to 1/8 in float32 (test_parity.py:244-263 there).
    case = dict(golden.load("known")["boundary_eps0.0"])
    eps = float(np.nextafter(np.float64(0.125), np.float64(1)))
    assert np.float32(eps) == np.float32(0.125)
    case["params"] = np.array([2, 1, eps])
    assert partition_equal(_run(case, "float64")["labels"], [0, 0, 0, 0, 1, 1, 1, 1])
    assert partition_equal(_run(case, "float32")["labels"], [0, 0, 1, 1, 2, 2, 3, 3])


def test_float64_keeps_coordinates_that_collapse_in_float32():
    case = golden.load("known")["collapsing"]
    assert partition_equal(_run(case, "float64")["labels"], np.repeat(np.arange(4), 2))
    assert partition_equal(_run(case, "float32")["labels"], np.full(8, -1))


@pytest.mark.parametrize("eps,clusters", [(float(np.nextafter(0.125, 0)), 4), (0.125, 4),
                                          (float(np.nextafter(0.125, 1)), 2)])
def test_float64_epsilon_boundary_known_answer(eps, clusters):
    case = golden.load("known")[f"boundary64_eps{eps!r}"]
    labels = _run(case, "float64")["labels"]
    assert partition_equal(labels, np.repeat(np.arange(clusters), 8 // clusters))


@pytest.mark.parametrize("mcs,ms", [(2, 8), (8, 1), (9, 2)])
def test_all_noise_known_answer(mcs, ms):
    case = golden.load("known")[f"allnoise_mcs{mcs}_ms{ms}"]
    for precision in PRECISIONS:
        np.testing.assert_array_equal(_run(case, precision)["labels"], np.full(8, -1))


def test_well_separated_gives_three_clusters():
    case = golden.load("corpus")["separated_mcs5_ms5_eps0.0"]
    assert partition_equal(_run(case, "float64")["labels"], np.repeat(np.arange(3), 24))


def test_partition_comparison_rejects_merges_and_splits():
    assert partition_equal([7, 7, 4, 4, -1], [0, 0, 1, 1, -1])
    for bad in ([0, 0, 1, 1, 1], [0, 0, 0, 0, -1], [0, 2, 1, 1, -1]):
        assert not partition_equal(bad, [0, 0, 1, 1, -1])


def test_golden_vectors_record_their_generators():
    for family in golden.FAMILIES:
        sk, npv, env = golden.versions(family)
        assert env.startswith("X86_V3")


# ---------------------------------------------------------------------------
# scikit-learn's selection options beyond the reference contract (leaf,
# allow_single_cluster) and membership probabilities (float64, bit for bit).
# ---------------------------------------------------------------------------
METHOD_NAMES = {0: "eom", 1: "leaf"}


@pytest.mark.parametrize("family,name", _cases("selection"))
def test_oracle_selection_options_match_sklearn(family, name):
    case = golden.load(family)[name]
    if "sk_failed" in case:
        pytest.skip("scikit-learn raised on this case")
    mcs, ms, eps = case["params"]
    method, allow = (int(v) for v in case["options"])
    out = oracle.cluster(case["x"], int(mcs), int(ms), float(eps), "float64", method=METHOD_NAMES[method],
                         allow_single_cluster=bool(allow))
    np.testing.assert_array_equal(out["labels"], case["sk_labels"])
    np.testing.assert_array_equal(out["probabilities"].view(np.uint64), case["sk_probabilities"].view(np.uint64))


def test_default_selection_is_the_reference_contract():
    case = golden.load("corpus")["overlap_mcs5_ms5_eps0.1"]
    base = _run(case, "float64")
    ext = oracle.cluster(case["x"], 5, 5, 0.1, "float64", method="eom", allow_single_cluster=False)
    np.testing.assert_array_equal(base["labels"], ext["labels"])


def test_batch_ex_packs_every_window_like_single_calls():
    """oracle.batch_ex (threads over windows) equals per-window oracle.cluster, packed as the GPU exports."""
    from hdbscan_gb300 import synthetic

    packed, offsets, p = synthetic.make("c3", windows=6, high=700)
    for precision in PRECISIONS:
        batch = oracle.batch_ex(packed, offsets, p["min_cluster_size"], p["min_samples"],
                                p["cluster_selection_epsilon"], precision, threads=3)
        for w in range(len(offsets) - 1):
            lo, hi = offsets[w], offsets[w + 1]
            one = oracle.cluster(packed[lo:hi], p["min_cluster_size"], p["min_samples"],
                                 p["cluster_selection_epsilon"], precision)
            k = int(batch["n_clusters"][w])
            assert k == len(one["cl_parent"])
            for name in ("labels", "point_parent", "core"):
                np.testing.assert_array_equal(_bits(batch[name][lo:hi]), _bits(one[name]))
            np.testing.assert_array_equal(_bits(batch["point_lambda"][lo:hi]), _bits(one["point_lambda"]))
            for name in ("edges_uv", "edge_w", "order", "link_lr", "link_w", "link_size"):
                np.testing.assert_array_equal(_bits(batch[name][lo - w:hi - w - 1]), _bits(one[name]))
            for name in ("cl_parent", "cl_birth", "cl_stability", "cl_selected", "cl_size"):
                np.testing.assert_array_equal(_bits(batch[name][lo:lo + k]), _bits(one[name]))


def test_condensed_tree_rows_equal_sklearn():
    """hdbscan_gb300.condensed_tree on the oracle's exports gives scikit-learn's condensed_tree_ rows."""
    torch = pytest.importorskip("torch")
    from hdbscan_gb300 import condensed_tree

    case = golden.load("configs")["c1"]
    x = case["x"]
    offsets = np.array([0, len(x)], np.int64)
    mcs, ms, eps = case["params"]
    out = oracle.batch_ex(x, offsets, int(mcs), int(ms), float(eps), "float64", threads=1)
    hierarchy = {k: torch.from_numpy(v) for k, v in out.items() if isinstance(v, np.ndarray)}
    tree = {k: v.numpy() for k, v in condensed_tree(hierarchy, offsets)[0].items()}
    got = list(zip(tree["parent"].tolist(), tree["child"].tolist(), tree["lambda_val"].tolist(),
                   tree["child_size"].tolist()))
    want = sorted(zip(case["sk_ct_parent"].tolist(), case["sk_ct_child"].tolist(), case["sk_ct_lambda"].tolist(),
                      case["sk_ct_size"].tolist()), key=lambda r: r[1])
    assert got == want
