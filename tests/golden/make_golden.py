"""Generate the golden vectors that pin the CPU oracle (and, through it, the CUDA path).

Run in the build container, where both scikit-learn and the reference checkout
exist:  python tests/golden/make_golden.py
Outputs tests/golden/golden_<family>.npz (one concatenated array per field
plus per-case lengths; tests/golden/golden.py reads them back).  Every case
stores its input and, per precision:
  * ref_*     outputs of the reference's own CUDA-C kernel bodies compiled for
              the CPU (oracle/build_ref.py): labels from the full cluster body;
              Prim edges, sort order and single-linkage rows from the
              linkage-only prefix the reference's kernel tests use;
  * sk_*      scikit-learn HDBSCAN (float64 arithmetic) on the float64 input:
              labels, _single_linkage_tree_ and the condensed tree;
  * sk32_*    the same on the float32-rounded input, as the reference's tests
              feed scikit-learn (tests/conftest.py:96-103 there), stored only
              when rounding changes the input.
NumPy's SIMD argsort changes tie order on AVX2/AVX-512 hosts, so the script
re-executes itself with NPY_DISABLE_CPU_FEATURES set (the reference's sort and
scikit-learn's MST ordering follow the scalar introsort).
"""

from __future__ import annotations

import ctypes
import json
import os
import subprocess
import sys
from itertools import combinations_with_replacement
from pathlib import Path

SCALAR = "X86_V3 X86_V4 AVX512_ICL AVX512_SPR"
if os.environ.get("NPY_DISABLE_CPU_FEATURES") != SCALAR:
    env = dict(os.environ, NPY_DISABLE_CPU_FEATURES=SCALAR, OMP_NUM_THREADS="1", OPENBLAS_NUM_THREADS="1")
    raise SystemExit(subprocess.call([sys.executable, __file__, *sys.argv[1:]], env=env))

import numpy as np  # noqa: E402

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

from oracle import build_ref  # noqa: E402

PRECISIONS = ("float32", "float64")


# ---------------------------------------------------------------------------
# Reference kernels (CPU build) and scikit-learn.
# ---------------------------------------------------------------------------
class Reference:
    def __init__(self):
        path = build_ref.build()
        if path is None:
            raise SystemExit("reference kernels unavailable: run with the reference checkout present")
        self.lib = ctypes.CDLL(str(path))
        self.layout = json.loads((build_ref.OUT / "layout.json").read_text())
        P = ctypes.c_void_p
        for suffix in ("f32", "f64"):
            fn = getattr(self.lib, f"hdb_ref_cluster_{suffix}")
            fn.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, P, P, P]
            fn.restype = ctypes.c_int
            fn = getattr(self.lib, f"hdb_ref_linkage_{suffix}")
            fn.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, P, P]
            fn.restype = ctypes.c_int

    def run(self, x, mcs, ms, eps, precision):
        dtype, suffix = (np.float32, "f32") if precision == "float32" else (np.float64, "f64")
        x = np.ascontiguousarray(x, dtype=dtype)
        n, d = x.shape
        labels = np.empty(n, np.int32)
        ints = np.zeros(self.layout["INTEGER_WORKSPACE"] * n, np.int32)
        reals = np.zeros(self.layout["REAL_WORKSPACE"] * n, dtype)
        status = getattr(self.lib, f"hdb_ref_cluster_{suffix}")(x.ctypes.data, n, d, mcs, ms, eps, labels.ctypes.data,
                                                               ints.ctypes.data, reals.ctypes.data)
        out = {"status": np.int32(status)}
        if status:
            return out
        out["labels"] = labels
        ints[:] = 0
        reals[:] = 0
        getattr(self.lib, f"hdb_ref_linkage_{suffix}")(x.ctypes.data, n, d, ms, ints.ctypes.data, reals.ctypes.data)
        names_i, names_r = self.layout["INTEGER_ARRAYS"], self.layout["REAL_ARRAYS"]
        I = {name: ints[2 * i * n:2 * i * n + 2 * n] for i, name in enumerate(names_i)}
        R = {name: reals[2 * i * n:2 * i * n + 2 * n] for i, name in enumerate(names_r)}
        m = n - 1
        out["edges_uv"] = np.stack([I["edge_u"][:m], I["edge_v"][:m]], 1).astype(np.int32)
        out["edge_w"] = R["edge_w"][:m].copy()
        out["order"] = I["order"][:m].astype(np.int32)
        out["link_lr"] = np.stack([I["left"][n:2 * n - 1], I["right"][n:2 * n - 1]], 1).astype(np.int32)
        out["link_size"] = I["sizes"][n:2 * n - 1].astype(np.int32)
        out["link_w"] = R["distance"][n:2 * n - 1].copy()
        return out


def sklearn_fit(x, mcs, ms, eps, method="eom", allow_single=False):
    from sklearn.cluster import HDBSCAN
    from sklearn.cluster._hdbscan._tree import _condense_tree

    h = HDBSCAN(algorithm="auto", metric="euclidean", cluster_selection_method=method,
                allow_single_cluster=allow_single, alpha=1.0, copy=True, min_cluster_size=mcs, min_samples=ms,
                cluster_selection_epsilon=eps)
    out = {}
    try:
        out["labels"] = h.fit_predict(np.asarray(x, dtype=np.float64)).astype(np.int32)
        out["probabilities"] = np.asarray(h.probabilities_, np.float64)
    except (TypeError, KeyError):
        # scikit-learn 1.9.0 with NumPy >= 2.5 raises in epsilon_search's
        # traverse_upwards, and _do_labelling raises KeyError when
        # allow_single_cluster meets one selected non-root cluster and a point
        # that reaches the root; the linkage below is computed before that.
        out["failed"] = np.int8(1)
    slt = getattr(h, "_single_linkage_tree_", None)
    if slt is not None:
        out["link_lr"] = np.stack([slt["left_node"], slt["right_node"]], 1).astype(np.int32)
        out["link_w"] = np.asarray(slt["value"], np.float64)
        out["link_size"] = np.asarray(slt["cluster_size"], np.int32)
        ct = _condense_tree(slt, mcs)
        out["ct_parent"] = np.asarray(ct["parent"], np.int32)
        out["ct_child"] = np.asarray(ct["child"], np.int32)
        out["ct_lambda"] = np.asarray(ct["value"], np.float64)
        out["ct_size"] = np.asarray(ct["cluster_size"], np.int32)
    return out


# ---------------------------------------------------------------------------
# Case families.  Every input is drawn from a seed recorded here.
# ---------------------------------------------------------------------------
def corpus_inputs():
    return [(name, x) for name, x in _corpus_cases().items()]


def _corpus_cases():
    rng = np.random.default_rng(20261203)
    sep = np.concatenate([rng.normal(c, 0.08, (24, 2)) for c in ((-3, -3), (0, 3), (3, -3))])
    return {
        "separated": sep,
        "overlap": np.concatenate([rng.normal(c, 0.45, (30, 2)) for c in ((-0.5, 0), (0.5, 0), (0, 0.8))]),
        "density": np.concatenate([rng.normal(c, s, (k, 2)) for c, s, k in
                                   (((-4, 0), 0.025, 30), ((0, 4), 0.3, 35), ((4, 0), 0.8, 40))]),
        "quantized3d": rng.integers(-12, 13, (48, 3)) / 8.0,
        "duplicates": np.repeat(np.array([[0, 0], [0.125, 0], [4, 0], [4.125, 0], [20, 20]]), [7, 5, 6, 8, 1], 0),
        "identical": np.ones((24, 3)),
        "grid5x5": np.array([(a, b) for a in range(5) for b in range(5)], float),
        "cross": np.tile(np.array([[0, 0], [1, 0], [-1, 0], [0, 1], [0, -1]], float), (4, 1)),
        "tiny": np.concatenate([rng.normal(c, 0.01, (k, 2)) for c, k in (((0, 0), 2), ((2, 2), 3), ((5, 0), 9))]),
        "outliers": np.concatenate([sep, np.array([[20, 20], [-20, 20], [0, -30]])]),
        "two": np.array([[0.0, 0.0], [1.0, 1.0]]),
    }


def corpus():
    rng = np.random.default_rng(20261203)
    sep = np.concatenate([rng.normal(c, 0.08, (24, 2)) for c in ((-3, -3), (0, 3), (3, -3))])
    cases = {
        "separated": sep,
        "overlap": np.concatenate([rng.normal(c, 0.45, (30, 2)) for c in ((-0.5, 0), (0.5, 0), (0, 0.8))]),
        "density": np.concatenate([rng.normal(c, s, (k, 2)) for c, s, k in
                                   (((-4, 0), 0.025, 30), ((0, 4), 0.3, 35), ((4, 0), 0.8, 40))]),
        "quantized3d": rng.integers(-12, 13, (48, 3)) / 8.0,
        "duplicates": np.repeat(np.array([[0, 0], [0.125, 0], [4, 0], [4.125, 0], [20, 20]]), [7, 5, 6, 8, 1], 0),
        "identical": np.ones((24, 3)),
        "grid5x5": np.array([(a, b) for a in range(5) for b in range(5)], float),
        "cross": np.tile(np.array([[0, 0], [1, 0], [-1, 0], [0, 1], [0, -1]], float), (4, 1)),
        "tiny": np.concatenate([rng.normal(c, 0.01, (k, 2)) for c, k in (((0, 0), 2), ((2, 2), 3), ((5, 0), 9))]),
        "outliers": np.concatenate([sep, np.array([[20, 20], [-20, 20], [0, -30]])]),
        "two": np.array([[0.0, 0.0], [1.0, 1.0]]),
    }
    params = [(2, 1), (2, 2), (5, 5), (7, 3)]
    for name, x in cases.items():
        for mcs, ms in params:
            ms = min(ms, len(x))
            for eps in (0.0, 0.1):
                yield f"{name}_mcs{mcs}_ms{ms}_eps{eps}", x, mcs, ms, eps


def exhaustive():
    grid = np.array([[0, 0], [0, 1], [1, 0], [1, 1]], float)
    for size in (4, 5):
        for idx in combinations_with_replacement(range(4), size):
            for ms in (1, 2):
                for eps in (0.0, 0.1):
                    yield f"g{''.join(map(str, idx))}_ms{ms}_eps{eps}", grid[list(idx)], 2, ms, eps


def sweep():
    for seed in range(36):
        rng = np.random.default_rng(seed + 90210)
        n, d = int(rng.integers(8, 81)), int(rng.integers(1, 9))
        if seed % 3 == 0:
            x = rng.integers(-8, 9, (n, d)) / 4.0
        elif seed % 3 == 1:
            x = rng.normal(size=(n, d))
        else:
            x = rng.normal(0, 4, (3, d))[np.arange(n) % 3] + rng.normal(0, 0.1, (n, d))
        mcs = int(rng.integers(2, min(10, n) + 1))
        ms = mcs if seed % 4 == 0 else int(rng.integers(1, min(8, n) + 1))
        yield f"s{seed}", x, mcs, ms, 0.1 if seed % 2 else 0.0


def known_answers():
    # Known-answer inputs of the reference's tests (tests/test_parity.py:63-73,
    # tests/test_float64.py:7-19): expected cluster counts are asserted in
    # tests/test_oracle.py.
    boundary = np.array([[0], [0], [0.125], [0.125], [4], [4], [4.125], [4.125]], float)
    for eps in (0.0, 0.1, float(np.nextafter(np.float32(0.125), np.float32(0))), 0.125,
                float(np.nextafter(np.float32(0.125), np.float32(1)))):
        yield f"boundary_eps{eps!r}", boundary, 2, 1, eps
    gap = 2.0 ** -30
    yield "collapsing", np.repeat(1 + np.array([0, gap, 16 * gap, 17 * gap]), 2)[:, None], 2, 1, 0.0
    b64 = np.repeat(1 + 2.0 ** -40 + np.array([0, 0.125, 4, 4.125]), 2)[:, None]
    for eps in (float(np.nextafter(0.125, 0)), 0.125, float(np.nextafter(0.125, 1))):
        yield f"boundary64_eps{eps!r}", b64, 2, 1, eps
    for mcs, ms in ((2, 8), (8, 1), (9, 2)):
        yield f"allnoise_mcs{mcs}_ms{ms}", np.arange(16, dtype=float).reshape(8, 2), mcs, ms, 0.0


def sort_fixtures():
    # Points on a line at cumulative integer offsets: Prim walks the path from
    # vertex 0, so edge i has weight w_i and the sort sees exactly w (ties!).
    for n in (5, 17, 18, 33, 129, 1024, 4096):
        rng = np.random.default_rng(n)
        for pattern, w in (("equal", np.ones(n - 1)), ("alternating", 1 + np.arange(n - 1) % 2),
                           ("quantized", rng.integers(1, 5, n - 1)), ("ascending", np.arange(1, n)),
                           ("descending", np.arange(n - 1, 0, -1))):
            x = np.concatenate([[0.0], np.cumsum(w)])[:, None].astype(float)
            yield f"path{n}_{pattern}", x, 2, 1, 0.0


def config_windows():
    from hdbscan_gb300 import synthetic

    packed, off, p = synthetic.c1()
    yield "c1", packed, p["min_cluster_size"], p["min_samples"], p["cluster_selection_epsilon"]
    for name, kwargs in (("c2", dict(windows=2)), ("c3", dict(windows=5, low=64, high=1200)),
                         ("c4", dict(windows=1, n=600)), ("c5", dict(windows=1, low=700, high=900))):
        packed, off, p = synthetic.make(name, **kwargs)
        for w in range(len(off) - 1):
            yield (f"{name}_w{w}", packed[off[w]:off[w + 1]], p["min_cluster_size"], p["min_samples"],
                   p["cluster_selection_epsilon"])


def selection():
    """scikit-learn's selection options beyond the reference contract (leaf
    selection, allow_single_cluster) and membership probabilities, with the
    reference's own (eom, no single cluster) setting for the probabilities."""
    base = dict(corpus_inputs())
    rng = np.random.default_rng(20261204)
    for seed in range(6):
        k = 1 + seed % 4
        centres = rng.normal(0, 3, (k, 3))
        base[f"blobs{seed}"] = centres[rng.integers(0, k, 60)] + rng.normal(0, 0.4 + 0.1 * seed, (60, 3))
    for name, x in base.items():
        for mcs, ms in ((2, 2), (5, 5), (4, 2)):
            ms = min(ms, len(x))
            for method in ("eom", "leaf"):
                for allow in (False, True):
                    for eps in (0.0, 0.1):
                        yield (f"{name}_{method}_single{int(allow)}_mcs{mcs}_ms{ms}_eps{eps}", x, mcs, ms, eps,
                               method, allow)


FAMILIES = {"corpus": corpus, "exhaustive": exhaustive, "sweep": sweep, "known": known_answers,
            "sort": sort_fixtures, "configs": config_windows, "selection": selection}


def pack(store: dict) -> dict:
    """One concatenated array per field plus per-case lengths (-1 = absent)."""
    cases = store.pop("_cases")
    fields = sorted({key.split("/", 1)[1] for key in store})
    out = {"_cases": np.array(cases), "_fields": np.array(fields)}
    for field in fields:
        parts, lengths, shapes = [], [], []
        for case in cases:
            value = store.get(f"{case}/{field}")
            if value is None:
                lengths.append(-1)
                shapes.append(0)
                continue
            value = np.asarray(value)
            shapes.append(value.shape[1] if value.ndim == 2 else 0)
            lengths.append(value.shape[0] if value.ndim else 1)
            parts.append(value.reshape(-1))
        out[f"{field}//data"] = np.concatenate(parts) if parts else np.zeros(0)
        out[f"{field}//len"] = np.array(lengths, np.int64)
        out[f"{field}//cols"] = np.array(shapes, np.int64)
    return out


def main(selected):
    ref = Reference()
    import sklearn

    for family, gen in FAMILIES.items():
        if selected and family not in selected:
            continue
        store = {}
        names = []
        if family == "selection":
            for name, x, mcs, ms, eps, method, allow in gen():
                names.append(name)
                x = np.asarray(x, np.float64)
                store[f"{name}/x"] = x
                store[f"{name}/params"] = np.array([mcs, ms, eps], np.float64)
                store[f"{name}/options"] = np.array([1 if method == "leaf" else 0, int(allow)], np.int32)
                for key, value in sklearn_fit(x, mcs, ms, eps, method, allow).items():
                    store[f"{name}/sk_{key}"] = value
            store["_cases"] = names
            packed = pack(store)
            packed["_versions"] = np.array([sklearn.__version__, np.__version__, SCALAR])
            np.savez_compressed(HERE / f"golden_{family}.npz", **packed)
            print(family, len(names), "cases")
            continue
        for name, x, mcs, ms, eps in gen():
            names.append(name)
            x = np.asarray(x, np.float64)
            store[f"{name}/x"] = x
            store[f"{name}/params"] = np.array([mcs, ms, eps], np.float64)
            for precision in PRECISIONS:
                for key, value in ref.run(x, mcs, ms, eps, precision).items():
                    store[f"{name}/{precision}/ref_{key}"] = value
            if family == "sort":
                store[f"{name}/argsort"] = np.argsort(np.diff(x[:, 0]), kind="quicksort").astype(np.int32)
                continue
            if family == "configs" and len(x) > 1500:
                continue
            x32 = x.astype(np.float32).astype(np.float64)
            for tag, xs in (("sk", x), ("sk32", x32)):
                if tag == "sk32" and np.array_equal(x32, x):
                    continue  # exactly representable: scikit-learn sees the same input
                for key, value in sklearn_fit(xs, mcs, ms, eps).items():
                    store[f"{name}/{tag}_{key}"] = value
        store["_cases"] = names
        packed = pack(store)
        packed["_versions"] = np.array([sklearn.__version__, np.__version__, SCALAR])
        np.savez_compressed(HERE / f"golden_{family}.npz", **packed)
        print(family, len(names), "cases")


if __name__ == "__main__":
    main(set(sys.argv[1:]))
