"""This library against the reference's own CUDA path on the same GPU.

oracle/ref_cuda.py compiles the reference's kernel strings with NVRTC and
`--fmad=false` and runs its host path (variant choice, distance kernel, core
distances, cluster kernel) exactly as hdbscan_gpu/_cuda.py:14-128 does -- the
production variants the reference launches: register-held Prim for windows up
to 1024 points, the parallel sort, the packed shared-memory workspace, the
unit-core and minimum-two shortcuts.  Labels must be equal bit for bit, on the
five seeded benchmark configurations at full size (ragged ones as dense calls
grouped by size under the reference's 512 MiB cap, as its callers must) and on
the golden corpus and seeded sweeps of the reference's parity tests.

Skipped when the reference's kernel strings were not generated
(oracle/build_ref.py needs the reference checkout when the tree is prepared).
"""

import numpy as np
import pytest

from tests.golden import golden

pytestmark = pytest.mark.gpu

CONFIGS = [("c1", None), ("c2", None), ("c3", "float32"), ("c3", "float64"), ("c4", None), ("c5", None)]


@pytest.fixture(scope="module")
def ref_cuda(cuda):
    from oracle import ref_cuda

    if not ref_cuda.available():
        pytest.skip("the reference's kernel strings (oracle/_ref/ref_cuda_source.json) were not generated")
    return ref_cuda


@pytest.mark.parametrize("config,precision", CONFIGS, ids=[f"{c}-{p or 'default'}" for c, p in CONFIGS])
def test_full_config_labels_equal_reference_cuda(ref_cuda, config, precision):
    import torch

    from hdbscan_gb300 import hdbscan_ragged, synthetic

    packed, offsets, p = synthetic.make(config)
    precision = precision or p["precision"]
    dtype = torch.float32 if precision == "float32" else torch.float64
    X = torch.as_tensor(packed, dtype=dtype, device="cuda")
    mcs, ms, eps = p["min_cluster_size"], p["min_samples"], p["cluster_selection_epsilon"]
    want = ref_cuda.cluster_windows(X, offsets, mcs, ms, eps, precision)
    got, _ = hdbscan_ragged(packed=X, offsets=offsets, min_cluster_size=mcs, min_samples=ms,
                            cluster_selection_epsilon=eps, precision=precision)
    torch.cuda.synchronize()
    want, got = want.cpu().numpy(), got.cpu().numpy()
    if not np.array_equal(got, want):
        bad = int(np.flatnonzero(got != want)[0])
        w = int(np.searchsorted(offsets, bad, side="right") - 1)
        raise AssertionError(f"{config} {precision}: labels differ from the reference CUDA path first in window "
                             f"{w} (n={offsets[w + 1] - offsets[w]})")


@pytest.mark.parametrize("family", ["corpus", "sweep", "known", "exhaustive"])
@pytest.mark.parametrize("precision", ["float32", "float64"])
def test_golden_cases_equal_reference_cuda(ref_cuda, family, precision):
    import torch

    from hdbscan_gb300 import hdbscan

    dtype = torch.float32 if precision == "float32" else torch.float64
    checked = 0
    for name, case in golden.load(family).items():
        x = case["x"]
        mcs, ms, eps = int(case["params"][0]), int(case["params"][1]), float(case["params"][2])
        if ms > len(x):
            continue  # rejected by both APIs' validation
        X = torch.as_tensor(x, dtype=dtype, device="cuda")
        if not bool(torch.isfinite(X).all()):
            continue  # non-finite input: both raise (checked by the API tests)
        try:
            want = ref_cuda.cluster(X, mcs, ms, eps, precision)
        except ValueError:
            continue  # the reference rejects it (overflow); the API tests cover our message
        got = hdbscan(X, min_cluster_size=mcs, min_samples=ms, cluster_selection_epsilon=eps, backend="cuda",
                      precision=precision)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(got.cpu().numpy(), want.cpu().numpy(), err_msg=f"{family}/{name} {precision}")
        checked += 1
    assert checked > 0
