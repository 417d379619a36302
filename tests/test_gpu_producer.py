"""Producer stage: bfloat16 / float16 encoder embeddings converted on the
device and optional L2 normalisation, against the oracle on the same values.

Conversion to float32 is exact, so the oracle sees the same coordinates; the
normalisation is restated by oracle.normalize_rows (coordinate-order sum of
squares, correctly rounded sqrt and division)."""

import numpy as np
import pytest

from oracle import oracle

pytestmark = pytest.mark.gpu


def _embeddings(seed, n, dims, k=6):
    rng = np.random.default_rng(seed)
    centres = rng.normal(0, 1, (k, dims))
    x = centres[rng.integers(0, k, n)] + rng.normal(0, 0.15, (n, dims))
    x[:3] = 0.0  # zero vectors stay as they are
    return x


@pytest.mark.parametrize("half", ["bfloat16", "float16"])
@pytest.mark.parametrize("normalize", [False, True])
def test_half_input_matches_oracle(cuda, half, normalize):
    import torch

    from hdbscan_gb300 import hdbscan

    dtype = getattr(torch, half)
    x = torch.as_tensor(_embeddings(1, 900, 24), device="cuda").to(dtype)
    labels, probs = hdbscan(x, min_cluster_size=10, min_samples=5, precision="float32", normalize=normalize,
                            return_probabilities=True)
    x32 = x.float().cpu().numpy()  # exact widening
    if normalize:
        x32 = oracle.normalize_rows(x32, "float32")
    o = oracle.cluster(x32, 10, 5, 0.0, "float32")
    np.testing.assert_array_equal(labels.cpu().numpy(), o["labels"])
    np.testing.assert_array_equal(probs.cpu().numpy().view(np.uint32), o["probabilities"].view(np.uint32))


@pytest.mark.parametrize("precision", ["float32", "float64"])
def test_normalize_in_compute_precision(cuda, precision):
    from hdbscan_gb300 import hdbscan

    x = _embeddings(2, 4 * 500, 16).reshape(4, 500, 16)
    labels = hdbscan(x, min_cluster_size=8, min_samples=4, precision=precision, normalize=True).cpu().numpy()
    for b in range(4):
        xb = oracle.normalize_rows(x[b], precision)
        np.testing.assert_array_equal(labels[b], oracle.cluster(xb, 8, 4, 0.0, precision)["labels"])


def test_ragged_bfloat16_windows(cuda):
    import torch

    from hdbscan_gb300 import hdbscan_ragged

    wins = [torch.as_tensor(_embeddings(s, n, 32), device="cuda").to(torch.bfloat16) for s, n in
            ((3, 200), (4, 1500), (5, 3000))]
    labels, offsets = hdbscan_ragged(wins, min_cluster_size=12, min_samples=6, precision="float32", normalize=True)
    labels = labels.cpu().numpy()
    for w, win in enumerate(wins):
        xw = oracle.normalize_rows(win.float().cpu().numpy(), "float32")
        np.testing.assert_array_equal(labels[offsets[w]:offsets[w + 1]], oracle.cluster(xw, 12, 6, 0.0, "float32")["labels"])


def test_backward_refuses_producer_plans(cuda):
    import torch

    from hdbscan_gb300._cuda import Plan

    plan = Plan(np.array([0, 50]), 4, min_cluster_size=5, min_samples=3, precision="float32", normalize=True)
    X = torch.randn(50, 4, device="cuda")
    ex = plan.export_buffers(hierarchy=False, gradients=True)
    plan.forward(X, exports=ex)
    with pytest.raises(ValueError, match="normalisation"):
        plan.backward(X, ex, torch.ones(plan.edges, device="cuda"))
