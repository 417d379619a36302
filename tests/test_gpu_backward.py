"""Gradients of the merge weights (no reference counterpart: the reference has none).

Loss L = sum_i w_i * merge_weight_i.  The backward kernel holds the discrete
structure fixed and routes each merge weight through the distance attaining
max(core_u, core_v, d_uv).  Checked against (1) torch autograd over the same
gathered distances and (2) float64 central finite differences (h = 1e-6) on
coordinates whose perturbation leaves the structure unchanged.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _windows(seed, batch, n, dims, precision):
    rng = np.random.default_rng(seed)
    centres = rng.uniform(-3, 3, (8, dims))
    x = centres[rng.integers(0, 8, (batch, n))] + rng.normal(0, 0.5, (batch, n, dims))
    return x.astype(np.float32 if precision == "float32" else np.float64)


def _run(X, mcs, ms, precision):
    import torch

    from hdbscan_gb300._cuda import plan_for

    B, n, d = X.shape
    offsets = np.arange(B + 1, dtype=np.int64) * n
    plan = plan_for(offsets, d, mcs, ms, 0.0, precision)
    buffers = plan.export_buffers(hierarchy=False, gradients=True)
    packed = X.reshape(B * n, d).contiguous()
    plan.forward(packed, exports=buffers)
    torch.cuda.synchronize()
    return plan, packed, buffers


def _gathered_loss(packed, buffers, g, n, B, ms):
    """The routing rule of the backward kernel, written with torch ops."""
    import torch

    uv = buffers["edges_uv"].long()
    order = buffers["order"].long()
    link_w = buffers["link_w"]
    rows = torch.arange(order.numel(), device=packed.device)
    window = rows // (n - 1)
    base = window * n
    e = order + window * (n - 1)
    u, v = uv[e, 0] + base, uv[e, 1] + base
    duv = torch.linalg.vector_norm(packed[u] - packed[v], dim=1)
    a, b = u, v
    if ms > 2:
        core, nbr = buffers["core"], buffers["core_nbr"].long()
        use_u = (duv.detach() != link_w) & (core[u] == link_w)
        use_v = (duv.detach() != link_w) & ~use_u & (core[v] == link_w)
        a = torch.where(use_u, u, torch.where(use_v, v, u))
        b = torch.where(use_u, nbr[u] + base, torch.where(use_v, nbr[v] + base, v))
    d = torch.linalg.vector_norm(packed[a] - packed[b], dim=1)
    return (g * d).sum()


@pytest.mark.parametrize("precision,ms", [("float64", 2), ("float64", 5), ("float32", 2), ("float32", 5)])
def test_backward_matches_autograd_over_gathered_distances(cuda, precision, ms):
    import torch

    B, n, d, mcs = 3, 300, 8, 15
    X = torch.as_tensor(_windows(7 + ms, B, n, d, precision), device=cuda)
    plan, packed, buffers = _run(X, mcs, ms, precision)
    g = torch.as_tensor(np.random.default_rng(1).normal(size=B * (n - 1)), dtype=packed.dtype, device=cuda)
    dX = plan.backward(packed, buffers, g)
    leaf = packed.detach().clone().requires_grad_(True)
    _gathered_loss(leaf, buffers, g, n, B, ms).backward()
    tol = 1e-10 if precision == "float64" else 1e-4
    torch.testing.assert_close(dX, leaf.grad, rtol=tol, atol=tol)


def test_merge_weights_autograd_function_matches_kernel(cuda):
    import torch

    from hdbscan_gb300 import merge_weights

    X = torch.as_tensor(_windows(3, 2, 200, 6, "float64"), device=cuda).requires_grad_(True)
    weights, labels = merge_weights(X, min_cluster_size=10, min_samples=4)
    assert weights.shape == (2, 199) and labels.shape == (2, 200)
    g = torch.randn_like(weights)
    (weights * g).sum().backward()
    assert X.grad is not None and torch.isfinite(X.grad).all()
    assert X.grad.abs().sum() > 0


@pytest.mark.parametrize("ms", [2, 5])
def test_backward_matches_float64_central_differences(cuda, ms):
    import torch

    B, n, d, mcs, h = 2, 160, 6, 10, 1e-6
    x0 = _windows(11 + ms, B, n, d, "float64")
    X = torch.as_tensor(x0, device=cuda)
    plan, packed, buffers = _run(X, mcs, ms, "float64")
    rng = np.random.default_rng(5)
    g = torch.as_tensor(rng.normal(size=B * (n - 1)), device=cuda)
    dX = plan.backward(packed, buffers, g).cpu().numpy().reshape(B, n, d)
    ref_uv = buffers["edges_uv"].cpu().numpy()
    ref_order = buffers["order"].cpu().numpy()

    def loss(x):
        _, _, b = _run(torch.as_tensor(x, device=cuda), mcs, ms, "float64")
        same = (np.array_equal(b["edges_uv"].cpu().numpy(), ref_uv)
                and np.array_equal(b["order"].cpu().numpy(), ref_order))
        return float((b["link_w"] * g).sum().item()), same

    checked = 0
    errors = []
    for _ in range(120):
        w, i, k = int(rng.integers(B)), int(rng.integers(n)), int(rng.integers(d))
        xp, xm = x0.copy(), x0.copy()
        xp[w, i, k] += h
        xm[w, i, k] -= h
        lp, sp = loss(xp)
        lm, sm = loss(xm)
        if not (sp and sm):
            continue  # near a tie: the structure changes inside the step
        fd = (lp - lm) / (2 * h)
        an = dX[w, i, k]
        scale = max(abs(fd), abs(an), 1e-3)
        errors.append(abs(fd - an) / scale)
        checked += 1
    assert checked >= 60
    assert max(errors) <= 1e-5, max(errors)
