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
    # merge_weights() through torch.autograd must return the forward's merge
    # weights and exactly the backward kernel's gradient.
    import torch

    from hdbscan_gb300 import merge_weights

    x = _windows(3, 2, 200, 6, "float64")
    X = torch.as_tensor(x, device=cuda).requires_grad_(True)
    weights, labels = merge_weights(X, min_cluster_size=10, min_samples=4)
    assert weights.shape == (2, 199) and labels.shape == (2, 200)
    g = torch.as_tensor(np.random.default_rng(2).normal(size=(2, 199)), device=cuda)
    (weights * g).sum().backward()
    plan, packed, buffers = _run(torch.as_tensor(x, device=cuda), 10, 4, "float64")
    torch.testing.assert_close(weights.detach().reshape(-1), buffers["link_w"], rtol=0, atol=0)
    direct = plan.backward(packed, buffers, g.reshape(-1)).reshape(2, 200, 6)
    # The kernel scatters with atomic adds, so two runs may round differently.
    torch.testing.assert_close(X.grad, direct, rtol=1e-12, atol=1e-12)
    assert X.grad.abs().sum() > 0


def _signature(buffers, offsets, w, ms):
    """The discrete structure the gradient holds fixed, for window w: Prim edges,
    sort order and, when min_samples > 2, which term attains each merge weight
    (core of u, core of v, or the distance) with the core neighbours involved."""
    lo, hi = int(offsets[w]), int(offsets[w + 1])
    e0, e1 = lo - w, hi - w - 1
    uv = buffers["edges_uv"][e0:e1]
    order = buffers["order"][e0:e1]
    parts = [uv.tobytes(), order.tobytes()]
    if ms > 2:
        core, nbr = buffers["core"][lo:hi], buffers["core_nbr"][lo:hi]
        u, v = uv[order, 0], uv[order, 1]
        weight = buffers["link_w"][e0:e1]
        term = np.where(weight == core[u], 0, np.where(weight == core[v], 1, 2))
        parts += [term.tobytes(), np.where(term == 0, nbr[u], np.where(term == 1, nbr[v], -1)).tobytes()]
    return b"".join(parts)


def _batched_losses(x_windows, g_windows, mcs, ms, precision="float64", chunk=96):
    """Loss sum(g * merge weights) and structure signature of every window, many windows per launch."""
    import torch

    from hdbscan_gb300._cuda import Plan

    losses, signatures = [], []
    for start in range(0, len(x_windows), chunk):
        xs = x_windows[start:start + chunk]
        gs = g_windows[start:start + chunk]
        offsets = np.concatenate([[0], np.cumsum([len(x) for x in xs])]).astype(np.int64)
        dtype = torch.float32 if precision == "float32" else torch.float64
        plan = Plan(offsets, xs[0].shape[1], min_cluster_size=mcs, min_samples=ms, precision=precision)
        buffers = plan.export_buffers(hierarchy=False, gradients=True)
        X = torch.as_tensor(np.concatenate(xs), dtype=dtype, device="cuda")
        _, status = plan.forward(X, exports=buffers)
        torch.cuda.synchronize()
        assert int(status.item()) == 0
        host = {k: v.cpu().numpy() for k, v in buffers.items()}
        for w in range(len(xs)):
            lo, hi = offsets[w], offsets[w + 1]
            weights = host["link_w"][lo - w:hi - w - 1].astype(np.float64)
            losses.append(float(np.dot(gs[w], weights)))
            signatures.append(_signature(host, offsets, w, ms))
        del plan, buffers, X
    return losses, signatures


def _central_difference_check(X0, mcs, ms, coords_per_window, seed, precision, h=1e-6, min_checked=None):
    """The analytic gradient (in `precision`) against float64 central differences on
    coordinates whose +-h steps leave the structure unchanged.  Returns the largest
    componentwise relative error |fd - an| / max(|fd|, |an|, 1e-3), the norm-wise
    relative error ||fd - an|| / ||fd|| over the checked coordinates, and their count."""
    import torch

    B, n, d = X0.shape
    rng = np.random.default_rng(seed)
    g = rng.normal(size=(B, n - 1))
    # Analytic gradient in the requested precision.
    Xp = torch.as_tensor(X0, dtype=torch.float32 if precision == "float32" else torch.float64, device="cuda")
    plan, packed, buffers = _run(Xp, mcs, ms, precision)
    dX = plan.backward(packed, buffers, torch.as_tensor(g.reshape(-1), device="cuda")).cpu().numpy()
    dX = dX.astype(np.float64).reshape(B, n, d)
    host = {k: v.cpu().numpy() for k, v in buffers.items()}
    offsets = np.arange(B + 1, dtype=np.int64) * n
    # The structure of the analytic run must be the float64 structure at X0 too.
    X64 = X0.astype(np.float64)
    base_losses, base_sigs = _batched_losses(list(X64), list(g), mcs, ms)
    analytic_sigs = [_signature(host, offsets, w, ms) for w in range(B)]
    picks, xs, gs = [], [], []
    for w in range(B):
        for _ in range(coords_per_window):
            i, k = int(rng.integers(n)), int(rng.integers(d))
            picks.append((w, i, k))
            for sign in (1.0, -1.0):
                x = X64[w].copy()
                x[i, k] += sign * h
                xs.append(x)
                gs.append(g[w])
    losses, sigs = _batched_losses(xs, gs, mcs, ms)
    errors, fds, ans = [], [], []
    for p, (w, i, k) in enumerate(picks):
        if not (sigs[2 * p] == sigs[2 * p + 1] == base_sigs[w] == analytic_sigs[w]):
            continue  # near a tie: the structure changes inside the step
        fd = (losses[2 * p] - losses[2 * p + 1]) / (2 * h)
        an = dX[w, i, k]
        errors.append(abs(fd - an) / max(abs(fd), abs(an), 1e-3))
        fds.append(fd)
        ans.append(an)
    checked = len(errors)
    assert checked >= (min_checked if min_checked is not None else len(picks) // 2), (checked, len(picks))
    fds, ans = np.asarray(fds), np.asarray(ans)
    normwise = float(np.linalg.norm(fds - ans) / np.linalg.norm(fds))
    return max(errors), normwise, checked


@pytest.mark.parametrize("ms", [2, 5])
def test_backward_matches_float64_central_differences(cuda, ms):
    worst, normwise, checked = _central_difference_check(_windows(11 + ms, 2, 160, 6, "float64"), 10, ms, 60, 5,
                                                         "float64")
    print(f"float64 n=160 d=6 ms={ms}: {checked} coordinates, max relative error {worst:.3e}, "
          f"norm-wise {normwise:.3e}")
    assert worst <= 1e-5, worst


@pytest.mark.parametrize("ms", [2, 5])
def test_float32_backward_matches_float64_central_differences(cuda, ms):
    # The float32 gradient against differences of the float64 forward on the same
    # (float32-representable) inputs.
    X0 = _windows(21 + ms, 2, 160, 6, "float32")
    worst, normwise, checked = _central_difference_check(X0, 10, ms, 60, 6, "float32")
    print(f"float32 n=160 d=6 ms={ms}: {checked} coordinates, max relative error {worst:.3e}, "
          f"norm-wise {normwise:.3e}")
    assert worst <= 1e-3, worst


def _same_structure_windows(X, mcs, ms, count):
    """Indices of the first `count` windows whose float32 and float64 structures agree
    (near-tied merge weights may order differently in the two precisions)."""
    g = [np.zeros(X.shape[1] - 1)] * len(X)
    _, sig64 = _batched_losses(list(X.astype(np.float64)), g, mcs, ms)
    _, sig32 = _batched_losses(list(X.astype(np.float32)), g, mcs, ms, precision="float32")
    same = [w for w in range(len(X)) if sig32[w] == sig64[w]]
    return same[:count]


@pytest.mark.parametrize("precision", ["float32", "float64"])
def test_backward_differentiation_config_shape(cuda, precision):
    # Windows of the differentiation configuration at full size (2048 points, 64
    # dims, mcs=15, ms=5), 200 random coordinates each.  float64: the first four
    # windows.  float32: the first four windows (of 16) whose float32 structure is
    # the float64 structure, since the differences are taken on the float64 forward.
    # With 64 coordinates per distance, the differences carry rounding noise of
    # about 1e-8 absolute (a few ulps of each changed weight over 2h), which is a
    # 1e-5 relative error for gradient components near 1e-3; the bound applies to
    # the norm-wise relative error, the componentwise one is reported.
    from hdbscan_gb300 import synthetic

    mcs, ms = 15, 5
    packed, offsets, params = synthetic.c4(windows=16 if precision == "float32" else 4)
    assert (params["min_cluster_size"], params["min_samples"]) == (mcs, ms)
    X = packed.reshape(-1, 2048, 64)
    if precision == "float32":
        X = X.astype(np.float32)
        keep = _same_structure_windows(X, mcs, ms, 4)
        assert len(keep) >= 2, keep
        X = X[keep]
    worst, normwise, checked = _central_difference_check(X, mcs, ms, 200, 9, precision)
    print(f"{precision} [{len(X)},2048,64] mcs=15 ms=5: {checked} of {200 * len(X)} coordinates, "
          f"norm-wise relative error {normwise:.3e}, max componentwise {worst:.3e}")
    tol = 1e-3 if precision == "float32" else 1e-5
    assert normwise <= tol, normwise
    assert worst <= 10 * tol, worst
