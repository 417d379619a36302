"""Named small workloads that reach each kernel of the library, for profiling.

`python -m hdbscan_gb300.cases <name> [--repeat R]` builds a seeded batch,
runs the forward (and, for `backward`, the gradient) R times through a plan on
cuda:0 and checks the status word.  Each case is sized to hold a few hundred
MB on the device at most, so an ncu capture of one launch stays short; the
kernel each case is meant for is named below (the other kernels of the plan
run as well).

  tile64     64 windows x 256 points x 64 dims float32, ms=5: hdb_distance_kernel<float>
             (64x64 tiles; small float32 windows of wide points take the matrix variant)
  tile128    16 windows x 2048 x 64 float32, ms=5: hdb_distance128_kernel, hdb_core_rows_kernel,
             hdb_forward_kernel<float, 512, 4, 0, 1> (matrix Prim)
  tile128d32 16 windows x 2048 x 32 float32, ms=10: the same kernels at the ragged workload's
             dimension and list length (hdb_core_rows_kernel<float, 16>)
  tile64f64  2 windows x 3072 x 128 float64, ms=16: hdb_distance_kernel<double>, hdb_core_rows_kernel<double>
  points     64 windows x 1000 x 32 float32, ms=10: hdb_core_points_kernel (register windows)
  select     16 windows x 512 x 8 float32, ms=80: hdb_core_select_kernel (lists longer than 64)
  key        8 windows x 2048 x 16 float64, ms=40: hdb_core_matrix_key_kernel (float64 lists of 64)
  prepare    64 windows x 1024 x 16 bfloat16 input, L2-normalised: hdb_prepare_kernel
  backward   8 windows x 2048 x 64 float32, ms=5, forward + hdb_backward_kernel
  c2         64 windows x 1024 x 16 float32 of the uniform-batch workload: hdb_forward_kernel<float, 512, 2, 16, 1>
"""

from __future__ import annotations

import argparse

import numpy as np

CASES = {
    # name: (windows, n, dims, precision, min_samples, extra)
    "tile64": (64, 256, 64, "float32", 5, {}),
    "tile128": (16, 2048, 64, "float32", 5, {}),
    "tile128d32": (16, 2048, 32, "float32", 10, {}),
    "tile64f64": (2, 3072, 128, "float64", 16, {}),
    "points": (64, 1000, 32, "float32", 10, {}),
    "select": (16, 512, 8, "float32", 80, {}),
    "key": (8, 2048, 16, "float64", 40, {}),
    "prepare": (64, 1024, 16, "float32", 2, {"bf16": True}),
    "backward": (8, 2048, 64, "float32", 5, {"backward": True}),
    "c2": (64, 1024, 16, "float32", 2, {}),
}


def make_batch(windows, n, dims, seed=20261204):
    """Seeded Gaussian mixtures (8 centres in [-4, 4]^dims, std 0.5) plus 5% uniform noise."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(windows):
        centres = rng.uniform(-4, 4, (8, dims))
        noise = n // 20
        pts = centres[rng.integers(0, 8, n - noise)] + rng.normal(0, 0.5, (n - noise, dims))
        out.append(np.concatenate([pts, rng.uniform(-6, 6, (noise, dims))])[rng.permutation(n)])
    return np.concatenate(out)


def run(name, repeat=3):
    import torch

    from ._cuda import Plan, raise_for_status

    windows, n, dims, precision, ms, extra = CASES[name]
    x = make_batch(windows, n, dims)
    offsets = np.arange(windows + 1, dtype=np.int64) * n
    dtype = torch.float32 if precision == "float32" else torch.float64
    bf16 = extra.get("bf16", False)
    X = torch.as_tensor(x, device="cuda").to(torch.bfloat16 if bf16 else dtype)
    plan = Plan(offsets, dims, min_cluster_size=5, min_samples=ms, precision=precision,
                input_dtype=torch.bfloat16 if bf16 else None, normalize=bf16)
    workspace = plan.workspace()
    backward = extra.get("backward", False)
    exports = plan.export_buffers(hierarchy=False, gradients=True) if backward else None
    grad = torch.ones(plan.edges, dtype=dtype, device="cuda") if backward else None
    for _ in range(repeat):
        labels, status = plan.forward(X, workspace=workspace, exports=exports)
        if backward:
            plan.backward(X, exports, grad, workspace=workspace)
    torch.cuda.synchronize()
    raise_for_status(int(status.item()))
    return labels


if __name__ == "__main__":
    parser = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    parser.add_argument("name", choices=sorted(CASES))
    parser.add_argument("--repeat", type=int, default=3)
    args = parser.parse_args()
    run(args.name, args.repeat)
    print(f"case {args.name}: ok")
