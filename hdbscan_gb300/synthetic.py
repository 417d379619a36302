"""Seeded synthetic windows with the shapes and distributions of the benchmark configs.

The reference quotes its numbers on a private learned-embedding corpus that is
not distributed; these generators stand in for it.  Each returns
(packed [T, D] float64 host array, offsets [B+1] int64, parameters dict).

  c1  [1, 512, 8] float64: 5 isotropic Gaussians (centres U[-5,5]^8, std 0.5,
      92 points each) + 52 uniform noise points in [-8,8]^8; mcs=ms=5, eps=0.
  c2  [256, 1024, 16] float32: per window k~U{3..12} Gaussians, centres
      U[-4,4]^16, per-cluster std U[0.2,0.8], 10% uniform noise in [-6,6]^16;
      mcs=ms=2, eps=0.1.
  c3  512 windows, N log-uniform in [64, 4096], D=32: L2-normalised mixture of
      4..20 components on the unit sphere (angular std 0.15) + 5% uniform
      directions; mcs=ms=10, eps=0.05.
  c4  [64, 2048, 64]: 8 Gaussians (std 0.5, centres U[-3,3]^64) + 5% uniform
      noise in [-4.5,4.5]^64; mcs=15, ms=5.
  c5  96 windows, N ~ U[2048, 4096], D=128: 6..24 anisotropic Gaussians
      (diagonal std U[0.1,1.0], centres U[-4,4]^128) + 8% uniform noise in
      [-6,6]^128; mcs=32, ms=16, eps=0.
"""

from __future__ import annotations

import numpy as np

SEEDS = {"c1": 20261001, "c2": 20261002, "c3": 20261003, "c4": 20261004, "c5": 20261005}
PARAMS = {
    "c1": dict(min_cluster_size=5, min_samples=5, cluster_selection_epsilon=0.0, precision="float64"),
    "c2": dict(min_cluster_size=2, min_samples=2, cluster_selection_epsilon=0.1, precision="float32"),
    "c3": dict(min_cluster_size=10, min_samples=10, cluster_selection_epsilon=0.05, precision="float32"),
    "c4": dict(min_cluster_size=15, min_samples=5, cluster_selection_epsilon=0.0, precision="float32"),
    "c5": dict(min_cluster_size=32, min_samples=16, cluster_selection_epsilon=0.0, precision="float64"),
}


def _pack(windows):
    offsets = np.zeros(len(windows) + 1, dtype=np.int64)
    offsets[1:] = np.cumsum([len(w) for w in windows])
    return np.ascontiguousarray(np.concatenate(windows)), offsets


def _gaussian_window(rng, n, dims, k, centre_range, std, noise_fraction, noise_range):
    noise = int(round(noise_fraction * n))
    members = n - noise
    centres = rng.uniform(-centre_range, centre_range, (k, dims))
    stds = np.broadcast_to(np.asarray(std, dtype=np.float64), (k,) if np.ndim(std) <= 1 else np.shape(std))
    labels = rng.integers(0, k, members)
    if np.ndim(std) == 2:  # anisotropic, [k, dims]
        points = centres[labels] + rng.standard_normal((members, dims)) * std[labels]
    else:
        points = centres[labels] + rng.standard_normal((members, dims)) * np.asarray(stds)[labels, None]
    points = np.concatenate([points, rng.uniform(-noise_range, noise_range, (noise, dims))])
    return points[rng.permutation(n)]


def c1(seed=SEEDS["c1"]):
    rng = np.random.default_rng(seed)
    centres = rng.uniform(-5, 5, (5, 8))
    points = [c + 0.5 * rng.standard_normal((92, 8)) for c in centres]
    points.append(rng.uniform(-8, 8, (52, 8)))
    return (*_pack([np.concatenate(points)]), PARAMS["c1"])


def c2(seed=SEEDS["c2"], windows=256, n=1024, dims=16):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(windows):
        k = int(rng.integers(3, 13))
        std = rng.uniform(0.2, 0.8, k)
        out.append(_gaussian_window(rng, n, dims, k, 4.0, std, 0.10, 6.0))
    return (*_pack(out), PARAMS["c2"])


def _sphere(rng, count, dims):
    v = rng.standard_normal((count, dims))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def c3(seed=SEEDS["c3"], windows=512, dims=32, low=64, high=4096):
    rng = np.random.default_rng(seed)
    sizes = np.rint(np.exp(rng.uniform(np.log(low), np.log(high), windows))).astype(int)
    out = []
    for n in sizes:
        k = int(rng.integers(4, 21))
        noise = int(round(0.05 * n))
        centres = _sphere(rng, k, dims)
        labels = rng.integers(0, k, n - noise)
        points = centres[labels] + 0.15 * rng.standard_normal((n - noise, dims))
        points = np.concatenate([points, _sphere(rng, noise, dims)])
        points /= np.linalg.norm(points, axis=1, keepdims=True)
        out.append(points[rng.permutation(n)])
    return (*_pack(out), PARAMS["c3"])


def c4(seed=SEEDS["c4"], windows=64, n=2048, dims=64):
    rng = np.random.default_rng(seed)
    out = [_gaussian_window(rng, n, dims, 8, 3.0, np.full(8, 0.5), 0.05, 4.5) for _ in range(windows)]
    return (*_pack(out), PARAMS["c4"])


def c5(seed=SEEDS["c5"], windows=96, dims=128, low=2048, high=4096):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(windows):
        n = int(rng.integers(low, high + 1))
        k = int(rng.integers(6, 25))
        std = rng.uniform(0.1, 1.0, (k, dims))
        out.append(_gaussian_window(rng, n, dims, k, 4.0, std, 0.08, 6.0))
    return (*_pack(out), PARAMS["c5"])


CONFIGS = {"c1": c1, "c2": c2, "c3": c3, "c4": c4, "c5": c5}


def make(name, **kwargs):
    """(packed float64 [T, D], offsets [B+1], parameters) for config `name`."""
    return CONFIGS[name](**kwargs)
