"""Shared fixtures.  GPU tests carry @pytest.mark.gpu; `-m "not gpu"` runs the CPU suite."""

import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

# NumPy's SIMD argsort changes tie order on x86 hosts with AVX2/AVX-512; the
# reference's introsort follows the scalar path.  Tests that compare against
# np.argsort or scikit-learn run them in a subprocess with this environment.
SCALAR_SORT_ENV = {"NPY_DISABLE_CPU_FEATURES": "X86_V3 X86_V4 AVX512_ICL AVX512_SPR"}


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 box)")


def cuda_available() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def cuda():
    if not cuda_available():
        pytest.skip("no CUDA GPU")
    import torch

    return torch.device("cuda", 0)


def partition_equal(actual, expected) -> bool:
    """Same noise mask and a bijection between cluster ids (reference tests/conftest.py:116-134)."""
    actual, expected = np.asarray(actual), np.asarray(expected)
    if actual.shape != expected.shape or not np.array_equal(actual == -1, expected == -1):
        return False
    forward, reverse = {}, {}
    for observed, reference in zip(actual.flat, expected.flat):
        if reference == -1:
            continue
        observed, reference = int(observed), int(reference)
        if observed < 0:
            return False
        if forward.setdefault(observed, reference) != reference:
            return False
        if reverse.setdefault(reference, observed) != observed:
            return False
    return True


@pytest.fixture
def assert_partition():
    def check(actual, expected):
        assert partition_equal(actual, expected), f"partitions differ:\n{np.asarray(actual)}\n{np.asarray(expected)}"

    return check
