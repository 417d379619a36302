"""Reader of the packed golden fixtures written by make_golden.py."""

from __future__ import annotations

from functools import lru_cache
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
FAMILIES = ("known", "corpus", "exhaustive", "sweep", "sort", "configs", "selection")


@lru_cache(maxsize=None)
def load(family: str) -> dict:
    """{case name: {field: array}} for one family."""
    raw = np.load(HERE / f"golden_{family}.npz", allow_pickle=False)
    cases = [str(c) for c in raw["_cases"]]
    out = {case: {} for case in cases}
    for field in (str(f) for f in raw["_fields"]):
        data, lengths, cols = raw[f"{field}//data"], raw[f"{field}//len"], raw[f"{field}//cols"]
        pos = 0
        for case, length, c in zip(cases, lengths, cols):
            if length < 0:
                continue
            size = int(length) * (int(c) if c else 1)
            value = data[pos:pos + size]
            pos += size
            out[case][field] = value.reshape(int(length), int(c)) if c else value
    return out


def versions(family: str):
    return [str(v) for v in np.load(HERE / f"golden_{family}.npz")["_versions"]]
