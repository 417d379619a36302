"""Autotuner: measure the compiled forward variants per window-size bucket.

For every (precision, core mode, n bucket, D bucket) the tuner builds a batch
of seeded Gaussian-mixture windows of the bucket's largest size, large enough
to fill every SM, times each compiled variant that can hold such a window
(`hdb_list_variants`: Prim threads x slots per thread, register dimensions or
the materialized-matrix variant, CTAs per window) and keeps the fastest.  The result is
written to autotune_table.json next to this file; the package applies it
through `hdb_set_tuning` when the library loads.  Replaces the fixed launch
choice of the reference (hdbscan_gpu/_cuda.py:82-88).

Run on the target GPU:  python -m hdbscan_gb300.autotune [--quick]
                        [--n 2048 4096] [--precision float32] (re-tune those
                        buckets only; the other rules of the table are kept)

The environment variable HDB_AUTOTUNE_TABLE names another table file to load,
or "none" to run on the compiled-in defaults.
"""

from __future__ import annotations

import argparse
import ctypes
import json
import os
import time
from pathlib import Path

import numpy as np

TABLE = Path(__file__).resolve().with_name("autotune_table.json")
N_BUCKETS = (64, 128, 256, 512, 1024, 2048, 4096)
D_BUCKETS = (8, 16, 32, 64, 128)


FIELDS = 9


def _rules_array(rules):
    # Older tables hold 7- or 8-field rules: one CTA per window, one CTA per SM.
    rows = [list(r) + [1] * (FIELDS - len(r)) for r in rules]
    return np.ascontiguousarray(np.asarray(rows, dtype=np.int32).reshape(-1, FIELDS))


def table_path() -> Path | None:
    """The table the package loads: HDB_AUTOTUNE_TABLE, else the committed one; None = defaults."""
    override = os.environ.get("HDB_AUTOTUNE_TABLE")
    if override is None:
        return TABLE
    return None if override.lower() == "none" else Path(override)


def apply_table(lib, path: Path | None = None) -> int:
    """Load the tuning table into the library; returns the number of rules."""
    path = table_path() if path is None else path
    if path is None or not path.exists():
        return 0
    rules = [r["rule"] for r in json.loads(path.read_text())["rules"]]
    arr = _rules_array(rules)
    rc = lib.hdb_set_tuning(arr.ctypes.data_as(ctypes.c_void_p), len(rules))
    if rc != 0:
        raise RuntimeError(f"invalid autotune table {path}: {lib.hdb_last_error().decode()}")
    return len(rules)


def variants(lib, precision_code):
    count = lib.hdb_list_variants(precision_code, None, 0)
    out = np.zeros(5 * count, np.int32)
    lib.hdb_list_variants(precision_code, out.ctypes.data_as(ctypes.c_void_p), count)
    return [tuple(int(v) for v in out[5 * i:5 * i + 5]) for i in range(count)]


def _windows(rng, batch, n, dims):
    centres = rng.uniform(-4, 4, (8, dims))
    x = centres[rng.integers(0, 8, (batch, n))] + rng.normal(0, 0.5, (batch, n, dims))
    return x.reshape(batch * n, dims)


def _time_plan(plan, X, repeats):
    import torch

    ws = plan.workspace()
    labels = torch.empty(plan.points, dtype=torch.int32, device=plan.device)
    status = torch.empty(1, dtype=torch.int32, device=plan.device)
    plan.forward(X, labels=labels, workspace=ws, status=status)
    torch.cuda.synchronize()
    times = []
    for _ in range(repeats):
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record()
        plan.forward(X, labels=labels, workspace=ws, status=status)
        end.record()
        end.synchronize()
        times.append(start.elapsed_time(end))
    if int(status.item()) != 0:
        raise RuntimeError("forward reported a nonzero status during tuning")
    return float(np.median(times)), labels


def tune(quick=False, out: Path = TABLE, log=print, sizes=None, precisions=None):
    import torch

    from . import _lib
    from ._cuda import Plan

    lib = _lib.lib()
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    rng = np.random.default_rng(20261203)
    records = []
    for precision, code in (("float32", _lib.HDB_F32), ("float64", _lib.HDB_F64)):
        if precisions and precision not in precisions:
            continue
        available = variants(lib, code)
        for unit in (1, 0):
            ms = 2 if unit else 8
            for n in (sizes or (N_BUCKETS[2:5:2] if quick else N_BUCKETS)):
                for dims in (D_BUCKETS[1:3] if quick else D_BUCKETS):
                    cands = [v for v in available if v[0] * v[1] * v[3] >= n and (v[2] == 0 or dims <= v[2])
                             and (v[3] == 1 or n > 1024)]
                    # The smallest slot shape that holds n, plus every matrix variant.
                    if not cands:
                        continue
                    batch = max(sms * 2, 4) if n <= 1024 else sms
                    if precision == "float64" and dims >= 64:
                        batch = max(sms // 2, 8)
                    offsets = np.arange(batch + 1, dtype=np.int64) * n
                    X = torch.as_tensor(_windows(rng, batch, n, dims), device="cuda").to(
                        torch.float32 if precision == "float32" else torch.float64)
                    timings = []
                    reference_labels = None
                    for threads, slots, dp, cluster, per_sm in cands:
                        rule = [code, unit, n, dims, threads, slots, dp, cluster, per_sm]
                        arr = _rules_array([rule])
                        lib.hdb_set_tuning(arr.ctypes.data_as(ctypes.c_void_p), 1)
                        plan = Plan(offsets, dims, min_cluster_size=5, min_samples=ms, precision=precision)
                        desc = json.loads(plan.describe())["classes"][0]
                        if (desc["threads"], desc["vertices_per_thread"], desc["register_dims"],
                                desc["cluster"], desc["per_sm"]) != (threads, slots, dp, cluster, per_sm):
                            continue  # the rule was not applicable (e.g. shared memory)
                        ms_time, labels = _time_plan(plan, X, 3 if quick else 5)
                        host = labels.cpu().numpy()
                        if reference_labels is None:
                            reference_labels = host
                        elif not np.array_equal(host, reference_labels):
                            raise RuntimeError(f"variant {threads}x{slots}/{dp}/c{cluster}/s{per_sm} changed the labels")
                        timings.append((ms_time, rule))
                        del plan
                    lib.hdb_set_tuning(None, 0)
                    if not timings:
                        continue
                    timings.sort(key=lambda t: t[0])
                    best_ms, best = timings[0]
                    records.append({"rule": best, "ms": best_ms, "windows": batch,
                                    "candidates": [{"rule": r, "ms": t} for t, r in timings]})
                    log(f"{precision} unit={unit} n<={n} D<={dims}: {best[4]}x{best[5]} dims={best[6]} "
                        f"cluster={best[7]} per_sm={best[8]} {best_ms:.3f} ms ({len(timings)} candidates)")
    if sizes or precisions:
        # Partial re-tune: keep the previous rules of every bucket not measured now.
        measured = {tuple(r["rule"][:4]) for r in records}
        if out.exists():
            for old in json.loads(out.read_text())["rules"]:
                old["rule"] = list(old["rule"]) + [1] * (FIELDS - len(old["rule"]))
                if tuple(old["rule"][:4]) not in measured:
                    records.append(old)
    # Most specific first: smaller n and D buckets are checked before larger ones.
    records.sort(key=lambda r: (r["rule"][0], -r["rule"][1], r["rule"][2], r["rule"][3]))
    table = {"device": torch.cuda.get_device_name(0), "when": time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime()),
             "fields": ["precision", "unit_core", "n_max", "d_max", "threads", "slots", "dims", "cluster", "per_sm"],
             "rules": records}
    out.write_text(json.dumps(table, indent=1) + "\n")
    apply_table(lib, out)
    return table


if __name__ == "__main__":
    parser = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    parser.add_argument("--quick", action="store_true")
    parser.add_argument("--out", type=Path, default=TABLE)
    parser.add_argument("--n", type=int, nargs="*", help="only these n buckets")
    parser.add_argument("--precision", nargs="*", choices=["float32", "float64"])
    args = parser.parse_args()
    tune(args.quick, args.out, sizes=args.n, precisions=args.precision)
