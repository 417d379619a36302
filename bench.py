"""Benchmark: windows/s of the batched HDBSCAN forward on one GB300.

Default workload (the config the headline metric is quoted on): 256 windows x
1024 points x 16 dims float32, mcs=ms=2, eps=0.1 (seeded Gaussian mixtures
standing in for the reference's private corpus; hdbscan_gb300/synthetic.py).

A step = one pass of the whole pipeline over the batch:
  value  device-resident: replay of the CUDA graph that holds the persistent
         ragged launch (inputs already in HBM), CUDA events per step, L2
         flushed (256 MiB write) between steps outside the events.
  e2e    the public hdbscan() call on a pinned host array: H2D of X, the
         forward, the status read and D2H of the labels inside the timing.
Also reported: the plain per-window launch of the same kernels (one launch per
window, no graph), labels bit-exact against the graph run and the oracle,
float32 agreement with the float64 oracle, per-phase device times (distance
and core phases as achieved GB/s against the measured HBM peak, Prim as ns per
iteration, hierarchy stages in us), the forward kernel's roofline, and the CPU
baselines: scikit-learn's HDBSCAN in a spawn process pool (one process per
host core) where scikit-learn is installed, and the oracle restatement on all
host threads.

`--impl reference` times the reference's own kernel code compiled for the CPU
(oracle/_ref) or, if that is absent, the oracle restatement, on all host
threads, same workload/metric.

`--gpus N` without a torchrun environment starts N ranks itself (torchrun on
127.0.0.1); each rank clusters its own shard (weak scaling).
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

CONFIG_NAMES = {"c2": "uniform batch [256,1024,16] float32 mcs=ms=2 eps=0.1",
                "c1": "single window [1,512,8] float64 mcs=ms=5",
                "c3": "ragged 512 windows N~logU[64,4096] D=32 mcs=ms=10 eps=0.05",
                "c4": "[64,2048,64] float32 mcs=15 ms=5",
                "c5": "ragged 96 windows N~U[2048,4096] D=128 float64 mcs=32 ms=16"}


def load_peaks():
    path = ROOT / "MEASURED_PEAKS.json"
    if path.exists():
        data = json.loads(path.read_text())
        return float(data["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.path = Path(tempfile.gettempdir()) / f"hdbscan_gb300_clocks_{os.getpid()}.csv"

    def __enter__(self):
        try:
            self.file = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
            # Start the timed region only once the sampler is writing (at most 3 s).
            deadline = time.perf_counter() + 3.0
            while time.perf_counter() < deadline and self.proc.poll() is None and self.path.stat().st_size == 0:
                time.sleep(0.01)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.file.close()

    def summary(self):
        if self.proc is None or not self.path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower() == "active":
                    reasons.add(name)
        try:
            self.path.unlink()
        except OSError:
            pass
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_reference_batch(packed, offsets, params, threads, prefer_reference=True):
    """Run the CPU implementation on the given windows; returns (labels, kind)."""
    import ctypes

    from oracle import oracle

    precision = params["precision"]
    mcs, ms, eps = params["min_cluster_size"], params["min_samples"], params["cluster_selection_epsilon"]
    ref_lib = ROOT / "oracle" / "_ref" / "libhdb_ref.so"
    if prefer_reference:
        try:
            from oracle import build_ref

            build_ref.build()
        except Exception:
            pass
    if prefer_reference and ref_lib.exists():
        lib = ctypes.CDLL(str(ref_lib))
        suffix = "f32" if precision == "float32" else "f64"
        fn = getattr(lib, f"hdb_ref_batch_{suffix}")
        fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                       ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        dtype = np.float32 if precision == "float32" else np.float64
        x = np.ascontiguousarray(packed, dtype=dtype)
        off = np.ascontiguousarray(offsets, dtype=np.int64)
        labels = np.empty(int(off[-1]), np.int32)
        status = np.zeros(len(off) - 1, np.int32)
        fn(x.ctypes.data, off.ctypes.data, len(off) - 1, x.shape[1], mcs, ms, eps, labels.ctypes.data,
           status.ctypes.data, threads)
        return labels, "reference"
    labels, _ = oracle.batch(packed, offsets, mcs, ms, eps, precision, threads=threads)
    return labels, "port"


def sample_windows(offsets, target_windows):
    count = min(len(offsets) - 1, target_windows)
    return offsets[: count + 1].copy(), count


# scikit-learn runs with the scalar NumPy sort on x86 (its AVX2/AVX-512 argsort
# orders ties differently from the reference's introsort) and one BLAS thread.
SCALAR_SORT_ENV = {"NPY_DISABLE_CPU_FEATURES": "X86_V3 X86_V4 AVX512_ICL AVX512_SPR"}
ONE_THREAD_ENV = {"OMP_NUM_THREADS": "1", "OPENBLAS_NUM_THREADS": "1", "MKL_NUM_THREADS": "1"}


def _sklearn_fit(job):
    x, mcs, ms, eps = job
    from sklearn.cluster import HDBSCAN

    model = HDBSCAN(algorithm="auto", metric="euclidean", cluster_selection_method="eom", allow_single_cluster=False,
                    alpha=1.0, n_jobs=1, copy=True, min_cluster_size=mcs, min_samples=ms, cluster_selection_epsilon=eps)
    return model.fit_predict(x).astype(np.int32)


def _sklearn_worker_ready(pause):
    import sklearn
    from sklearn.cluster import HDBSCAN  # noqa: F401  (imported before the timing)

    time.sleep(pause)  # hold this worker so every worker takes one warm-up task
    return sklearn.__version__, np.__version__, os.environ.get("NPY_DISABLE_CPU_FEATURES", "")


def sklearn_baseline(packed, offsets, params, count):
    """scikit-learn's HDBSCAN, the reference's CPU comparison (benchmarks/benchmark.py:90-94 there), on
    the first `count` windows: a persistent spawn process pool, one single-threaded process per host
    core, every worker started and warmed before the timing (the reference's start barrier,
    benchmarks/benchmark.py:222-238 there).  Float32 configurations give scikit-learn the
    float32-rounded points (it computes in float64)."""
    import importlib.util
    import multiprocessing
    import platform
    from concurrent.futures import ProcessPoolExecutor

    if importlib.util.find_spec("sklearn") is None:
        return {"unavailable": "scikit-learn is not installed on this host"}
    cores = len(os.sched_getaffinity(0))
    env = dict(ONE_THREAD_ENV)
    if platform.machine().lower() in ("x86_64", "amd64"):
        env.update(SCALAR_SORT_ENV)
    saved = {k: os.environ.get(k) for k in env}
    os.environ.update(env)  # inherited by the spawned workers
    try:
        pool = ProcessPoolExecutor(cores, mp_context=multiprocessing.get_context("spawn"))
        versions = list(pool.map(_sklearn_worker_ready, [0.5] * cores))[0]
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    mcs, ms, eps = params["min_cluster_size"], params["min_samples"], params["cluster_selection_epsilon"]
    x = packed if params["precision"] == "float64" else packed.astype(np.float32).astype(np.float64)
    jobs = [(np.ascontiguousarray(x[int(offsets[w]):int(offsets[w + 1])]), mcs, ms, eps) for w in range(count)]
    with pool:
        t0 = time.perf_counter()
        labels = list(pool.map(_sklearn_fit, jobs))
        elapsed = time.perf_counter() - t0
    return {"value": count / elapsed, "unit": "windows/s", "cores": cores, "kind": "sklearn",
            "sample": f"first {count} windows, {cores} spawn processes x 1 thread",
            "versions": {"sklearn": versions[0], "numpy": versions[1], "NPY_DISABLE_CPU_FEATURES": versions[2]},
            "labels": labels}


def phase_report(phase_ms, phase_launches, describe, D, itemsize, peak, core_distances):
    """Distance and core phases as achieved GB/s of algorithmic bytes (against the HBM peak), the
    distance phase also as pair-coordinates per second (its arithmetic rate), the forward as device
    ms.  Algorithmic bytes (sums over the windows of each kind):
      distance: read X (n*D*s) + write the n x n block (n^2*s), matrix-variant windows;
      core:     matrix windows read their block (n^2*s) + write core and neighbour (n*(s+4));
                recompute windows read X (n*D*s) + the same writes (these are SIMT-bound)."""
    matrix = [c for c in describe["classes"] if c["variant"] == "matrix"]
    recompute = [c for c in describe["classes"] if c["variant"] != "matrix"]
    points_m = sum(c["points"] for c in matrix)
    n2_m = sum(c["sum_n2"] for c in matrix)
    points_r = sum(c["points"] for c in recompute)
    out = {}
    dist_bytes = (n2_m + points_m * D) * itemsize
    if phase_launches["distance"]:
        gbs = dist_bytes / (phase_ms["distance"] / 1e3) / 1e9
        pair_coords = (n2_m - points_m) // 2 * D  # distinct pairs i < j times coordinates
        out["distance"] = {"ms": phase_ms["distance"], "launches": phase_launches["distance"], "bytes": dist_bytes,
                           "achieved_gbs": gbs, "frac_of_measured_hbm": gbs / peak,
                           "pair_coordinates": pair_coords,
                           "pair_coordinates_per_s": pair_coords / (phase_ms["distance"] / 1e3),
                           "note": "arithmetic-bound: FP64 and ALU pipes (float64), FMA-pipe issue (float32)"}
    if core_distances and phase_launches["core"]:
        core_bytes = n2_m * itemsize + (points_m + points_r) * (itemsize + 4) + points_r * D * itemsize
        gbs = core_bytes / (phase_ms["core"] / 1e3) / 1e9
        out["core"] = {"ms": phase_ms["core"], "launches": phase_launches["core"], "bytes": core_bytes,
                       "achieved_gbs": gbs, "frac_of_measured_hbm": gbs / peak}
    if phase_launches["prepare"]:
        out["prepare"] = {"ms": phase_ms["prepare"], "launches": phase_launches["prepare"]}
    out["forward"] = {"ms": phase_ms["forward"], "launches": phase_launches["forward"],
                      "note": "persistent Prim + hierarchy kernels: latency-bound, see stages"}
    out["note"] = "every launch serialized on one stream and event-timed (the graph overlaps them)"
    return out


def run_reference_arm(args, packed, offsets, params):
    threads = len(os.sched_getaffinity(0))
    sub_offsets, count = sample_windows(offsets, args.cpu_windows)
    sub = packed[: int(sub_offsets[-1])]
    times = []
    kind = "port"
    for step in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        _, kind = cpu_reference_batch(sub, sub_offsets, params, threads)
        elapsed = time.perf_counter() - t0
        if step >= args.warmup:
            times.append(elapsed)
    per_step = statistics.median(times)
    value = count / per_step
    reference_cuda = reference_cuda_timing(args, packed, offsets, params)
    line = {
        "impl": "reference", "metric": "windows_per_s", "value": value, "unit": "windows/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": per_step * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32" if params["precision"] == "float32" else "f64",
        "data": "synthetic", "config": {"workload": CONFIG_NAMES[args.config], "windows_timed": count},
        "cpu_baseline": {"value": value, "unit": "windows/s", "cores": threads, "kind": kind,
                         "sample": f"first {count} windows of the workload per step"},
        "e2e": {"value": value, "unit": "windows/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "reference_cuda": reference_cuda,
    }
    print(json.dumps(line))


def reference_cuda_timing(args, packed, offsets, params, passes=3):
    """The reference's own CUDA path on this GPU (oracle/ref_cuda.py: its kernel strings compiled
    by NVRTC with --fmad=false, its host path of hdbscan_gpu/_cuda.py:91-128) over the whole
    workload, device-resident input; ragged windows become dense calls grouped by size under its
    512 MiB distance-buffer cap, as its API requires.  None without a GPU or kernel strings."""
    try:
        import torch

        from oracle import ref_cuda
    except Exception as error:
        return {"unavailable": f"cannot import torch/oracle.ref_cuda: {error}"}
    if not torch.cuda.is_available():
        return {"unavailable": "no CUDA GPU on this host"}
    if not ref_cuda.available():
        return {"unavailable": "the reference's kernel strings were not generated (oracle/_ref/ref_cuda_source.json)"}
    precision = params["precision"]
    mcs, ms, eps = params["min_cluster_size"], params["min_samples"], params["cluster_selection_epsilon"]
    X = torch.as_tensor(packed, dtype=torch.float32 if precision == "float32" else torch.float64, device="cuda")
    ref_cuda.cluster_windows(X, offsets, mcs, ms, eps, precision)  # warm-up: NVRTC compiles
    torch.cuda.synchronize()
    times = []
    for _ in range(passes):
        t0 = time.perf_counter()
        ref_cuda.cluster_windows(X, offsets, mcs, ms, eps, precision)
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    windows = len(offsets) - 1
    per_pass = statistics.median(times)
    return {"value": windows / per_pass, "unit": "windows/s", "ms_per_pass": per_pass * 1e3, "passes": passes,
            "windows": windows, "note": "the reference's kernels and host path on this GPU, device-resident input, "
                                        "dense calls grouped by window size under its 512 MiB cap"}


def dist_env():
    """(rank, world, local rank) from the torchrun environment (1 process = 1 GPU)."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def rank_workload(config, rank, windows=None):
    """This rank's shard of a weak-scaling run: the config's batch drawn with the seed of shard `rank`
    (rank 0 is the config itself).  Windows are independent, so ranks exchange no data."""
    from hdbscan_gb300 import synthetic

    kwargs = {"windows": windows} if windows else {}
    if rank:
        kwargs["seed"] = synthetic.SEEDS[config] + 7919 * rank
    return synthetic.make(config, **kwargs)


def reduce_max(value, world, device):
    """Max over ranks (the slowest rank bounds the whole job)."""
    if world <= 1:
        return float(value)
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(windows_per_rank, world, ms_per_step):
    """Units all ranks processed per second of the max-over-ranks step time."""
    return windows_per_rank * world / (ms_per_step / 1e3)


def launch_ranks(gpus):
    """Start `gpus` ranks of this command under torchrun on 127.0.0.1 (one process per GPU); returns
    torchrun's exit status.  Rank 0 prints the JSON line."""
    import socket

    with socket.socket() as probe:
        probe.bind(("127.0.0.1", 0))
        port = probe.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={gpus}",
           "--master-addr", "127.0.0.1", "--master-port", str(port), str(Path(__file__).resolve()), *sys.argv[1:]]
    return subprocess.call(cmd)


def main():
    parser = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    parser.add_argument("--gpus", type=int, default=1)
    parser.add_argument("--steps", type=int, default=20)
    parser.add_argument("--warmup", type=int, default=5)
    parser.add_argument("--impl", choices=("ours", "reference"), default="ours")
    parser.add_argument("--config", choices=sorted(CONFIG_NAMES), default="c2")
    parser.add_argument("--cpu-windows", type=int, default=256)
    parser.add_argument("--plain-passes", type=int, default=2)
    parser.add_argument("--skip-cpu", action="store_true")
    parser.add_argument("--windows", type=int, default=None,
                        help="override the config's window count (small cases for ncu captures)")
    parser.add_argument("--stages", action="store_true", help="(always on) per-stage device time of the forward")
    parser.add_argument("--sklearn-windows", type=int, default=256,
                        help="windows of the scikit-learn CPU baseline sample (where scikit-learn is installed)")
    parser.add_argument("--backward", choices=("auto", "on", "off"), default="auto",
                        help="time forward+backward (default: on for the c4/c5 differentiation configs)")
    parser.add_argument("--profile", action="store_true",
                        help="only warm-up + timed graph replays (for ncu captures); prints nothing else")
    args = parser.parse_args()
    if args.warmup < 3:
        parser.error("--warmup must be >= 3")
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(launch_ranks(args.gpus))

    rank, world, local = dist_env()
    packed64, offsets, params = rank_workload(args.config, rank, args.windows)
    if args.impl == "reference":
        if rank == 0:
            run_reference_arm(args, packed64, offsets, params)
        return

    import torch

    import hdbscan_gb300
    from hdbscan_gb300 import _lib
    from hdbscan_gb300._cuda import Plan, raise_for_status

    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    precision = params["precision"]
    dtype = torch.float32 if precision == "float32" else torch.float64
    np_dtype = np.float32 if precision == "float32" else np.float64
    mcs, ms, eps = params["min_cluster_size"], params["min_samples"], params["cluster_selection_epsilon"]
    B = len(offsets) - 1
    T = int(offsets[-1])
    D = packed64.shape[1]
    host = np.ascontiguousarray(packed64, dtype=np_dtype)
    X = torch.from_numpy(host).to(device)

    plan = Plan(offsets, D, min_cluster_size=mcs, min_samples=ms, cluster_selection_epsilon=eps,
                precision=precision)
    workspace = plan.workspace()
    backward = args.backward == "on" or (args.backward == "auto" and args.config in ("c4", "c5"))
    exports = plan.export_buffers(hierarchy=False, gradients=True) if backward else None
    labels, status = plan.capture(X, workspace=workspace, exports=exports)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=device)
    stream = torch.cuda.current_stream(device)
    if backward:
        # Loss L = sum_i w_i * merge_weight_i with w ~ N(0, 1) seeded.
        grad_w = torch.as_tensor(np.random.default_rng(7).normal(size=plan.edges), dtype=dtype, device=device)
        dX = torch.zeros_like(X)

    def step():
        plan.replay()
        if backward:
            dX.zero_()
            plan.backward(X, exports, grad_w, dX=dX, workspace=workspace)

    # Warm-up + correctness of the graph run.
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    raise_for_status(int(status.item()))
    graph_labels = labels.cpu().numpy().copy()

    # ---- timed: graph replay, device resident ------------------------------
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    step_ms = []
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            flush.fill_(1)
            start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            start.record(stream)
            step()
            end.record(stream)
            end.synchronize()
            step_ms.append(start.elapsed_time(end))
    torch.cuda.synchronize()
    if args.profile:
        print(json.dumps({"profile_ms_per_step": float(np.mean(step_ms))}))
        return
    ms_per_step = reduce_max(float(np.mean(step_ms)), world, device)
    value = whole_job_rate(B, world, ms_per_step)

    # ---- per-phase device time: every launch serialized and event-timed ------
    # (hdb_plan_profile), with globaltimer stamps per window inside the forward.
    profiles = []
    stamps = torch.zeros((B, 8), dtype=torch.int64, device=device)
    for i in range(3):
        flush.fill_(1)
        profiles.append(plan.profile(X, labels=labels, workspace=workspace, status=status,
                                     exports={"stage_ns": stamps} if i == 0 else None))
    raise_for_status(int(status.item()))
    phase_ms = {name: float(np.mean([pr[name][0] for pr in profiles])) for name in _lib.PHASES}
    phase_launches = {name: profiles[0][name][1] for name in _lib.PHASES}
    kernel_ms_mean = phase_ms["forward"]
    st = stamps.cpu().numpy().astype(np.float64)
    stage_names = ["stage", "prim", "handoff_wait", "sort", "linkage", "condense", "select_label"]
    dur = np.diff(st, axis=1) / 1e3
    stages = {name: {"median_us": float(np.median(dur[:, i])), "max_us": float(dur[:, i].max())}
              for i, name in enumerate(stage_names)}
    sizes = np.diff(offsets)
    per_iter = dur[:, 1] * 1e3 / np.maximum(sizes - 1, 1)
    stages["prim_ns_per_iteration"] = {"median": float(np.median(per_iter)),
                                       "largest_window": float(per_iter[int(np.argmax(sizes))])}
    stages["note"] = "per window, from the serialized profile run (globaltimer stamps)"

    # ---- plain per-window launches of the same kernels ----------------------
    plain_plans = {}
    plain_labels = torch.empty(T, dtype=torch.int32, device=device)
    one_ws = {}
    for w in range(B):
        n = int(offsets[w + 1] - offsets[w])
        if n not in plain_plans:
            plain_plans[n] = Plan(np.array([0, n]), D, min_cluster_size=mcs, min_samples=ms,
                                  cluster_selection_epsilon=eps, precision=precision)
            one_ws[n] = plain_plans[n].workspace()
    plain_status = torch.empty(1, dtype=torch.int32, device=device)

    plain_exports = {n: plain_plans[n].export_buffers(hierarchy=False, gradients=True) for n in plain_plans} \
        if backward else {}

    def plain_pass():
        for w in range(B):
            lo, hi = int(offsets[w]), int(offsets[w + 1])
            p = plain_plans[hi - lo]
            ex = plain_exports.get(hi - lo)
            p.forward(X[lo:hi], labels=plain_labels[lo:hi], workspace=one_ws[hi - lo], status=plain_status,
                      exports=ex)
            if backward:
                p.backward(X[lo:hi], ex, grad_w[lo - w:hi - w - 1], dX=dX[lo:hi], workspace=one_ws[hi - lo])

    plain_pass()
    torch.cuda.synchronize()
    plain_ms = []
    for _ in range(args.plain_passes):
        flush.fill_(1)
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record(stream)
        plain_pass()
        end.record(stream)
        end.synchronize()
        plain_ms.append(start.elapsed_time(end))
    plain_value = (whole_job_rate(B, world, reduce_max(float(np.mean(plain_ms)), world, device))
                   if plain_ms else None)
    plain_exact = bool(np.array_equal(plain_labels.cpu().numpy(), graph_labels))

    # ---- end to end through the public API ----------------------------------
    pinned = torch.from_numpy(host).pin_memory()
    uniform = len(set(np.diff(offsets).tolist())) == 1
    e2e_ms = []
    for step in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        if backward:
            Xd = pinned.to(device, non_blocking=True).requires_grad_(True)
            weights, result = hdbscan_gb300.merge_weights(Xd, offsets, min_cluster_size=mcs, min_samples=ms,
                                                          cluster_selection_epsilon=eps, precision=precision)
            loss = (weights * grad_w).sum()
            loss.backward()
            loss_value = float(loss.item())
        elif uniform:
            n = int(offsets[1])
            result = hdbscan_gb300.hdbscan(pinned.view(B, n, D).to(device, non_blocking=True),
                                           min_cluster_size=mcs, min_samples=ms,
                                           cluster_selection_epsilon=eps, backend="cuda", precision=precision)
        else:
            result, _ = hdbscan_gb300.hdbscan_ragged(packed=pinned.to(device, non_blocking=True), offsets=offsets,
                                                     min_cluster_size=mcs, min_samples=ms,
                                                     cluster_selection_epsilon=eps, precision=precision)
        out = result.cpu()
        if step >= args.warmup:
            e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e_exact = bool(np.array_equal(out.numpy().reshape(-1), graph_labels))
    e2e_value = whole_job_rate(B, world, reduce_max(float(np.median(e2e_ms)), world, device))

    # ---- checks after the timing: oracle parity on a sample, float32 vs the --
    # float64 oracle (the checker in float64 on the same float32-rounded input)
    from oracle import oracle
    from tests.conftest import partition_equal

    sample = list(range(0, B, max(1, B // 8)))[:8]
    oracle_exact = True
    for w in sample:
        lo, hi = int(offsets[w]), int(offsets[w + 1])
        o = oracle.cluster(host[lo:hi], mcs, ms, eps, precision)
        oracle_exact &= bool(np.array_equal(o["labels"], graph_labels[lo:hi]))
    agreement = None
    if precision == "float32":
        count = min(B, 64)
        sub = offsets[:count + 1]
        want = oracle.batch_ex(host[:int(sub[-1])].astype(np.float64), sub, mcs, ms, eps, "float64")
        check_exports = plan.export_buffers(hierarchy=False, gradients=True)
        plan.forward(X, labels=labels, workspace=workspace, status=status, exports=check_exports)
        got_w = check_exports["link_w"].cpu().numpy()
        torch.cuda.synchronize()
        exact, worst = 0, 0.0
        for w in range(count):
            lo, hi = int(sub[w]), int(sub[w + 1])
            exact += partition_equal(graph_labels[lo:hi], want["labels"][lo:hi])
            a = np.sort(got_w[lo - w:hi - w - 1].astype(np.float64))
            b = np.sort(want["link_w"][lo - w:hi - w - 1])
            worst = max(worst, float(np.max(np.abs(a - b) / np.maximum(np.abs(b), np.finfo(np.float64).tiny))))
        agreement = {"windows": count, "exact_partitions": exact, "exact_partition_rate": exact / count,
                     "max_rel_merge_weight_error": worst,
                     "against": "float64 oracle on the same float32-rounded input (first windows)"}

    # ---- CPU baselines (rank 0): scikit-learn in a spawn pool, oracle port ---
    cpu = None
    cpu_port = None
    if not args.skip_cpu and rank == 0:
        threads = len(os.sched_getaffinity(0))
        sub_offsets, count = sample_windows(offsets, args.cpu_windows)
        t0 = time.perf_counter()
        _, kind = cpu_reference_batch(host[: int(sub_offsets[-1])], sub_offsets, params, threads,
                                      prefer_reference=False)
        elapsed = time.perf_counter() - t0
        cpu_port = {"value": count / elapsed, "unit": "windows/s", "cores": threads, "kind": kind,
                    "sample": f"first {count} of {B} windows, oracle restatement on {threads} host threads"}
        sk = sklearn_baseline(host.astype(np.float64), offsets, params, min(count, args.sklearn_windows))
        if "labels" in sk:
            got = [graph_labels[int(offsets[w]):int(offsets[w + 1])] for w in range(len(sk["labels"]))]
            sk["exact_partition_rate_vs_ours"] = float(np.mean([partition_equal(g, l)
                                                                for g, l in zip(got, sk.pop("labels"))]))
            cpu = sk
        else:
            cpu = dict(cpu_port, sklearn=sk)

    # ---- roofline of the forward kernel -------------------------------------
    peak, peak_kind = load_peaks()
    itemsize = 4 if precision == "float32" else 8
    sizes = np.diff(offsets)
    describe = json.loads(plan.describe())
    # Algorithmic bytes per launch: read X (N*D*s) + write labels (4N) per window,
    # plus the N^2*s distance block read by windows of the matrix variant.
    algo_bytes = float(np.sum(sizes * D * itemsize + sizes * 4))
    algo_bytes += float(sum(c["sum_n2"] for c in describe["classes"] if c["variant"] == "matrix") * itemsize)
    achieved = algo_bytes / (kernel_ms_mean / 1e3) / 1e9
    traffic = None
    traffic_path = ROOT / "profiles" / f"traffic_{args.config}.json"
    if traffic_path.exists():
        traffic = json.loads(traffic_path.read_text()).get("dram_bytes_per_launch")
    launches_per_step = sum(phase_launches.values())  # this library's kernels in one forward
    if backward:
        launches_per_step += 1  # the backward kernel (dX is zeroed by torch)
    line = {
        "metric": "windows_per_s", "value": value, "unit": "windows/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32" if precision == "float32" else "f64", "data": "synthetic",
        "config": {"workload": CONFIG_NAMES[args.config], "windows": B, "points": T, "dims": D,
                   "l2": "256 MiB flush between timed steps", "graph": True, "parallelism": "replicas"},
        "points_per_s": T * world / (ms_per_step / 1e3),
        "plain_per_window": {"value": plain_value, "unit": "windows/s", "labels_bit_exact": plain_exact},
        "speedup_vs_plain": value / plain_value if plain_value else None,
        "labels_bit_exact": {"graph_vs_oracle_sample": oracle_exact, "e2e_vs_graph": e2e_exact},
        "e2e": {"value": e2e_value, "unit": "windows/s", "h2d_bytes_per_step": int(host.nbytes),
                "d2h_bytes_per_step": int(T * 4 + (host.itemsize if backward else 4))},
        "mode": "forward+backward" if backward else "forward",
        "gpu_launches": launches_per_step * args.steps,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                     "kernel": "hdb_forward_kernel", "kernel_ms": kernel_ms_mean,
                     "note": "latency-bound (serial Prim/tree chains); algorithmic bytes per launch over the "
                             "forward kernels' event-timed duration"},
        "cpu_baseline": cpu,
        "cpu_baseline_port": cpu_port,
        "float32_vs_float64_oracle": agreement,
        "phases": phase_report(phase_ms, phase_launches, describe, D, itemsize, peak, ms > 2),
        "stages": stages,
        "clocks": clocks.summary(),
        "plan": describe["classes"],
    }
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
