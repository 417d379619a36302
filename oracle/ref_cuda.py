"""The reference's own CUDA path, run on this GPU (test infrastructure only).

The reference (CosineAI/hdbscan) keeps its kernels as CUDA-C strings, JIT-compiles
them with NVRTC through CuPy (`--fmad=false`, hdbscan_gpu/_cuda.py:14-42), picks the
production cluster-kernel variant per window size (hdbscan_gpu/_cuda.py:46-88) and
runs distance kernel -> finiteness checks -> `cp.partition` core distances -> cluster
kernel (hdbscan_gpu/_cuda.py:91-128).  CuPy is not installed here, so this module
restates that host path: NVRTC and the CUDA driver through ctypes, torch for memory,
streams, the finiteness reductions and the k-th-smallest selection (`torch.kthvalue`,
value-exact like `cp.partition`).  The kernel strings are those of the reference
checkout, written by oracle/build_ref.py into oracle/_ref/ref_cuda_source.json
(git-ignored, never committed); nothing here is this project's kernel code.

Only tests and the reference arm of bench.py use this module: it is the reference's
GPU path for parity and for a GPU-to-GPU comparison, never the product.
"""

from __future__ import annotations

import ctypes
import ctypes.util
import json
import threading
from pathlib import Path

import numpy as np

SOURCE = Path(__file__).resolve().parent / "_ref" / "ref_cuda_source.json"
MAX_DISTANCE_BYTES = 512 * 1024 * 1024  # the reference's dense-buffer cap (hdbscan_gpu/_api.py:8)
MAX_SAMPLES = 4096

_lock = threading.Lock()
_state = {}


def available() -> bool:
    """True when the generated kernel strings and NVRTC are present."""
    if not SOURCE.exists():
        return False
    try:
        _libs()
    except OSError:
        return False
    return True


def _load(names):
    for name in names:
        try:
            return ctypes.CDLL(name)
        except OSError:
            continue
    raise OSError(f"none of {names} could be loaded")


def _libs():
    if "nvrtc" not in _state:
        _state["nvrtc"] = _load(["libnvrtc.so", "libnvrtc.so.13", "/usr/local/cuda/lib64/libnvrtc.so"])
        _state["cuda"] = _load(["libcuda.so.1", "libcuda.so"])
    return _state["nvrtc"], _state["cuda"]


def _check_nvrtc(rc, what):
    if rc:
        nvrtc, _ = _libs()
        nvrtc.nvrtcGetErrorString.restype = ctypes.c_char_p
        raise RuntimeError(f"{what}: {nvrtc.nvrtcGetErrorString(rc).decode()}")


def _check_cu(rc, what):
    if rc:
        _, cu = _libs()
        message = ctypes.c_char_p()
        cu.cuGetErrorString(rc, ctypes.byref(message))
        raise RuntimeError(f"{what}: CUDA driver error {rc} ({(message.value or b'').decode()})")


def _sources():
    if "sources" not in _state:
        _state["sources"] = json.loads(SOURCE.read_text())
    return _state["sources"]


def _arch():
    import torch

    major, minor = torch.cuda.get_device_capability()
    suffix = "a" if major >= 9 else ""
    return f"sm_{major}{minor}{suffix}"


def _compile(source: str, name: str):
    """CUfunction of `name` in `source`, compiled by NVRTC with the reference's options."""
    import torch

    key = (torch.cuda.current_device(), hash(source), name)
    with _lock:
        if key in _state:
            return _state[key]
        nvrtc, cu = _libs()
        _check_cu(cu.cuInit(0), "cuInit")
        prog = ctypes.c_void_p()
        _check_nvrtc(nvrtc.nvrtcCreateProgram(ctypes.byref(prog), source.encode(), f"{name}.cu".encode(), 0, None,
                                              None), "nvrtcCreateProgram")
        # The reference passes --fmad=false (hdbscan_gpu/_cuda.py:24, :41); the
        # architecture is this GPU's, as CuPy compiles for the current device.
        opts = [b"--fmad=false", f"--gpu-architecture={_arch()}".encode()]
        arr = (ctypes.c_char_p * len(opts))(*opts)
        rc = nvrtc.nvrtcCompileProgram(prog, len(opts), arr)
        if rc:
            size = ctypes.c_size_t()
            nvrtc.nvrtcGetProgramLogSize(prog, ctypes.byref(size))
            log = ctypes.create_string_buffer(size.value)
            nvrtc.nvrtcGetProgramLog(prog, log)
            raise RuntimeError(f"NVRTC failed on {name}:\n{log.value.decode(errors='replace')}")
        size = ctypes.c_size_t()
        _check_nvrtc(nvrtc.nvrtcGetCUBINSize(prog, ctypes.byref(size)), "nvrtcGetCUBINSize")
        image = ctypes.create_string_buffer(size.value)
        _check_nvrtc(nvrtc.nvrtcGetCUBIN(prog, image), "nvrtcGetCUBIN")
        nvrtc.nvrtcDestroyProgram(ctypes.byref(prog))
        torch.cuda.current_stream()  # the runtime's primary context is current on this thread
        module = ctypes.c_void_p()
        _check_cu(cu.cuModuleLoadData(ctypes.byref(module), image), "cuModuleLoadData")
        function = ctypes.c_void_p()
        _check_cu(cu.cuModuleGetFunction(ctypes.byref(function), module, name.encode()), "cuModuleGetFunction")
        _state[key] = (module, function)
        return _state[key]


def _kernels(precision, shared_workspace=False, unit_core=False, minimum_two=False, register_prim=0, threads=None,
             parallel_sort=False):
    """The two kernels of one variant, assembled as hdbscan_gpu/_cuda.py:18-42 does."""
    src = _sources()
    threads = threads or src["cluster_threads"]
    common = src["header"][precision]
    distances = (common + 'extern "C" __global__ void distances_kernel(const Real* x, const int* params, '
                 'Real* distances) {' + src["distance"] + "}")
    clusters = (
        common + "#define PARALLEL_PRIM\n"
        + ("#define CUDA_PACKED_WORKSPACE\n" if shared_workspace else "")
        + ("#define UNIT_CORE\n" if unit_core else "")
        + ("#define MINIMUM_TWO\n" if minimum_two else "")
        + (f"#define REGISTER_PRIM {register_prim}\n" if register_prim else "")
        + ("#define PARALLEL_SORT\n" if parallel_sort else "")
        + f'extern "C" __global__ __launch_bounds__({threads}) void clusters_kernel(const Real* distances, '
        + "const Real* core, const int* params, const Real* options, int* labels, int* integers, Real* reals) {"
        + src["cluster"] + "}")
    return _compile(distances, "distances_kernel")[1], _compile(clusters, "clusters_kernel")[1]


def _func_attribute(function, attribute):
    _, cu = _libs()
    value = ctypes.c_int()
    _check_cu(cu.cuFuncGetAttribute(ctypes.byref(value), attribute, function), "cuFuncGetAttribute")
    return value.value


def _production(precision, size, minimum, samples):
    """Variant choice of hdbscan_gpu/_cuda.py:46-88: block width, register Prim,
    parallel sort, and the packed shared workspace when it fits the opt-in limit."""
    import torch

    threads = max(32, 1 << (size - 1).bit_length()) if size <= 1024 else _sources()["cluster_threads"]
    options = dict(unit_core=samples <= 2, minimum_two=minimum == 2, register_prim=1 if size <= 1024 else 0,
                   threads=threads, parallel_sort=size <= 1024)
    required = size * (19 + 3 * (4 if precision == "float32" else 8))
    _, shared_kernel = _kernels(precision, shared_workspace=True, **options)
    _, cu = _libs()
    limit = ctypes.c_int()
    device = ctypes.c_int()
    _check_cu(cu.cuDeviceGet(ctypes.byref(device), torch.cuda.current_device()), "cuDeviceGet")
    _check_cu(cu.cuDeviceGetAttribute(ctypes.byref(limit), 97, device), "cuDeviceGetAttribute")  # smem opt-in
    capacity = limit.value - _func_attribute(shared_kernel, 1)  # CU_FUNC_ATTRIBUTE_SHARED_SIZE_BYTES
    if required <= capacity:
        _check_cu(cu.cuFuncSetAttribute(shared_kernel, 8, capacity), "cuFuncSetAttribute")  # max dynamic smem
        return shared_kernel, required, threads
    _, global_kernel = _kernels(precision, **options)
    return global_kernel, 0, threads


def _launch(function, grid, block, smem, stream, *args):
    _, cu = _libs()
    holders = [ctypes.c_void_p(a) for a in args]
    params = (ctypes.c_void_p * len(holders))(*[ctypes.addressof(h) for h in holders])
    _check_cu(cu.cuLaunchKernel(function, grid, 1, 1, block, 1, 1, smem, ctypes.c_void_p(stream), params, None),
              "cuLaunchKernel")


def cluster(x, min_cluster_size, min_samples, epsilon, precision):
    """Labels [B, N] (or [N]) of a torch CUDA tensor [B, N, D] (or [N, D]) by the
    reference's CUDA path: hdbscan_gpu/_cuda.py:91-128 step by step."""
    import torch

    dtype = torch.float32 if precision == "float32" else torch.float64
    x = x.to(dtype).contiguous()
    if not bool(torch.isfinite(x).all().item()):  # host sync #1 (_cuda.py:98-99)
        raise ValueError("X must contain only finite values in the requested precision")
    unbatched = x.ndim == 2
    if unbatched:
        x = x[None]
    batch, n, dimensions = x.shape
    params = torch.tensor([n, dimensions, batch, min_cluster_size], dtype=torch.int32, device=x.device)
    options = torch.tensor([epsilon], dtype=dtype, device=x.device)
    distance_kernel, _ = _kernels(precision)
    cluster_kernel, shared_mem, threads = _production(precision, n, min_cluster_size, min_samples)
    stream = torch.cuda.current_stream().cuda_stream
    distances = torch.empty((batch, n, n), dtype=dtype, device=x.device)
    _launch(distance_kernel, (distances.numel() + 255) // 256, 256, 0, stream, x.data_ptr(), params.data_ptr(),
            distances.data_ptr())
    if not bool(torch.isfinite(distances).all().item()):  # host sync #2 (_cuda.py:112-113)
        raise ValueError("pairwise distances overflow the requested precision")
    core = distances if min_samples <= 2 else \
        torch.kthvalue(distances, min_samples, dim=-1).values.contiguous()  # cp.partition(d, ms-1)[..., ms-1]
    labels = torch.empty((batch, n), dtype=torch.int32, device=x.device)
    src = _sources()
    integers = torch.empty((1,) if shared_mem else (batch, src["integer_workspace"] * n), dtype=torch.int32,
                           device=x.device)
    reals = torch.empty((1,) if shared_mem else (batch, src["real_workspace"] * n), dtype=dtype, device=x.device)
    _launch(cluster_kernel, batch, threads, shared_mem, stream, distances.data_ptr(), core.data_ptr(),
            params.data_ptr(), options.data_ptr(), labels.data_ptr(), integers.data_ptr(), reals.data_ptr())
    return labels[0] if unbatched else labels


def cluster_windows(packed, offsets, min_cluster_size, min_samples, epsilon, precision):
    """Labels of a ragged batch as a caller of the reference must compute them: its
    API takes dense [B, N, D] batches under a 512 MiB distance-buffer cap
    (hdbscan_gpu/_api.py:77-83), so windows are grouped by size, in order of first
    appearance, and each group is cut into chunks under the cap."""
    import torch

    offsets = np.asarray(offsets, dtype=np.int64)
    sizes = np.diff(offsets)
    itemsize = 4 if precision == "float32" else 8
    out = torch.empty(int(offsets[-1]), dtype=torch.int32, device=packed.device)
    groups = {}
    for w, n in enumerate(sizes.tolist()):
        groups.setdefault(n, []).append(w)
    for n, windows in groups.items():
        per_call = max(1, MAX_DISTANCE_BYTES // (2 * n * n * itemsize))
        for start in range(0, len(windows), per_call):
            chunk = windows[start:start + per_call]
            rows = torch.as_tensor(np.concatenate([np.arange(offsets[w], offsets[w + 1]) for w in chunk]),
                                   device=packed.device)
            x = packed[rows].reshape(len(chunk), n, packed.shape[1])
            labels = cluster(x, min_cluster_size, min_samples, epsilon, precision)
            out[rows] = labels.reshape(-1)
    return out
