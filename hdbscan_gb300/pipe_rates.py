"""Measured issue rates of the arithmetic pipes the distance kernels lean on.

`python -m hdbscan_gb300.pipe_rates` compiles a small CUDA program for sm_103a
(nvcc, into a temporary directory), runs it on cuda:0 and prints one JSON line:
operations per second for float64 add (the FP64 pipe), float32 add (the FMA
pipes) and 32-bit integer multiply-add.  (Chains of a single logic operation
are folded by the compiler, so the ALU pipe is read from the ncu pipe counters
in profiles/ instead.)
Each kernel runs 8 independent dependency chains of one inline-PTX instruction
per thread over every SM, timed with CUDA events after a warm-up; the count is
threads x chains x iterations.  These are the denominators quoted for the
float32 and float64 distance kernels; the ncu pipe utilisations in profiles/
measure the same pipes directly.
"""

from __future__ import annotations

import json
import shutil
import subprocess
import tempfile
from pathlib import Path

PROGRAM = r"""
#include <cstdio>
#include <cuda_runtime.h>

constexpr int kIters = 4096;

#define CHAINS(OP, TYPE, INIT)                                                   \
    TYPE v0 = INIT + 0, v1 = INIT + 1, v2 = INIT + 2, v3 = INIT + 3,           \
         v4 = INIT + 4, v5 = INIT + 5, v6 = INIT + 6, v7 = INIT + 7;           \
    for (int i = 0; i < kIters; ++i) {                                          \
        OP(v0); OP(v1); OP(v2); OP(v3); OP(v4); OP(v5); OP(v6); OP(v7);         \
    }                                                                           \
    out[blockIdx.x * blockDim.x + threadIdx.x] = v0 + v1 + v2 + v3 + v4 + v5 + v6 + v7;

#define DADD(v) asm volatile("add.rn.f64 %0, %0, %1;" : "+d"(v) : "d"(s))
#define FADD(v) asm volatile("add.rn.f32 %0, %0, %1;" : "+f"(v) : "f"(s))
#define IMAD(v) asm volatile("mad.lo.u32 %0, %0, %1, %2;" : "+r"(v) : "r"(m), "r"(s))

__global__ void dadd(double* out, double s) { CHAINS(DADD, double, s) }
__global__ void fadd(float* out, float s) { CHAINS(FADD, float, s) }
__global__ void imad(unsigned* out, unsigned m, unsigned s) { CHAINS(IMAD, unsigned, s) }

template <typename F>
double rate(F launch, int blocks, int threads) {
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    launch();
    cudaDeviceSynchronize();
    float best = 1e30f;
    for (int r = 0; r < 5; ++r) {
        cudaEventRecord(a);
        launch();
        cudaEventRecord(b);
        cudaEventSynchronize(b);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        if (ms < best) best = ms;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return (double)blocks * threads * 8.0 * kIters / (best * 1e-3);
}

int main() {
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
    const int threads = 512, blocks = sms * 4;
    void* out = nullptr;
    cudaMalloc(&out, (size_t)blocks * threads * sizeof(double));
    const double r_dadd = rate([&] { dadd<<<blocks, threads>>>((double*)out, 1e-9); }, blocks, threads);
    const double r_fadd = rate([&] { fadd<<<blocks, threads>>>((float*)out, 1e-9f); }, blocks, threads);
    const double r_imad = rate([&] { imad<<<blocks, threads>>>((unsigned*)out, 3u, 7u); }, blocks, threads);
    const cudaError_t e = cudaGetLastError();
    cudaFree(out);
    printf("{\"sms\": %d, \"dadd_per_s\": %.4g, \"fadd_per_s\": %.4g, \"imad_per_s\": %.4g, \"error\": \"%s\"}\n",
           sms, r_dadd, r_fadd, r_imad, cudaGetErrorString(e));
    return e == cudaSuccess ? 0 : 1;
}
"""


def measure() -> dict:
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    with tempfile.TemporaryDirectory() as tmp:
        src = Path(tmp) / "pipe_rates.cu"
        exe = Path(tmp) / "pipe_rates"
        src.write_text(PROGRAM)
        subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", str(src), "-o",
                        str(exe)], check=True)
        result = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
        if result.returncode:
            raise RuntimeError(result.stdout + result.stderr)
        return json.loads(result.stdout.strip().splitlines()[-1])


if __name__ == "__main__":
    print(json.dumps(measure()))
