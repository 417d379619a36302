"""The integer-pipe binary64 square and addition (hdbscan_gb300/csrc/hdb_exact.h)
against the host's IEEE multiply and add, bit for bit: random bit patterns
over every exponent, the exponent boundaries of the fast path, rounding
carries and halfway cases, zeros, subnormals, infinities and NaN (square);
non-negative operands of every class and exponent gap, carries, halfway cases
and overflow (addition)."""

import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]

PROGRAM = r"""
#include <cstdio>
#include <cstdint>
#include <cstdlib>
#include <cmath>
#include <random>
#include "hdb_exact.h"
using namespace hdb;

static uint64_t count = 0, bad = 0;
static void check(double d) {
    volatile double vd = d;
    const double want = vd * vd;                      // host IEEE multiply
    const double got = sqr_rn(d);
    ++count;
    const uint64_t a = exact_bits(want), b = exact_bits(got);
    const bool both_nan = std::isnan(want) && std::isnan(got);
    if (a != b && !both_nan) {
        if (bad < 10) std::printf("mismatch d=%a want=%a got=%a\n", d, want, got);
        ++bad;
    }
}

int main(int argc, char** argv) {
    const long n = argc > 1 ? std::atol(argv[1]) : 1000000;
    std::mt19937_64 rng(20261203);
    for (long i = 0; i < n; ++i) check(exact_double(rng()));                       // any pattern
    for (long i = 0; i < n; ++i) {                                                  // fast-path exponents
        const uint64_t e = 500 + rng() % 1050, f = rng() & ((1ull << 52) - 1);
        check(exact_double((e << 52) | f | ((rng() & 1) << 63)));
    }
    for (uint64_t e : {0ull, 1ull, 510ull, 511ull, 512ull, 513ull, 1022ull, 1023ull, 1024ull, 1532ull, 1533ull,
                       1534ull, 1535ull, 2046ull, 2047ull})
        for (uint64_t f : {0ull, 1ull, 2ull, (1ull << 52) - 1, (1ull << 52) - 2, 1ull << 51, (1ull << 51) + 1,
                           0x6a09e667f3bcdull, 0x6a09e667f3bccull, 0x6a09e667f3bceull})
            for (uint64_t s : {0ull, 1ull}) check(exact_double((s << 63) | (e << 52) | f));
    // Significands whose square is within a few ulps of a rounding boundary.
    for (long i = 0; i < n / 4; ++i) {
        const double x = std::sqrt(1.0 + (double)(rng() % (1ull << 40)) * 0x1p-40);
        const uint64_t b = exact_bits(x);
        for (int k = -2; k <= 2; ++k) check(exact_double(b + k));
    }
    check(0.0); check(-0.0); check(INFINITY); check(-INFINITY); check(NAN);
    check(0x1p-1074); check(0x1p-1022); check(0x1.fffffffffffffp+1023); check(0x1p+511); check(0x1p-511);
    // Differences of operands accepted by sqr_operand_safe square exactly without the fallback.
    auto safe_value = [&]() -> double {
        const uint64_t r = rng();
        if ((r & 15) == 0) return 0.0;
        const uint64_t e = (1023 - 459) + rng() % (459 + 509);
        return exact_double(((r >> 63) << 63) | (e << 52) | (rng() & ((1ull << 52) - 1)));
    };
    for (long i = 0; i < n; ++i) {
        const double a = safe_value();
        double b = (i & 1) ? safe_value() : exact_double(exact_bits(a) + (rng() % 5) - 2);  // near-equal pairs
        if (!sqr_operand_safe(b)) b = a;
        if (!sqr_operand_safe(a)) { ++bad; continue; }
        volatile double va = a, vb = b;
        const double d = va - vb;
        volatile double vd = d;
        const double want = vd * vd, got = sqr_rn_safe(d);
        ++count;
        if (exact_bits(want) != exact_bits(got)) {
            if (bad < 10) std::printf("safe mismatch a=%a b=%a want=%a got=%a\n", a, b, want, got);
            ++bad;
        }
    }
    for (double a : {0x1p-459, -0x1p-459, 0x1.fffffffffffffp+508, -0x1.fffffffffffffp+508})
        for (double b : {0.0, 0x1p-459, -0x1p-459, 0x1.0000000000001p-459, 0x1.fffffffffffffp+508,
                         -0x1.fffffffffffffp+508}) {
            volatile double va = a, vb = b;
            const double d = va - vb;
            volatile double vd = d;
            ++count;
            if (exact_bits(vd * vd) != exact_bits(sqr_rn_safe(d))) ++bad;
        }
    std::printf("checked %llu mismatches %llu\n", (unsigned long long)count, (unsigned long long)bad);
    return bad != 0;
}
"""


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_integer_square_matches_ieee_multiply(tmp_path):
    src = tmp_path / "sqr.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "sqr"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math",
                    "-I", str(ROOT / "hdbscan_gb300" / "csrc"), str(src), "-o", str(exe)], check=True)
    result = subprocess.run([str(exe), "2000000"], capture_output=True, text=True)
    assert result.returncode == 0, result.stdout + result.stderr
    assert "mismatches 0" in result.stdout
    assert int(result.stdout.split("checked ")[1].split()[0]) > 5_000_000


DEVICE_PROGRAM = r"""
#include <cstdio>
#include <cstdint>
#include <random>
#include <vector>
#include <cuda_runtime.h>
#include "hdb_exact.h"
using namespace hdb;

__global__ void compare(const unsigned long long* in, unsigned long long* bad, unsigned long long* first, long n) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    // Every lane of every warp stays active (n is a multiple of the block size).
    const double d = __longlong_as_double((long long)in[i]);
    const double want = __dmul_rn(d, d);
    const double got = sqr_rn(d);
    const bool nan_both = want != want && got != got;
    if (__double_as_longlong(want) != __double_as_longlong(got) && !nan_both) {
        if (atomicAdd(bad, 1ull) == 0ull) *first = in[i];
    }
}

int main() {
    const long n = 1l << 24;  // multiple of 256
    std::vector<unsigned long long> host(n);
    std::mt19937_64 rng(7);
    for (long i = 0; i < n; ++i) {
        switch (i & 3) {
            case 0: host[i] = rng(); break;                                                       // any pattern
            case 1: host[i] = ((500 + rng() % 1050) << 52) | (rng() & ((1ull << 52) - 1)); break;  // fast path
            case 2: host[i] = (1023ull << 52) | (rng() & ((1ull << 52) - 1)); break;               // [1, 2)
            default: host[i] = (rng() & 1) ? 0ull : (rng() & ((1ull << 52) - 1)); break;          // zero, subnormal
        }
    }
    unsigned long long *d_in, *d_bad, *d_first;
    cudaMalloc(&d_in, n * sizeof(unsigned long long));
    cudaMalloc(&d_bad, sizeof(unsigned long long));
    cudaMalloc(&d_first, sizeof(unsigned long long));
    cudaMemcpy(d_in, host.data(), n * sizeof(unsigned long long), cudaMemcpyHostToDevice);
    cudaMemset(d_bad, 0, sizeof(unsigned long long));
    cudaMemset(d_first, 0, sizeof(unsigned long long));
    compare<<<n / 256, 256>>>(d_in, d_bad, d_first, n);
    unsigned long long bad = 0, first = 0;
    cudaMemcpy(&bad, d_bad, sizeof(bad), cudaMemcpyDeviceToHost);
    cudaMemcpy(&first, d_first, sizeof(first), cudaMemcpyDeviceToHost);
    const cudaError_t e = cudaGetLastError();
    std::printf("checked %ld mismatches %llu first %llx (%s)\n", n, bad, first, cudaGetErrorString(e));
    cudaFree(d_in); cudaFree(d_bad); cudaFree(d_first);
    return (bad != 0 || e != cudaSuccess) ? 1 : 0;
}
"""


@pytest.mark.gpu
def test_device_integer_square_matches_dmul(cuda, tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    src = tmp_path / "sqr_device.cu"
    src.write_text(DEVICE_PROGRAM)
    exe = tmp_path / "sqr_device"
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "--fmad=false", "-std=c++17",
                    "-I", str(ROOT / "hdbscan_gb300" / "csrc"), str(src), "-o", str(exe)], check=True)
    result = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert result.returncode == 0, result.stdout + result.stderr
    assert "mismatches 0" in result.stdout


ADD_PROGRAM = r"""
#include <cstdio>
#include <cstdint>
#include <cstdlib>
#include <cmath>
#include <random>
#include "hdb_exact.h"
using namespace hdb;

static uint64_t count = 0, bad = 0;
static void check(double a, double b) {
    volatile double va = a, vb = b;
    const double want = va + vb;  // host IEEE add
    const double got = add_rn_nonneg(a, b);
    ++count;
    if (exact_bits(want) != exact_bits(got)) {
        if (bad < 10) std::printf("mismatch a=%a b=%a want=%a got=%a\n", a, b, want, got);
        ++bad;
    }
}

int main(int argc, char** argv) {
    const long n = argc > 1 ? std::atol(argv[1]) : 1000000;
    std::mt19937_64 rng(20261204);
    const unsigned long long frac = (1ull << 52) - 1;
    auto with_exp = [&](unsigned long long e) { return exact_double((e << 52) | (rng() & frac)); };
    for (long i = 0; i < n; ++i) check(with_exp(1 + rng() % 2046), with_exp(1 + rng() % 2046));  // any gap
    for (long i = 0; i < n; ++i) {                                                                 // close exponents
        const unsigned long long e = 1 + rng() % 2040;
        const long long f = (long long)e - (long long)(rng() % 60);
        const double a = with_exp(e), b = with_exp(f < 1 ? 1ull : (unsigned long long)f);
        check(a, b);
        check(b, a);
    }
    for (long i = 0; i < n; ++i) {  // any non-negative non-NaN pattern, subnormals included
        const double a = exact_double(rng() >> 1), b = exact_double((rng() >> 1) & ((i & 1) ? ~0ull : ((1ull << 56) - 1)));
        if (std::isnan(a) || std::isnan(b)) continue;
        check(a, b);
    }
    for (long i = 0; i < n / 4; ++i) check(with_exp(2000 + rng() % 47), with_exp(1995 + rng() % 52));  // overflow
    // Halfway and carry patterns at every exponent gap.
    for (unsigned long long e = 60; e < 2040; e += 37)
        for (unsigned long long d = 0; d < 60; ++d)
            for (unsigned long long fa : {0ull, 1ull, 2ull, 3ull, frac, 1ull << 51})
                for (unsigned long long fb : {0ull, 1ull, frac, 1ull << 51, (1ull << 51) + 1, 1ull << 50}) {
                    const double a = exact_double((e << 52) | fa), b = exact_double(((e - d) << 52) | fb);
                    check(a, b);
                    check(b, a);
                }
    for (double a : {0.0, 0x1p-1074, 0x1p-1022, 1.0, (double)INFINITY, 0x1.fffffffffffffp+1023})
        for (double b : {0.0, 0x1p-1074, 0x1p-1022, 1.0, 0x1p+1023, 0x1.fffffffffffffp+1022, (double)INFINITY}) {
            check(a, b);
            check(b, a);
        }
    std::printf("checked %llu mismatches %llu\n", (unsigned long long)count, (unsigned long long)bad);
    return bad != 0;
}
"""


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_integer_add_matches_ieee_add(tmp_path):
    src = tmp_path / "add.cpp"
    src.write_text(ADD_PROGRAM)
    exe = tmp_path / "add"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math",
                    "-I", str(ROOT / "hdbscan_gb300" / "csrc"), str(src), "-o", str(exe)], check=True)
    result = subprocess.run([str(exe), "1000000"], capture_output=True, text=True)
    assert result.returncode == 0, result.stdout + result.stderr
    assert "mismatches 0" in result.stdout
    assert int(result.stdout.split("checked ")[1].split()[0]) > 4_000_000


DEVICE_ADD_PROGRAM = r"""
#include <cstdio>
#include <cstdint>
#include <random>
#include <vector>
#include <cuda_runtime.h>
#include "hdb_exact.h"
using namespace hdb;

__global__ void compare(const unsigned long long* in, unsigned long long* bad, unsigned long long* first, long n) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double a = __longlong_as_double((long long)in[2 * i]), b = __longlong_as_double((long long)in[2 * i + 1]);
    const double want = __dadd_rn(a, b);
    const double got = add_rn_nonneg(a, b);
    if (__double_as_longlong(want) != __double_as_longlong(got)) {
        if (atomicAdd(bad, 1ull) == 0ull) *first = (unsigned long long)i;
    }
}

int main() {
    const long n = 1l << 23;
    std::vector<unsigned long long> host(2 * n);
    std::mt19937_64 rng(11);
    const unsigned long long frac = (1ull << 52) - 1;
    for (long i = 0; i < n; ++i) {
        unsigned long long a, b;
        switch (i & 3) {
            case 0: a = rng() >> 1; b = rng() >> 1; break;                                     // any non-negative
            case 1: a = ((1 + rng() % 2046) << 52) | (rng() & frac); b = ((1 + rng() % 2046) << 52) | (rng() & frac); break;
            case 2: { const unsigned long long e = 60 + rng() % 1980; a = (e << 52) | (rng() & frac);
                      b = ((e - rng() % 58) << 52) | (rng() & frac); break; }                       // close exponents
            default: a = (rng() & 1) ? 0ull : (rng() & frac); b = rng() & frac; break;             // zero, subnormal
        }
        if (((a >> 52) & 0x7ff) == 0x7ff && (a & frac)) a = 0;  // no NaN operands
        if (((b >> 52) & 0x7ff) == 0x7ff && (b & frac)) b = 0;
        host[2 * i] = a;
        host[2 * i + 1] = b;
    }
    unsigned long long *d_in, *d_bad, *d_first;
    cudaMalloc(&d_in, 2 * n * sizeof(unsigned long long));
    cudaMalloc(&d_bad, sizeof(unsigned long long));
    cudaMalloc(&d_first, sizeof(unsigned long long));
    cudaMemcpy(d_in, host.data(), 2 * n * sizeof(unsigned long long), cudaMemcpyHostToDevice);
    cudaMemset(d_bad, 0, sizeof(unsigned long long));
    cudaMemset(d_first, 0, sizeof(unsigned long long));
    compare<<<(n + 255) / 256, 256>>>(d_in, d_bad, d_first, n);
    unsigned long long bad = 0, first = 0;
    cudaMemcpy(&bad, d_bad, sizeof(bad), cudaMemcpyDeviceToHost);
    cudaMemcpy(&first, d_first, sizeof(first), cudaMemcpyDeviceToHost);
    const cudaError_t e = cudaGetLastError();
    std::printf("checked %ld mismatches %llu first %llu (%s)\n", n, bad, first, cudaGetErrorString(e));
    cudaFree(d_in); cudaFree(d_bad); cudaFree(d_first);
    return (bad != 0 || e != cudaSuccess) ? 1 : 0;
}
"""


@pytest.mark.gpu
def test_device_integer_add_matches_dadd(cuda, tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    src = tmp_path / "add_device.cu"
    src.write_text(DEVICE_ADD_PROGRAM)
    exe = tmp_path / "add_device"
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "--fmad=false", "-std=c++17",
                    "-I", str(ROOT / "hdbscan_gb300" / "csrc"), str(src), "-o", str(exe)], check=True)
    result = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert result.returncode == 0, result.stdout + result.stderr
    assert "mismatches 0" in result.stdout
