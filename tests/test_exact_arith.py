"""The integer-pipe binary64 square and fused square-and-add
(hdbscan_gb300/csrc/hdb_exact.h) against the host's and the device's IEEE
multiply and add, bit for bit: random bit patterns over every exponent, the
exponent boundaries of the fast path, rounding carries and halfway cases,
zeros, subnormals, infinities and NaN (square); accumulators and differences
over the fused operation's whole domain, close exponents, exact and halfway
squares, zeros and k-ordered chains as the distance kernel runs them
(square-and-add)."""

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


FUSED_PROGRAM = r"""
#include <cstdio>
#include <cstdint>
#include <cstdlib>
#include <cmath>
#include <random>
#include "hdb_exact.h"
using namespace hdb;

static uint64_t count = 0, bad = 0;
static void check(double acc, double d) {
    volatile double va = acc, vd = d;
    volatile double sq = vd * vd;
    const double want = va + sq;  // host IEEE multiply, then add
    const double got = sqr_add_rn(acc, d);
    ++count;
    if (exact_bits(want) != exact_bits(got)) {
        if (bad < 10) std::printf("mismatch acc=%a d=%a want=%a got=%a\n", acc, d, want, got);
        ++bad;
    }
}

int main(int argc, char** argv) {
    const long n = argc > 1 ? std::atol(argv[1]) : 1000000;
    std::mt19937_64 rng(20261205);
    const unsigned long long frac = (1ull << 52) - 1;
    auto make = [&](unsigned long long e, unsigned long long f, bool neg) {
        return exact_double(((unsigned long long)neg << 63) | (e << 52) | (f & frac));
    };
    // The domain: d = 0 or |d| in [2^-511, 2^501] (biased exponents 512..1524),
    // acc = +0 or normal below 2^1008 (biased exponents 1..2030).
    auto any_d = [&]() { return make(512 + rng() % 1013, rng(), rng() & 1); };
    auto any_acc = [&]() { return make(1 + rng() % 2030, rng(), false); };
    for (long i = 0; i < n; ++i) check(any_acc(), any_d());
    for (long i = 0; i < 2 * n; ++i) {  // accumulator exponent within 65 of the square's
        const double d = any_d();
        const long long eq = 2 * (long long)((exact_bits(d) >> 52) & 0x7ff) - 1023;
        long long ea = eq + (long long)(rng() % 131) - 65;
        ea = ea < 1 ? 1 : (ea > 2030 ? 2030 : ea);
        unsigned long long f = rng();
        switch (rng() % 4) {
            case 1: f = frac; break;
            case 2: f &= 0xffffff; break;
            case 3: f = (f & ~0xffffffull) | (1ull << (rng() % 52)); break;
            default: break;
        }
        check(make((unsigned long long)ea, f, false), d);
    }
    for (long i = 0; i < n; ++i) {  // exact and halfway squares: short significands of d
        const unsigned long long e = 512 + rng() % 1013;
        unsigned long long f = (rng() & ((1ull << 27) - 1)) << 25;
        if (rng() & 1) f |= 1ull << (rng() % 25);
        const long long eq = 2 * (long long)e - 1023;
        long long ea = eq + (long long)(rng() % 121) - 60;
        ea = ea < 1 ? 1 : (ea > 2030 ? 2030 : ea);
        unsigned long long fa = rng();
        if (rng() & 1) fa &= ~((1ull << (rng() % 52)) - 1);
        check(make((unsigned long long)ea, fa, false), make(e, f, rng() & 1));
    }
    for (long i = 0; i < n / 10; ++i) {  // zeros
        check(0.0, any_d());
        check(any_acc(), 0.0);
        check(any_acc(), -0.0);
    }
    for (double d : {0.0, -0.0, 0x1p-511, -0x1p-511, 0x1p501, -0x1p501, 0x1.fffffffffffffp500, 0x1.0000000000001p-511})
        for (double a : {0.0, 0x1p-1022, 0x1.fffffffffffffp999, 0x1.fffffffffffffp1006, 1.0, 0x1.8p-1000}) check(a, d);
    // k-ordered chains of squared differences, as the distance kernel runs them.
    for (long i = 0; i < n / 20; ++i) {
        const int D = 1 + (int)(rng() % 128), scale = (int)(rng() % 200) - 100;
        std::normal_distribution<double> normal(0.0, 1.0);
        double acc = 0.0;
        volatile double want = 0.0;
        for (int k = 0; k < D; ++k) {
            const double xi = std::ldexp(normal(rng), scale);
            const double xj = (rng() % 16 == 0) ? xi : std::ldexp(normal(rng), scale);
            volatile double vi = xi, vj = xj;
            volatile double d = vi - vj;
            volatile double sq = d * d;
            want = want + sq;
            acc = sqr_add_rn(acc, d);
        }
        ++count;
        if (exact_bits(acc) != exact_bits((double)want)) {
            if (bad < 10) std::printf("chain mismatch D=%d\n", D);
            ++bad;
        }
    }
    std::printf("checked %llu mismatches %llu\n", (unsigned long long)count, (unsigned long long)bad);
    return bad != 0;
}
"""


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_fused_square_add_matches_ieee(tmp_path):
    src = tmp_path / "fused.cpp"
    src.write_text(FUSED_PROGRAM)
    exe = tmp_path / "fused"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math",
                    "-I", str(ROOT / "hdbscan_gb300" / "csrc"), str(src), "-o", str(exe)], check=True)
    result = subprocess.run([str(exe), "1000000"], capture_output=True, text=True)
    assert result.returncode == 0, result.stdout + result.stderr
    assert "mismatches 0" in result.stdout
    assert int(result.stdout.split("checked ")[1].split()[0]) > 4_000_000


DEVICE_FUSED_PROGRAM = r"""
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
    const double acc = __longlong_as_double((long long)in[2 * i]), d = __longlong_as_double((long long)in[2 * i + 1]);
    const double want = __dadd_rn(acc, __dmul_rn(d, d));
    const double got = sqr_add_rn(acc, d);
    if (__double_as_longlong(want) != __double_as_longlong(got)) {
        if (atomicAdd(bad, 1ull) == 0ull) *first = (unsigned long long)i;
    }
}

int main() {
    const long n = 1l << 23;
    std::vector<unsigned long long> host(2 * n);
    std::mt19937_64 rng(12);
    const unsigned long long frac = (1ull << 52) - 1;
    for (long i = 0; i < n; ++i) {
        const unsigned long long ed = 512 + rng() % 1013;
        unsigned long long d = ((rng() & 1) << 63) | (ed << 52) | (rng() & frac), a;
        if ((i & 3) == 3) d &= ~((1ull << (25 + rng() % 27)) - 1);  // short significands: exact and halfway squares
        if (i % 64 == 5) d = (rng() & 1) << 63;                      // zero difference
        long long ea;
        if (i & 1) {
            ea = 2 * (long long)ed - 1023 + (long long)(rng() % 131) - 65;  // close exponents
        } else {
            ea = 1 + (long long)(rng() % 2030);
        }
        ea = ea < 1 ? 1 : (ea > 2030 ? 2030 : ea);
        a = ((unsigned long long)ea << 52) | (rng() & frac);
        if (i % 64 == 9) a = 0;  // zero accumulator
        host[2 * i] = a;
        host[2 * i + 1] = d;
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
def test_device_fused_square_add_matches_hardware(cuda, tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    src = tmp_path / "fused_device.cu"
    src.write_text(DEVICE_FUSED_PROGRAM)
    exe = tmp_path / "fused_device"
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "--fmad=false", "-std=c++17",
                    "-I", str(ROOT / "hdbscan_gb300" / "csrc"), str(src), "-o", str(exe)], check=True)
    result = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert result.returncode == 0, result.stdout + result.stderr
    assert "mismatches 0" in result.stdout
