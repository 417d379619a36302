// Common device definitions for the GB300 batched HDBSCAN kernels (sm_103a).
//
// Arithmetic contract (reference: hdbscan_gpu/_kernels.py:45-88 compiled with
// --fmad=false at hdbscan_gpu/_cuda.py:24): every distance is
//   total = 0; for k in 0..D-1: delta = x_i[k] - x_j[k]; total = total + delta*delta
//   d = sqrt(total)          (IEEE round-to-nearest at every step, no FMA)
// The _rn intrinsics below pin both rounding and the absence of contraction.
// Zero-padding coordinates is exact: (0-0)^2 = +0 and t + 0 = t for t >= +0.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "hdb_args.h"
#include "hdb_exact.h"

namespace hdb {


template <typename Real> struct RealTraits;

template <> struct RealTraits<float> {
    using Bits = uint32_t;
    static constexpr float kMax = 3.4028234663852886e+38F;
    __device__ __forceinline__ static float inf() { return __int_as_float(0x7f800000); }
    __device__ __forceinline__ static float sub(float a, float b) { return __fsub_rn(a, b); }
    __device__ __forceinline__ static float mul(float a, float b) { return __fmul_rn(a, b); }
    // Correctly rounded a*a of a difference of operand_safe values.
    __device__ __forceinline__ static float sqr(float a) { return __fmul_rn(a, a); }
    __device__ __forceinline__ static bool operand_safe(float) { return true; }
    __device__ __forceinline__ static float mul_ru(float a, float b) { return __fmul_ru(a, b); }
    __device__ __forceinline__ static float add(float a, float b) { return __fadd_rn(a, b); }
    __device__ __forceinline__ static float sqrt_rn(float a) { return __fsqrt_rn(a); }
    __device__ __forceinline__ static float recip(float a) { return __fdiv_rn(1.0f, a); }
    __device__ __forceinline__ static float div(float a, float b) { return __fdiv_rn(a, b); }
    __device__ __forceinline__ static float maxr(float a, float b) { return fmaxf(a, b); }
    // Order-preserving key for non-negative values; NaN and -0 are folded so
    // the key is total and below the "in tree" sentinel.
    __device__ __forceinline__ static Bits key(float a) { return __float_as_uint(a) & 0x7fffffffu; }
    __device__ __forceinline__ static float from_key(Bits k) { return __uint_as_float(k); }
};

template <> struct RealTraits<double> {
    using Bits = unsigned long long;
    static constexpr double kMax = 1.7976931348623157e+308;
    __device__ __forceinline__ static double inf() { return __longlong_as_double(0x7ff0000000000000ll); }
    __device__ __forceinline__ static double sub(double a, double b) { return __dsub_rn(a, b); }
    __device__ __forceinline__ static double mul(double a, double b) { return __dmul_rn(a, b); }
    // Correctly rounded a*a of a difference of operand_safe values, on the
    // integer pipes (hdb_exact.h): the FP64 pipe then carries only the
    // subtraction and the addition.
    __device__ __forceinline__ static double sqr(double a) { return sqr_rn_safe(a); }
    __device__ __forceinline__ static bool operand_safe(double x) { return sqr_operand_safe(x); }
    __device__ __forceinline__ static double mul_ru(double a, double b) { return __dmul_ru(a, b); }
    __device__ __forceinline__ static double add(double a, double b) { return __dadd_rn(a, b); }
    __device__ __forceinline__ static double sqrt_rn(double a) { return __dsqrt_rn(a); }
    __device__ __forceinline__ static double recip(double a) { return __ddiv_rn(1.0, a); }
    __device__ __forceinline__ static double div(double a, double b) { return __ddiv_rn(a, b); }
    __device__ __forceinline__ static double maxr(double a, double b) { return fmax(a, b); }
    __device__ __forceinline__ static Bits key(double a) {
        return (Bits)__double_as_longlong(a) & 0x7fffffffffffffffull;
    }
    __device__ __forceinline__ static double from_key(Bits k) { return __longlong_as_double((long long)k); }
};

// Warp-wide lexicographic minimum of (key, index) with redux.sync; the
// result is identical in every lane.  Index ties are impossible (indices are
// unique), so this is the reference's "(weight, then lowest global vertex)"
// argmin (_kernels.py:241-246, :255-259).
__device__ __forceinline__ void warp_argmin(uint32_t& key, uint32_t& idx) {
    const uint32_t k = __reduce_min_sync(0xffffffffu, key);
    idx = __reduce_min_sync(0xffffffffu, key == k ? idx : 0xffffffffu);
    key = k;
}

__device__ __forceinline__ void warp_argmin(unsigned long long& key, uint32_t& idx) {
    const uint32_t hi = __reduce_min_sync(0xffffffffu, (uint32_t)(key >> 32));
    const uint32_t lo = __reduce_min_sync(0xffffffffu, (uint32_t)(key >> 32) == hi ? (uint32_t)key : 0xffffffffu);
    const unsigned long long k = ((unsigned long long)hi << 32) | lo;
    idx = __reduce_min_sync(0xffffffffu, key == k ? idx : 0xffffffffu);
    key = k;
}

__device__ __forceinline__ void atomic_status(int32_t* status, int32_t code) {
    if (status && code) atomicOr(status, code);
}

}  // namespace hdb
