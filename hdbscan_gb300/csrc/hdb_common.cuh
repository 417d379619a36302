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


// Comparisons, maxima and selections of NON-NEGATIVE values (distances,
// cores, weights, lambdas) go through lt / vmax / sel / finite_nn.  For
// float they are the plain operations.  For double they work on the two
// 32-bit words of the bit pattern: the patterns of non-negative doubles order
// like the values (the sign bit is masked, folding -0 onto +0), and GB300
// issues double compares, double selects and 64-bit integer compares to its
// FP64 pipe, a small fraction of the integer pipes' rate.
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
    __device__ __forceinline__ static bool lt(float a, float b) { return a < b; }
    __device__ __forceinline__ static float vmax(float a, float b) { return fmaxf(a, b); }
    __device__ __forceinline__ static float sel(bool c, float a, float b) { return c ? a : b; }
    __device__ __forceinline__ static bool finite_nn(float a) { return a <= kMax; }
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
    // subtraction and the addition.  operand_safe is the domain of the fused
    // integer square-and-add (sqr_add_rn), a subset of sqr_rn_safe's.
    __device__ __forceinline__ static double sqr(double a) { return sqr_rn_safe(a); }
    __device__ __forceinline__ static bool operand_safe(double x) { return sqr_add_operand_safe(x); }
    __device__ __forceinline__ static double mul_ru(double a, double b) { return __dmul_ru(a, b); }
    __device__ __forceinline__ static double add(double a, double b) { return __dadd_rn(a, b); }
    __device__ __forceinline__ static double sqrt_rn(double a) { return __dsqrt_rn(a); }
    __device__ __forceinline__ static double recip(double a) { return __ddiv_rn(1.0, a); }
    __device__ __forceinline__ static double div(double a, double b) { return __ddiv_rn(a, b); }
    __device__ __forceinline__ static double maxr(double a, double b) { return fmax(a, b); }
    __device__ __forceinline__ static bool lt(double a, double b) {
        const uint32_t ah = (uint32_t)__double2hiint(a) & 0x7fffffffu, bh = (uint32_t)__double2hiint(b) & 0x7fffffffu;
        const uint32_t al = (uint32_t)__double2loint(a), bl = (uint32_t)__double2loint(b);
        return ah < bh || (ah == bh && al < bl);
    }
    __device__ __forceinline__ static double sel(bool c, double a, double b) {
        return __hiloint2double(c ? __double2hiint(a) : __double2hiint(b), c ? __double2loint(a) : __double2loint(b));
    }
    __device__ __forceinline__ static double vmax(double a, double b) { return sel(lt(a, b), b, a); }
    // a <= DBL_MAX for a >= 0: not infinite and not NaN.
    __device__ __forceinline__ static bool finite_nn(double a) {
        return ((uint32_t)__double2hiint(a) & 0x7ff00000u) != 0x7ff00000u;
    }
    __device__ __forceinline__ static Bits key(double a) {
        return (Bits)__double_as_longlong(a) & 0x7fffffffffffffffull;
    }
    __device__ __forceinline__ static double from_key(Bits k) { return __longlong_as_double((long long)k); }
};

// (key, index) lexicographic order and key equality; 64-bit keys compare
// their 32-bit words.
__device__ __forceinline__ bool key_eq(uint32_t a, uint32_t b) { return a == b; }
__device__ __forceinline__ bool key_eq(unsigned long long a, unsigned long long b) {
    return (((uint32_t)a ^ (uint32_t)b) | ((uint32_t)(a >> 32) ^ (uint32_t)(b >> 32))) == 0u;
}
__device__ __forceinline__ bool key_lt(uint32_t a, uint32_t b) { return a < b; }
__device__ __forceinline__ bool key_lt(unsigned long long a, unsigned long long b) {
    const uint32_t ah = (uint32_t)(a >> 32), bh = (uint32_t)(b >> 32);
    return ah < bh || (ah == bh && (uint32_t)a < (uint32_t)b);
}
template <typename Key>
__device__ __forceinline__ bool key_idx_lt(Key k, uint32_t i, Key lk, uint32_t li) {
    return key_lt(k, lk) || (key_eq(k, lk) && i < li);
}

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
    const bool mine = (uint32_t)(key >> 32) == hi && (uint32_t)key == lo;
    idx = __reduce_min_sync(0xffffffffu, mine ? idx : 0xffffffffu);
    key = ((unsigned long long)hi << 32) | lo;
}

__device__ __forceinline__ void atomic_status(int32_t* status, int32_t code) {
    if (status && code) atomicOr(status, code);
}

}  // namespace hdb
