// Producer stage: encoder embeddings in bfloat16 / float16 (or the compute
// type) to the compute type, optionally L2-normalised per point, in one pass.
//
// No reference counterpart: the reference takes float32/float64 input only
// (hdbscan_gpu/_cuda.py:95-97 casts on the host side of CuPy).  Conversion
// from bfloat16/float16 to float32 is exact.  Normalisation is defined
// exactly: s = 0; for k in 0..D-1: s = s + x_k*x_k (round-to-nearest, no
// FMA); r = sqrt_rn(s); x_k' = x_k / r (round-to-nearest); a zero vector is
// left as it is (as scikit-learn's normalize does).  One thread per point; the
// result goes to the workspace and every later stage reads it, so the
// normalisation is computed once per point rather than once per distance tile.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "hdb_common.cuh"

namespace hdb {

enum InputType : int { kInputCompute = 0, kInputBF16 = 1, kInputF16 = 2 };

template <typename Real, typename In>
__device__ __forceinline__ Real to_compute(In v) {
    if constexpr (std::is_same<In, __nv_bfloat16>::value) return (Real)__bfloat162float(v);
    else if constexpr (std::is_same<In, __half>::value) return (Real)__half2float(v);
    else return (Real)v;
}

template <typename Real, typename In>
__global__ void __launch_bounds__(256) hdb_prepare_kernel(const In* __restrict__ X, Real* __restrict__ out,
                                                          int64_t points, int D, int normalize) {
    using T = RealTraits<Real>;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= points) return;
    const In* x = X + i * D;
    Real* y = out + i * D;
    if (!normalize) {
        for (int k = 0; k < D; ++k) y[k] = to_compute<Real>(x[k]);
        return;
    }
    Real s = Real(0);
    for (int k = 0; k < D; ++k) {
        const Real v = to_compute<Real>(x[k]);
        s = T::add(s, T::mul(v, v));
    }
    const Real r = T::sqrt_rn(s);
    for (int k = 0; k < D; ++k) {
        const Real v = to_compute<Real>(x[k]);
        y[k] = r > Real(0) ? T::div(v, r) : v;
    }
}

}  // namespace hdb
