// Contraction-proof IEEE arithmetic helpers.
//
// The ray/triangle predicates, facet geometry and form-factor formula must
// give the same bits as the CPU oracle (plain C compiled with
// -ffp-contract=off) and as numpy.  These wrappers use the _rn intrinsics,
// which the compiler never fuses into FMAs, whatever -fmad says.
#pragma once
#include <cuda_runtime.h>

namespace fgb {

__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float fsqrt(float a) { return __fsqrt_rn(a); }

__device__ __forceinline__ double fmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double fadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double fsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double fdiv(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ double fsqrt(double a) { return __dsqrt_rn(a); }

// numpy: np.sum(a*b, axis=1) over 3 contiguous components -> ((a0b0+a1b1)+a2b2)
template <class R>
__device__ __forceinline__ R dot3(R a0, R a1, R a2, R b0, R b1, R b2) {
  return fadd(fadd(fmul(a0, b0), fmul(a1, b1)), fmul(a2, b2));
}

}  // namespace fgb
