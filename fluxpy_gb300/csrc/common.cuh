// Shared helpers for the fluxgb CUDA library (sm_103a only).
//
// Every exported entry point returns an fgb_status code (include/fluxgb.h);
// the message of the last failure on the calling thread is kept in a
// thread-local buffer readable through fgb_last_error().
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <stdarg.h>

#include "../../include/fluxgb.h"

namespace fgb {

void set_error(const char* fmt, ...);

// Record a CUDA error (if any) and turn it into FGB_CUDA_ERR.
inline int cuda_status(cudaError_t e, const char* where) {
  if (e == cudaSuccess) return FGB_OK;
  set_error("%s: %s", where, cudaGetErrorString(e));
  return FGB_CUDA_ERR;
}

#define FGB_CUDA_TRY(expr)                                   \
  do {                                                       \
    cudaError_t _e = (expr);                                 \
    if (_e != cudaSuccess) return ::fgb::cuda_status(_e, #expr); \
  } while (0)

// Every kernel launch is followed by this check, which also counts the
// launch (fgb_launch_count()).
void count_launch();
#define FGB_LAUNCH_CHECK(name)                                \
  do {                                                        \
    ::fgb::count_launch();                                    \
    cudaError_t _e = cudaGetLastError();                      \
    if (_e != cudaSuccess) return ::fgb::cuda_status(_e, name); \
  } while (0)

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

constexpr int kNumSMs = 152;  // GB300: 2 dies x 76 SMs

inline unsigned grid_for(long long n, int block, long long cap = 152LL * 32) {
  long long g = (n + block - 1) / block;
  if (g < 1) g = 1;
  if (g > cap) g = cap;
  return (unsigned)g;
}

// Scratch allocation on the stream (stream-ordered allocator).
template <class T>
inline int scratch_alloc(T** p, size_t count, cudaStream_t s) {
  if (count == 0) count = 1;
  cudaError_t e = cudaMallocAsync((void**)p, count * sizeof(T), s);
  if (e != cudaSuccess) {
    set_error("cudaMallocAsync(%zu bytes): %s", count * sizeof(T), cudaGetErrorString(e));
    return FGB_NO_MEMORY;
  }
  return FGB_OK;
}
inline void scratch_free(void* p, cudaStream_t s) {
  if (p) cudaFreeAsync(p, s);
}

// Status flag bits that kernels OR into a device-side status word.
enum : unsigned {
  kFlagNonfiniteIn = 1u << 0,
  kFlagNegativeIn = 1u << 1,
  kFlagNonfiniteOut = 1u << 2,
  kFlagNegativeOut = 1u << 3,
  kFlagZeroPivot = 1u << 4,
  kFlagPredCorrMax = 1u << 5,
  kFlagStackOverflow = 1u << 6,
  kFlagIndexRange = 1u << 7,
  kFlagRankCap = 1u << 8,
  kFlagNoConverge = 1u << 10,
};

}  // namespace fgb
