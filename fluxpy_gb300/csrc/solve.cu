// Element-wise kernels of the radiosity solve (src/flux/solve.py:4-45) and of
// the iterative refinement around it.  All operate on N x K row-major FP32
// blocks in cluster order; rho is per facet (length N) or a scalar when the
// pointer is NULL.
//   Jacobi, right placement (solve.py:36-45):  B1 = E + F (rho B); stop when
//     max |B1 - B| <= tol per column (the reference uses one global max).
//   refinement residual: R = E - (B - F (rho B)).
// Column maxima are accumulated with atomicMax on the IEEE bits of
// non-negative floats (order-preserving as unsigned integers).
#include "common.cuh"

#include <cuda_bf16.h>

namespace fgb {
namespace {

__device__ __forceinline__ float rho_at(const float* rho, float rho_s, long long i) {
  return rho ? rho[i] : rho_s;
}

template <class TO>
__device__ __forceinline__ TO cvt(float v);
template <> __device__ __forceinline__ float cvt<float>(float v) { return v; }
template <> __device__ __forceinline__ __nv_bfloat16 cvt<__nv_bfloat16>(float v) { return __float2bfloat16(v); }

// X = rho .* B  (optionally in bf16)
template <class TO>
__global__ void scale_rows_kernel(const float* __restrict__ B, const float* __restrict__ rho,
                                  float rho_s, TO* __restrict__ X, long long N, int K) {
  const long long total = N * K;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x) {
    long long i = q / K;
    X[q] = cvt<TO>(rho_at(rho, rho_s, i) * B[q]);
  }
}

// colmax[c] = max_i |Y - B|, then B = Y (when swap == 0 the caller swaps)
__global__ void colmax_absdiff_kernel(const float* __restrict__ Y, const float* __restrict__ B,
                                      long long N, int K, unsigned* __restrict__ colmax) {
  // one CTA handles a slab of rows for up to blockDim.x columns
  extern __shared__ unsigned s_max[];
  for (int c = threadIdx.x; c < K; c += blockDim.x) s_max[c] = 0u;
  __syncthreads();
  for (long long i = blockIdx.x; i < N; i += gridDim.x) {
    for (int c = threadIdx.x; c < K; c += blockDim.x) {
      float d = fabsf(B ? Y[i * K + c] - B[i * K + c] : Y[i * K + c]);
      if (d != d) d = INFINITY;  // NaN never converges
      unsigned u = __float_as_uint(d);
      if (u > s_max[c]) s_max[c] = u;
    }
  }
  __syncthreads();
  for (int c = threadIdx.x; c < K; c += blockDim.x) atomicMax(&colmax[c], s_max[c]);
}

// R = E - B + Y  (Y = F (rho B)); colmax[c] = max_i |R|
__global__ void residual_kernel(const float* __restrict__ Y, const float* __restrict__ B,
                                const float* __restrict__ E, float* __restrict__ R, long long N,
                                int K, unsigned* __restrict__ colmax) {
  extern __shared__ unsigned s_max[];
  for (int c = threadIdx.x; c < K; c += blockDim.x) s_max[c] = 0u;
  __syncthreads();
  for (long long i = blockIdx.x; i < N; i += gridDim.x) {
    for (int c = threadIdx.x; c < K; c += blockDim.x) {
      long long q = i * K + c;
      float r = (E[q] - B[q]) + Y[q];
      R[q] = r;
      float a = fabsf(r);
      if (a != a) a = INFINITY;
      unsigned u = __float_as_uint(a);
      if (u > s_max[c]) s_max[c] = u;
    }
  }
  __syncthreads();
  for (int c = threadIdx.x; c < K; c += blockDim.x) atomicMax(&colmax[c], s_max[c]);
}

// B += D on the columns whose mask entry is nonzero (all when mask == NULL)
__global__ void axpy_cols_kernel(float* __restrict__ B, const float* __restrict__ D,
                                 const unsigned char* __restrict__ mask, long long N, int K) {
  const long long total = N * K;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x) {
    int c = (int)(q % K);
    if (!mask || mask[c]) B[q] += D[q];
  }
}

// out[i, :] = in[idx[i], :]  (row gather; permute / unpermute)
template <class T>
__global__ void gather_rows_kernel(const T* __restrict__ in, const long long* __restrict__ idx,
                                   T* __restrict__ out, long long N, int K) {
  const long long total = N * K;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x) {
    long long i = q / K;
    int c = (int)(q % K);
    out[q] = in[idx[i] * K + c];
  }
}

int col_grid(long long N) { return (int)min(N, 152LL * 8); }

// Y[i, :] = add[i, :] + alpha * sum_q data[q] X[indices[q], :] for q in row i
// (one warp per row; lanes over the K columns).  Used for scipy CSR
// operators handed to the solver (the uncompressed matrix of
// get_form_factor_matrix).
template <class T>
__global__ void csr_spmm_kernel(const long long* __restrict__ indptr, const int* __restrict__ indices,
                                const T* __restrict__ data, long long m, const T* __restrict__ X,
                                int K, T* __restrict__ Y, const T* __restrict__ add, T alpha) {
  const int lane = threadIdx.x & 31;
  const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long i = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5; i < m; i += warps) {
    const long long a = indptr[i], b = indptr[i + 1];
    for (int c0 = 0; c0 < K; c0 += 32) {
      const int c = c0 + lane;
      T acc = T(0);
      if (c < K)
        for (long long q = a; q < b; q++) acc += data[q] * X[(long long)indices[q] * K + c];
      if (c < K) Y[i * K + c] = add ? add[i * K + c] + alpha * acc : alpha * acc;
    }
  }
}

}  // namespace
}  // namespace fgb

extern "C" {

int fgb_scale_rows_f32(const float* B, const float* rho, float rho_scalar, float* X, long long N,
                       int K, void* stream) {
  if (N < 0 || K < 1) { fgb::set_error("bad sizes"); return FGB_BAD_ARG; }
  if (N == 0) return FGB_OK;
  fgb::scale_rows_kernel<float><<<fgb::grid_for(N * K, 256), 256, 0, fgb::as_stream(stream)>>>(
      B, rho, rho_scalar, X, N, K);
  FGB_LAUNCH_CHECK("scale_rows_kernel");
  return FGB_OK;
}

int fgb_scale_rows_bf16(const float* B, const float* rho, float rho_scalar, void* X, long long N,
                        int K, void* stream) {
  if (N < 0 || K < 1) { fgb::set_error("bad sizes"); return FGB_BAD_ARG; }
  if (N == 0) return FGB_OK;
  fgb::scale_rows_kernel<__nv_bfloat16><<<fgb::grid_for(N * K, 256), 256, 0, fgb::as_stream(stream)>>>(
      B, rho, rho_scalar, static_cast<__nv_bfloat16*>(X), N, K);
  FGB_LAUNCH_CHECK("scale_rows_kernel");
  return FGB_OK;
}

int fgb_colmax_absdiff(const float* Y, const float* B, long long N, int K, unsigned* colmax,
                       void* stream) {
  if (N < 0 || K < 1 || K > 8192) { fgb::set_error("bad sizes (K <= 8192)"); return FGB_BAD_ARG; }
  if (N == 0) return FGB_OK;
  int threads = K < 256 ? ((K + 31) / 32) * 32 : 256;
  fgb::colmax_absdiff_kernel<<<fgb::col_grid(N), threads, sizeof(unsigned) * K,
                               fgb::as_stream(stream)>>>(Y, B, N, K, colmax);
  FGB_LAUNCH_CHECK("colmax_absdiff_kernel");
  return FGB_OK;
}

int fgb_residual(const float* Y, const float* B, const float* E, float* R, long long N, int K,
                 unsigned* colmax, void* stream) {
  if (N < 0 || K < 1 || K > 8192) { fgb::set_error("bad sizes (K <= 8192)"); return FGB_BAD_ARG; }
  if (N == 0) return FGB_OK;
  int threads = K < 256 ? ((K + 31) / 32) * 32 : 256;
  fgb::residual_kernel<<<fgb::col_grid(N), threads, sizeof(unsigned) * K, fgb::as_stream(stream)>>>(
      Y, B, E, R, N, K, colmax);
  FGB_LAUNCH_CHECK("residual_kernel");
  return FGB_OK;
}

int fgb_axpy_cols(float* B, const float* D, const unsigned char* mask, long long N, int K,
                  void* stream) {
  if (N < 0 || K < 1) { fgb::set_error("bad sizes"); return FGB_BAD_ARG; }
  if (N == 0) return FGB_OK;
  fgb::axpy_cols_kernel<<<fgb::grid_for(N * K, 256), 256, 0, fgb::as_stream(stream)>>>(B, D, mask, N, K);
  FGB_LAUNCH_CHECK("axpy_cols_kernel");
  return FGB_OK;
}

int fgb_gather_rows_f32(const float* in, const long long* idx, float* out, long long N, int K,
                        void* stream) {
  if (N < 0 || K < 1) { fgb::set_error("bad sizes"); return FGB_BAD_ARG; }
  if (N == 0) return FGB_OK;
  fgb::gather_rows_kernel<float><<<fgb::grid_for(N * K, 256), 256, 0, fgb::as_stream(stream)>>>(
      in, idx, out, N, K);
  FGB_LAUNCH_CHECK("gather_rows_kernel");
  return FGB_OK;
}

int fgb_gather_rows_f64(const double* in, const long long* idx, double* out, long long N, int K,
                        void* stream) {
  if (N < 0 || K < 1) { fgb::set_error("bad sizes"); return FGB_BAD_ARG; }
  if (N == 0) return FGB_OK;
  fgb::gather_rows_kernel<double><<<fgb::grid_for(N * K, 256), 256, 0, fgb::as_stream(stream)>>>(
      in, idx, out, N, K);
  FGB_LAUNCH_CHECK("gather_rows_kernel");
  return FGB_OK;
}

int fgb_csr_spmm_f64(const long long* indptr, const int* indices, const double* data, long long m,
                     const double* X, int K, double* Y, const double* add, double alpha,
                     void* stream) {
  if (m < 0 || K < 1) { fgb::set_error("bad sizes"); return FGB_BAD_ARG; }
  if (m == 0) return FGB_OK;
  fgb::csr_spmm_kernel<double><<<fgb::grid_for(m * 32, 256, 152LL * 64), 256, 0, fgb::as_stream(stream)>>>(
      indptr, indices, data, m, X, K, Y, add, alpha);
  FGB_LAUNCH_CHECK("csr_spmm_kernel");
  return FGB_OK;
}

int fgb_csr_spmm_f32(const long long* indptr, const int* indices, const float* data, long long m,
                     const float* X, int K, float* Y, const float* add, float alpha, void* stream) {
  if (m < 0 || K < 1) { fgb::set_error("bad sizes"); return FGB_BAD_ARG; }
  if (m == 0) return FGB_OK;
  fgb::csr_spmm_kernel<float><<<fgb::grid_for(m * 32, 256, 152LL * 64), 256, 0, fgb::as_stream(stream)>>>(
      indptr, indices, data, m, X, K, Y, add, alpha);
  FGB_LAUNCH_CHECK("csr_spmm_kernel");
  return FGB_OK;
}

}  // extern "C"
