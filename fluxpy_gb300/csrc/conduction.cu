// Batched 1-D Crank-Nicolson heat conduction, one facet per thread.
//
// Restates the per-facet C routines of the reference thermal model
// (src/flux/pcc/conductionQ.c:10-186, conductionT.c:4-88, tridag.c:5-34),
// which src/flux/thermal.pyx:249-261 calls in a serial loop over facets.
// Here every facet of the mesh is stepped by one launch:
//   * the grid-only coefficients (alpha, gamma, a, c, b[2..nz]) are
//     computed once per CTA into shared memory, in the reference's order of
//     operations, so FP64 results are bit-identical to the C code compiled
//     without FMA contraction (this file is compiled with -fmad=false);
//   * the temperature rows (num_faces x (nz+1), the reference's row-major
//     layout) are staged through shared memory with coalesced loads/stores;
//   * the linearised radiative boundary (predictor-corrector, at most 10
//     redos, conductionQ.c:103-172) and the Thomas solve are fused: the
//     right-hand side is formed on the fly during the forward sweep from the
//     pre-step profile, which the reference resets T to before every redo.
//   * T_in and T_out may be distinct (double buffering) so that a step with
//     bad input can be discarded by the host, as the reference raises before
//     touching T (thermal.pyx:240-247).
#include "common.cuh"

namespace fgb {
namespace {

template <class R> struct Consts;
template <> struct Consts<double> { static constexpr double sigSB = 5.6704e-8; };
template <> struct Consts<float> { static constexpr float sigSB = 5.6704e-8f; };

// Grid coefficients shared by all facets (conductionQ.c:69-97).
template <class R>
__device__ void grid_coeffs_q(int nz, const R* z, R dt, const R* ti, const R* rhoc,
                              R* k, R* alpha, R* gamma, R* a, R* b, R* c, R* k1_out) {
  for (int i = 1; i <= nz; i++) k[i] = ti[i] * ti[i] / rhoc[i];
  R dz = R(2) * z[1];
  R beta = dt / rhoc[1] / (R(2) * dz * dz);
  alpha[1] = beta * k[2];
  gamma[1] = beta * k[1];
  for (int i = 2; i < nz; i++) {
    R buf = dt / (z[i + 1] - z[i - 1]);
    alpha[i] = R(2) * k[i + 1] * buf / (rhoc[i] + rhoc[i + 1]) / (z[i + 1] - z[i]);
    gamma[i] = R(2) * k[i] * buf / (rhoc[i] + rhoc[i + 1]) / (z[i] - z[i - 1]);
  }
  R buf = dt / (z[nz] - z[nz - 1]) / (z[nz] - z[nz - 1]);
  gamma[nz] = k[nz] * buf / (R(2) * rhoc[nz]);
  alpha[nz] = R(0);  // never read by the solve (c[nz] unused, b[nz] reset)
  *k1_out = k[1] / dz;
  for (int i = 1; i <= nz; i++) {
    a[i] = -gamma[i];
    b[i] = R(1) + alpha[i] + gamma[i];
    c[i] = -alpha[i];
  }
  b[nz] = R(1) + gamma[nz];
}

// Grid coefficients for the prescribed-temperature boundary (conductionT.c:45-64).
template <class R>
__device__ void grid_coeffs_t(int nz, const R* z, R dt, const R* ti, const R* rhoc,
                              R* k, R* alpha, R* gamma, R* a, R* b, R* c) {
  for (int i = 1; i <= nz; i++) k[i] = ti[i] * ti[i] / rhoc[i];
  alpha[1] = k[2] * dt / rhoc[1] / (z[2] - z[1]) / z[2];
  gamma[1] = k[1] * dt / rhoc[1] / z[1] / z[2];
  for (int i = 2; i < nz; i++) {
    R buf = dt / (z[i + 1] - z[i - 1]);
    alpha[i] = R(2) * k[i + 1] * buf / (rhoc[i] + rhoc[i + 1]) / (z[i + 1] - z[i]);
    gamma[i] = R(2) * k[i] * buf / (rhoc[i] + rhoc[i + 1]) / (z[i] - z[i - 1]);
  }
  R buf = dt / (z[nz] - z[nz - 1]) / (z[nz] - z[nz - 1]);
  gamma[nz] = k[nz] * buf / (rhoc[nz] + rhoc[nz]);
  alpha[nz] = R(0);
  for (int i = 1; i <= nz; i++) {
    a[i] = -gamma[i];
    b[i] = R(1) + alpha[i] + gamma[i];
    c[i] = -alpha[i];
  }
  b[nz] = R(1) + gamma[nz];
}

constexpr int kThreads = 128;

// Shared layout: per-layer coefficient arrays (7 x (nz+1)) then the staged
// temperature tile (kThreads x (nz+1)).
template <class R>
__device__ inline R* coeff(R* sh, int which, int nz) { return sh + which * (nz + 1); }

template <class R>
__device__ void stage_in(R* tile, const R* T, long long f0, int rows, int w) {
  const R* src = T + f0 * w;
  long long n = (long long)rows * w;
  for (long long q = threadIdx.x; q < n; q += blockDim.x) tile[q] = src[q];
}

template <class R>
__device__ void stage_out(R* T, const R* tile, long long f0, int rows, int w) {
  R* dst = T + f0 * w;
  long long n = (long long)rows * w;
  for (long long q = threadIdx.x; q < n; q += blockDim.x) dst[q] = tile[q];
}

template <class R>
__device__ inline bool finite_val(R x) { return isfinite(x); }

// One step of the radiative-flux boundary problem for every facet.
template <class R, int NZMAX>
__global__ void __launch_bounds__(kThreads)
conduction_q_kernel(int num_faces, int nz, const R* __restrict__ z, R dt,
                    const R* __restrict__ Qn, const R* __restrict__ Qnp1,
                    const R* T_in, R* T_out,
                    const R* __restrict__ ti, const R* __restrict__ rhoc,
                    const R* __restrict__ emiss, const R* __restrict__ Fgeotherm,
                    R* __restrict__ Fsurf, unsigned* __restrict__ flags) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  R* sh = reinterpret_cast<R*>(smem_raw);
  const int w = nz + 1;
  R* s_k = coeff(sh, 0, nz);
  R* s_alpha = coeff(sh, 1, nz);
  R* s_gamma = coeff(sh, 2, nz);
  R* s_a = coeff(sh, 3, nz);
  R* s_b = coeff(sh, 4, nz);
  R* s_c = coeff(sh, 5, nz);
  R* s_misc = coeff(sh, 6, nz);  // [0] = k1
  R* tile = sh + 7 * w;

  if (threadIdx.x == 0) {
    R k1;
    grid_coeffs_q<R>(nz, z, dt, ti, rhoc, s_k, s_alpha, s_gamma, s_a, s_b, s_c, &k1);
    s_misc[0] = k1;
  }
  const long long f0 = (long long)blockIdx.x * kThreads;
  const int rows = (int)min((long long)kThreads, (long long)num_faces - f0);
  stage_in(tile, T_in, f0, rows, w);
  __syncthreads();

  const int t = threadIdx.x;
  unsigned my_flags = 0;
  if (t < rows) {
    const long long f = f0 + t;
    R* Trow = tile + (long long)t * w;
    R Told[NZMAX + 1];
    R u[NZMAX + 1];
    R gam[NZMAX + 1];
    for (int i = 1; i <= nz; i++) Told[i] = Trow[i];
    const R qn = Qn[f], qnp1 = Qnp1[f], em = emiss[f], fg = Fgeotherm[f];
    if (!finite_val(qnp1)) my_flags |= kFlagNonfiniteIn;
    if (qnp1 < R(0)) my_flags |= kFlagNegativeIn;
    const R k1 = s_misc[0];
    const R sig = Consts<R>::sigSB;
    R Tr = Trow[0];
    R T0 = Tr;
    int iter = 0;
    const R alpha1 = s_alpha[1], gamma1 = s_gamma[1];
    const R rhs_bottom = dt / rhoc[nz] * fg / (z[nz] - z[nz - 1]);
    while (true) {
      R arad = R(-3) * em * sig * Tr * Tr * Tr * Tr;
      R brad = R(2) * em * sig * Tr * Tr * Tr;
      R ann = (qn - arad) / (k1 + brad);
      R annp1 = (qnp1 - arad) / (k1 + brad);
      R bn = (k1 - brad) / (k1 + brad);
      R b1 = R(1) + alpha1 + gamma1 - gamma1 * bn;
      // Thomas forward sweep, right-hand side formed from Told on the fly.
      R r1 = gamma1 * (annp1 + ann) + (R(1) - alpha1 - gamma1 + gamma1 * bn) * Told[1] +
             alpha1 * Told[2];
      R bet = b1;
      if (bet == R(0)) { my_flags |= kFlagZeroPivot; break; }
      u[1] = r1 / bet;
      for (int j = 2; j <= nz; j++) {
        R rj;
        if (j < nz) {
          const R ga = s_gamma[j], al = s_alpha[j];
          rj = ga * Told[j - 1] + (R(1) - al - ga) * Told[j] + al * Told[j + 1];
        } else {
          const R ga = s_gamma[nz];
          rj = ga * Told[nz - 1] + (R(1) - ga) * Told[nz] + rhs_bottom;
        }
        const R aj = s_a[j];
        gam[j] = s_c[j - 1] / bet;
        bet = s_b[j] - aj * gam[j];
        if (bet == R(0)) { my_flags |= kFlagZeroPivot; break; }
        u[j] = (rj - aj * u[j - 1]) / bet;
      }
      if (my_flags & kFlagZeroPivot) break;
      for (int j = nz - 1; j >= 1; j--) u[j] -= gam[j + 1] * u[j + 1];
      T0 = R(0.5) * (annp1 + bn * u[1] + u[1]);
      if ((T0 > R(1.2) * Tr || T0 < R(0.8) * Tr) && iter < 10) {
        iter++;
        Tr = sqrt(Tr * T0);
        continue;
      }
      break;
    }
    if (iter >= 9) my_flags |= kFlagPredCorrMax;
    Trow[0] = T0;
    for (int i = 1; i <= nz; i++) Trow[i] = u[i];
    Fsurf[f] = -s_k[1] * (u[1] - T0) / z[1];
    for (int i = 0; i <= nz; i++) {
      if (!finite_val(Trow[i])) my_flags |= kFlagNonfiniteOut;
      if (Trow[i] < R(0)) my_flags |= kFlagNegativeOut;
    }
  }
  __syncthreads();
  stage_out(T_out, tile, f0, rows, w);
  if (my_flags) atomicOr(flags, my_flags);
}

// One step of the prescribed-surface-temperature problem (conductionT.c).
template <class R, int NZMAX>
__global__ void __launch_bounds__(kThreads)
conduction_t_kernel(int num_faces, int nz, const R* __restrict__ z, R dt,
                    const R* __restrict__ Tsurf, const R* __restrict__ Tsurfp1,
                    const R* T_in, R* T_out,
                    const R* __restrict__ ti, const R* __restrict__ rhoc,
                    const R* __restrict__ Fgeotherm, R* __restrict__ Fsurf,
                    unsigned* __restrict__ flags) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  R* sh = reinterpret_cast<R*>(smem_raw);
  const int w = nz + 1;
  R* s_k = coeff(sh, 0, nz);
  R* s_alpha = coeff(sh, 1, nz);
  R* s_gamma = coeff(sh, 2, nz);
  R* s_a = coeff(sh, 3, nz);
  R* s_b = coeff(sh, 4, nz);
  R* s_c = coeff(sh, 5, nz);
  R* tile = sh + 7 * w;
  if (threadIdx.x == 0)
    grid_coeffs_t<R>(nz, z, dt, ti, rhoc, s_k, s_alpha, s_gamma, s_a, s_b, s_c);
  const long long f0 = (long long)blockIdx.x * kThreads;
  const int rows = (int)min((long long)kThreads, (long long)num_faces - f0);
  stage_in(tile, T_in, f0, rows, w);
  __syncthreads();
  const int t = threadIdx.x;
  unsigned my_flags = 0;
  if (t < rows) {
    const long long f = f0 + t;
    R* Trow = tile + (long long)t * w;
    R Told[NZMAX + 1];
    R u[NZMAX + 1];
    R gam[NZMAX + 1];
    for (int i = 1; i <= nz; i++) Told[i] = Trow[i];
    const R ts = Tsurf[f], tsp1 = Tsurfp1[f], fg = Fgeotherm[f];
    if (!finite_val(tsp1)) my_flags |= kFlagNonfiniteIn;
    if (tsp1 < R(0)) my_flags |= kFlagNegativeIn;
    const R alpha1 = s_alpha[1], gamma1 = s_gamma[1];
    R r1 = alpha1 * Told[2] + (R(1) - alpha1 - gamma1) * Told[1] + gamma1 * (ts + tsp1);
    R bet = s_b[1];
    if (bet == R(0)) my_flags |= kFlagZeroPivot;
    else {
      u[1] = r1 / bet;
      const R rhs_bottom = dt / rhoc[nz] * fg / (z[nz] - z[nz - 1]);
      for (int j = 2; j <= nz; j++) {
        R rj;
        if (j < nz) {
          const R ga = s_gamma[j], al = s_alpha[j];
          rj = ga * Told[j - 1] + (R(1) - al - ga) * Told[j] + al * Told[j + 1];
        } else {
          const R ga = s_gamma[nz];
          rj = ga * Told[nz - 1] + (R(1) - ga) * Told[nz] + rhs_bottom;
        }
        const R aj = s_a[j];
        gam[j] = s_c[j - 1] / bet;
        bet = s_b[j] - aj * gam[j];
        if (bet == R(0)) { my_flags |= kFlagZeroPivot; break; }
        u[j] = (rj - aj * u[j - 1]) / bet;
      }
      if (!(my_flags & kFlagZeroPivot)) {
        for (int j = nz - 1; j >= 1; j--) u[j] -= gam[j + 1] * u[j + 1];
        for (int i = 1; i <= nz; i++) Trow[i] = u[i];
        Fsurf[f] = -s_k[1] * (u[1] - tsp1) / z[1];
      }
    }
    for (int i = 1; i <= nz; i++) {
      if (!finite_val(Trow[i])) my_flags |= kFlagNonfiniteOut;
      if (Trow[i] < R(0)) my_flags |= kFlagNegativeOut;
    }
  }
  __syncthreads();
  stage_out(T_out, tile, f0, rows, w);
  if (my_flags) atomicOr(flags, my_flags);
}

template <class R>
size_t smem_bytes(int nz) { return sizeof(R) * (size_t)(nz + 1) * (7 + kThreads); }

template <class R, int NZMAX>
int launch_q(int num_faces, int nz, const R* z, R dt, const R* Qn, const R* Qnp1,
             const R* T_in, R* T_out, const R* ti, const R* rhoc, const R* emiss,
             const R* Fgeotherm, R* Fsurf, unsigned* flags, cudaStream_t s) {
  size_t sm = smem_bytes<R>(nz);
  auto k = conduction_q_kernel<R, NZMAX>;
  FGB_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  unsigned grid = (unsigned)((num_faces + kThreads - 1) / kThreads);
  k<<<grid, kThreads, sm, s>>>(num_faces, nz, z, dt, Qn, Qnp1, T_in, T_out, ti, rhoc, emiss,
                               Fgeotherm, Fsurf, flags);
  FGB_LAUNCH_CHECK("conduction_q_kernel");
  return FGB_OK;
}

template <class R, int NZMAX>
int launch_t(int num_faces, int nz, const R* z, R dt, const R* Ts, const R* Tsp1,
             const R* T_in, R* T_out, const R* ti, const R* rhoc, const R* Fgeotherm,
             R* Fsurf, unsigned* flags, cudaStream_t s) {
  size_t sm = smem_bytes<R>(nz);
  auto k = conduction_t_kernel<R, NZMAX>;
  FGB_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  unsigned grid = (unsigned)((num_faces + kThreads - 1) / kThreads);
  k<<<grid, kThreads, sm, s>>>(num_faces, nz, z, dt, Ts, Tsp1, T_in, T_out, ti, rhoc, Fgeotherm,
                               Fsurf, flags);
  FGB_LAUNCH_CHECK("conduction_t_kernel");
  return FGB_OK;
}

template <class R>
int check_args(int num_faces, int nz) {
  if (num_faces < 0) { set_error("num_faces must be >= 0"); return FGB_BAD_ARG; }
  if (nz < 2 || nz > 255) { set_error("nz (interior layers) must be in [2, 255], got %d", nz); return FGB_BAD_ARG; }
  if (smem_bytes<R>(nz) > 227 * 1024) { set_error("nz too large for the staged tile"); return FGB_BAD_ARG; }
  return FGB_OK;
}

template <class R>
int dispatch_q(int num_faces, int nz, const R* z, R dt, const R* Qn, const R* Qnp1,
               const R* T_in, R* T_out, const R* ti, const R* rhoc, const R* emiss,
               const R* Fgeotherm, R* Fsurf, unsigned* flags, void* stream) {
  int st = check_args<R>(num_faces, nz);
  if (st) return st;
  if (num_faces == 0) return FGB_OK;
  cudaStream_t s = as_stream(stream);
  if (nz <= 47) return launch_q<R, 47>(num_faces, nz, z, dt, Qn, Qnp1, T_in, T_out, ti, rhoc, emiss, Fgeotherm, Fsurf, flags, s);
  if (nz <= 63) return launch_q<R, 63>(num_faces, nz, z, dt, Qn, Qnp1, T_in, T_out, ti, rhoc, emiss, Fgeotherm, Fsurf, flags, s);
  if (nz <= 127) return launch_q<R, 127>(num_faces, nz, z, dt, Qn, Qnp1, T_in, T_out, ti, rhoc, emiss, Fgeotherm, Fsurf, flags, s);
  return launch_q<R, 255>(num_faces, nz, z, dt, Qn, Qnp1, T_in, T_out, ti, rhoc, emiss, Fgeotherm, Fsurf, flags, s);
}

template <class R>
int dispatch_t(int num_faces, int nz, const R* z, R dt, const R* Ts, const R* Tsp1,
               const R* T_in, R* T_out, const R* ti, const R* rhoc, const R* Fgeotherm,
               R* Fsurf, unsigned* flags, void* stream) {
  int st = check_args<R>(num_faces, nz);
  if (st) return st;
  if (num_faces == 0) return FGB_OK;
  cudaStream_t s = as_stream(stream);
  if (nz <= 47) return launch_t<R, 47>(num_faces, nz, z, dt, Ts, Tsp1, T_in, T_out, ti, rhoc, Fgeotherm, Fsurf, flags, s);
  if (nz <= 63) return launch_t<R, 63>(num_faces, nz, z, dt, Ts, Tsp1, T_in, T_out, ti, rhoc, Fgeotherm, Fsurf, flags, s);
  if (nz <= 127) return launch_t<R, 127>(num_faces, nz, z, dt, Ts, Tsp1, T_in, T_out, ti, rhoc, Fgeotherm, Fsurf, flags, s);
  return launch_t<R, 255>(num_faces, nz, z, dt, Ts, Tsp1, T_in, T_out, ti, rhoc, Fgeotherm, Fsurf, flags, s);
}

}  // namespace
}  // namespace fgb

extern "C" {

int fgb_conduction_q_f64(int num_faces, int nz, const double* z, double dt, const double* Qn,
                         const double* Qnp1, const double* T_in, double* T_out,
                         const double* ti, const double* rhoc, const double* emiss,
                         const double* Fgeotherm, double* Fsurf, unsigned* flags,
                         void* stream) {
  return fgb::dispatch_q<double>(num_faces, nz, z, dt, Qn, Qnp1, T_in, T_out, ti, rhoc, emiss,
                                 Fgeotherm, Fsurf, flags, stream);
}

int fgb_conduction_q_f32(int num_faces, int nz, const float* z, float dt, const float* Qn,
                         const float* Qnp1, const float* T_in, float* T_out, const float* ti,
                         const float* rhoc, const float* emiss, const float* Fgeotherm,
                         float* Fsurf, unsigned* flags, void* stream) {
  return fgb::dispatch_q<float>(num_faces, nz, z, dt, Qn, Qnp1, T_in, T_out, ti, rhoc, emiss,
                                Fgeotherm, Fsurf, flags, stream);
}

int fgb_conduction_t_f64(int num_faces, int nz, const double* z, double dt,
                         const double* Tsurf, const double* Tsurfp1, const double* T_in,
                         double* T_out, const double* ti, const double* rhoc,
                         const double* Fgeotherm, double* Fsurf, unsigned* flags,
                         void* stream) {
  return fgb::dispatch_t<double>(num_faces, nz, z, dt, Tsurf, Tsurfp1, T_in, T_out, ti, rhoc,
                                 Fgeotherm, Fsurf, flags, stream);
}

}  // extern "C"
