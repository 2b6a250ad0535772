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
//     the sweep reads the pre-step profile from there;
//   * the sweep's own arrays never touch local memory: the solution u is
//     written in place into the staged row (the right-hand side has read
//     each pre-step value before), and gam, the elimination factors, is a
//     per-thread column of shared memory (element j of thread t at
//     j * nt + t, conflict-free); a predictor-corrector redo reloads the
//     pre-step row from T_in, which no CTA overwrites before its own
//     rows are done; the facets per CTA (32..128) follow from nz;
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

// What the forward sweep reads for row j, packed so that a thread fetches it
// with two or three 16-byte shared loads: gamma_j, alpha_j,
// mid_j = 1 - alpha_j - gamma_j (the explicit half's diagonal, evaluated as
// in conductionQ.c), a_j, b_j and c_{j-1}.
template <class R>
struct alignas(16) Layer {
  R ga, al, mid, a, b, cm1;
};

template <class R> struct Consts;
template <> struct Consts<double> { static constexpr double sigSB = 5.6704e-8; };
template <> struct Consts<float> { static constexpr float sigSB = 5.6704e-8f; };

// Grid coefficients shared by all facets (conductionQ.c:69-97), computed by
// the CTA's threads in parallel, one layer each, with the reference's
// operations for every element (bit-identical to the serial loops).
template <class R>
__device__ void grid_coeffs_q(int nz, const R* z, R dt, const R* ti, const R* rhoc,
                              R* k, R* alpha, R* gamma, R* a, R* b, R* c, R* k1_out) {
  for (int i = threadIdx.x + 1; i <= nz; i += blockDim.x) k[i] = ti[i] * ti[i] / rhoc[i];
  __syncthreads();
  const R dz = R(2) * z[1];
  for (int i = threadIdx.x + 1; i <= nz; i += blockDim.x) {
    R al, ga;
    if (i == 1) {
      const R beta = dt / rhoc[1] / (R(2) * dz * dz);
      al = beta * k[2];
      ga = beta * k[1];
    } else if (i < nz) {
      const R buf = dt / (z[i + 1] - z[i - 1]);
      al = R(2) * k[i + 1] * buf / (rhoc[i] + rhoc[i + 1]) / (z[i + 1] - z[i]);
      ga = R(2) * k[i] * buf / (rhoc[i] + rhoc[i + 1]) / (z[i] - z[i - 1]);
    } else {
      const R buf = dt / (z[nz] - z[nz - 1]) / (z[nz] - z[nz - 1]);
      ga = k[nz] * buf / (R(2) * rhoc[nz]);
      al = R(0);  // never read by the solve (c[nz] unused, b[nz] reset)
    }
    alpha[i] = al;
    gamma[i] = ga;
    a[i] = -ga;
    b[i] = (i == nz) ? R(1) + ga : R(1) + al + ga;
    c[i] = -al;
  }
  if (threadIdx.x == 0) *k1_out = k[1] / dz;
}

// Grid coefficients for the prescribed-temperature boundary (conductionT.c:45-64).
template <class R>
__device__ void grid_coeffs_t(int nz, const R* z, R dt, const R* ti, const R* rhoc,
                              R* k, R* alpha, R* gamma, R* a, R* b, R* c) {
  for (int i = threadIdx.x + 1; i <= nz; i += blockDim.x) k[i] = ti[i] * ti[i] / rhoc[i];
  __syncthreads();
  for (int i = threadIdx.x + 1; i <= nz; i += blockDim.x) {
    R al, ga;
    if (i == 1) {
      al = k[2] * dt / rhoc[1] / (z[2] - z[1]) / z[2];
      ga = k[1] * dt / rhoc[1] / z[1] / z[2];
    } else if (i < nz) {
      const R buf = dt / (z[i + 1] - z[i - 1]);
      al = R(2) * k[i + 1] * buf / (rhoc[i] + rhoc[i + 1]) / (z[i + 1] - z[i]);
      ga = R(2) * k[i] * buf / (rhoc[i] + rhoc[i + 1]) / (z[i] - z[i - 1]);
    } else {
      const R buf = dt / (z[nz] - z[nz - 1]) / (z[nz] - z[nz - 1]);
      ga = k[nz] * buf / (rhoc[nz] + rhoc[nz]);
      al = R(0);
    }
    alpha[i] = al;
    gamma[i] = ga;
    a[i] = -ga;
    b[i] = (i == nz) ? R(1) + ga : R(1) + al + ga;
    c[i] = -al;
  }
}

constexpr int kMaxThreads = 128;
constexpr size_t kSmemBudget = 227 * 1024;  // the per-CTA opt-in maximum

// Shared layout, all of element type R: 7 coefficient arrays of nz+1 (k,
// alpha, gamma, a, b, c, misc), then the staged temperature tile, nt rows
// of stride ws = (nz+1)|1 (odd, so that the threads of a warp reading
// element i of their own rows hit distinct banks).  The sweep's own arrays
// (u, gam) are per-thread local arrays: the shared layout stays small, so
// that many CTAs (warps) share an SM and hide the sweep's dependent chain.
__host__ __device__ inline int tile_stride(int nz) { return (nz + 1) | 1; }

// Shared layout: the coefficients, the tile (nt rows of stride ws), the
// threads' gam columns (nz + 1 rows of nt), then the packed layer table
// (nz + 1 entries, 16-byte aligned).
template <class R>
__host__ __device__ inline size_t cond_smem_scalars(int nz, int nt) {
  return (size_t)7 * (nz + 1) + (size_t)nt * (tile_stride(nz) + nz + 1);
}

template <class R>
size_t cond_smem(int nz, int nt) {
  const size_t bytes = sizeof(R) * cond_smem_scalars<R>(nz, nt);
  return (bytes + 15) / 16 * 16 + sizeof(Layer<R>) * (size_t)(nz + 1);
}

template <class R>
__device__ Layer<R>* layers_at(R* sh, int nz, int nt) {
  const size_t bytes = sizeof(R) * cond_smem_scalars<R>(nz, nt);
  return reinterpret_cast<Layer<R>*>(reinterpret_cast<unsigned char*>(sh) +
                                     (bytes + 15) / 16 * 16);
}

// Facets per CTA: the multiple of 32 (at most 128) that keeps the most
// facets resident per SM (228 KiB of shared memory, 1 KiB of it reserved
// per CTA), the larger on ties; 0 if even one warp does not fit.
template <class R>
int cond_threads(int nz) {
  int best = 0, best_res = 0;
  for (int nt = 32; nt <= kMaxThreads; nt += 32) {
    const size_t sm = cond_smem<R>(nz, nt);
    if (sm > kSmemBudget) break;
    const int ctas = (int)((228 * 1024) / (sm + 1024));
    const int res = nt * (ctas < 2048 / nt ? ctas : 2048 / nt);
    if (res >= best_res) { best_res = res; best = nt; }
  }
  return best;
}

template <class R>
__device__ inline R* coeff(R* sh, int which, int nz) { return sh + which * (nz + 1); }

// Row-major global rows [f0, f0+rows) x w  <->  tile rows of stride ws.
// Thread q of the CTA visits elements q, q + nt, ... of the rows (coalesced
// in global memory); its (row, column) advances by (nt / w, nt % w) per
// step, one division per thread.
template <class R, bool IN>
__device__ void stage(R* tile, R* T, long long f0, int rows, int w, int ws) {
  const int nt = blockDim.x;
  const int n = rows * w;
  const int dr = nt / w, dc = nt - dr * w;
  int q = threadIdx.x;
  int r = q / w, c = q - r * w;
  R* g = T + f0 * w;
  for (; q < n; q += nt) {
    if (IN) tile[r * ws + c] = g[q];
    else g[q] = tile[r * ws + c];
    r += dr;
    c += dc;
    if (c >= w) { c -= w; r++; }
  }
}

template <class R>
__device__ inline bool finite_val(R x) { return isfinite(x); }

// x / d. FP64 keeps the IEEE quotient of the reference's C code (results
// bit-identical to it); FP32 multiplies by one fast approximate reciprocal
// of the pivot per layer (the FP32 kernel is a faster, less exact variant).
template <class R> struct Pivot;
template <> struct Pivot<double> {
  double d;
  __device__ explicit Pivot(double v) : d(v) {}
  __device__ double div(double x) const { return x / d; }
};
template <> struct Pivot<float> {
  float r;
  __device__ explicit Pivot(float v) { r = __fdividef(1.0f, v); }
  __device__ float div(float x) const { return x * r; }
};

template <class R>
__device__ void pack_layers(int nz, const R* s_alpha, const R* s_gamma, const R* s_a,
                            const R* s_b, const R* s_c, Layer<R>* L) {
  for (int j = threadIdx.x + 2; j <= nz; j += blockDim.x) {
    const R al = j < nz ? s_alpha[j] : R(0), ga = s_gamma[j];
    L[j] = {ga, al, R(1) - al - ga, s_a[j], s_b[j], s_c[j - 1]};
  }
}

// Forward sweep and back substitution of the tridiagonal system with
// sub/main/super diagonals (a, b, c) from shared memory, except the first
// main-diagonal entry b1 (facet dependent under the radiative boundary).
// The right-hand side is formed on the fly from the pre-step profile in
// Trow (crank-nicolson explicit half, conductionQ.c:123-137 /
// conductionT.c:66-77), r1 precomputed by the caller; the solution
// overwrites Trow[1..nz] (each pre-step value is read before it is
// overwritten).  gam: the thread's shared column (element j at gam[j * gs]).
// The arithmetic is the reference's tridag (tridag.c:5-34) in its order.
// Returns false on a zero pivot.
template <class R>
__device__ bool thomas_cn(int nz, R* Trow, R r1, R b1, R rhs_bottom, const Layer<R>* L, R* gam,
                          int gs) {
  R bet = b1;
  if (bet == R(0)) return false;
  Pivot<R> pv(bet);
  R tm1 = Trow[1], t0 = Trow[2];
  R uprev = pv.div(r1);
  Trow[1] = uprev;
  for (int j = 2; j <= nz; j++) {
    const Layer<R> l = L[j];
    R rj;
    if (j < nz) {
      const R tp1 = Trow[j + 1];
      rj = l.ga * tm1 + l.mid * t0 + l.al * tp1;
      tm1 = t0;
      t0 = tp1;
    } else {
      rj = l.ga * tm1 + l.mid * t0 + rhs_bottom;
    }
    const R g = pv.div(l.cm1);
    gam[j * gs] = g;
    bet = l.b - l.a * g;
    if (bet == R(0)) return false;
    pv = Pivot<R>(bet);
    uprev = pv.div(rj - l.a * uprev);
    Trow[j] = uprev;
  }
  R unext = uprev;
  for (int j = nz - 1; j >= 1; j--) {
    unext = Trow[j] - gam[(j + 1) * gs] * unext;
    Trow[j] = unext;
  }
  return true;
}

// One step of the radiative-flux boundary problem for every facet.
template <class R, int NZMAX>
__global__ void __launch_bounds__(kMaxThreads, 1)
conduction_q_kernel(int num_faces, int nz, const R* __restrict__ z, R dt,
                    const R* __restrict__ Qn, const R* __restrict__ Qnp1,
                    const R* T_in, R* T_out,
                    const R* __restrict__ ti, const R* __restrict__ rhoc,
                    const R* __restrict__ emiss, const R* __restrict__ Fgeotherm,
                    R* __restrict__ Fsurf, unsigned* __restrict__ flags) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  R* sh = reinterpret_cast<R*>(smem_raw);
  const int w = nz + 1, ws = tile_stride(nz), nt = blockDim.x;
  R* s_k = coeff(sh, 0, nz);
  R* s_alpha = coeff(sh, 1, nz);
  R* s_gamma = coeff(sh, 2, nz);
  R* s_a = coeff(sh, 3, nz);
  R* s_b = coeff(sh, 4, nz);
  R* s_c = coeff(sh, 5, nz);
  R* s_misc = coeff(sh, 6, nz);  // [0] = k1
  R* tile = sh + 7 * w;

  Layer<R>* s_L = layers_at(sh, nz, nt);
  grid_coeffs_q<R>(nz, z, dt, ti, rhoc, s_k, s_alpha, s_gamma, s_a, s_b, s_c, &s_misc[0]);
  __syncthreads();
  pack_layers<R>(nz, s_alpha, s_gamma, s_a, s_b, s_c, s_L);
  const long long f0 = (long long)blockIdx.x * nt;
  const int rows = (int)min((long long)nt, (long long)num_faces - f0);
  stage<R, true>(tile, const_cast<R*>(T_in), f0, rows, w, ws);
  __syncthreads();

  const int t = threadIdx.x;
  R* gam = tile + nt * ws + t;   // this thread's column, stride nt
  unsigned my_flags = 0;
  if (t < rows) {
    const long long f = f0 + t;
    R* Trow = tile + t * ws;
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
      R r1 = gamma1 * (annp1 + ann) + (R(1) - alpha1 - gamma1 + gamma1 * bn) * Trow[1] +
             alpha1 * Trow[2];
      if (!thomas_cn<R>(nz, Trow, r1, b1, rhs_bottom, s_L, gam, nt)) {
        my_flags |= kFlagZeroPivot;
        break;
      }
      T0 = R(0.5) * (annp1 + bn * Trow[1] + Trow[1]);
      if ((T0 > R(1.2) * Tr || T0 < R(0.8) * Tr) && iter < 10) {
        iter++;
        Tr = sqrt(Tr * T0);
        // redo from the pre-step profile (conductionQ.c resets T)
        const R* src = T_in + f * w;
        for (int i = 1; i <= nz; i++) Trow[i] = src[i];
        continue;
      }
      break;
    }
    if (iter >= 9) my_flags |= kFlagPredCorrMax;
    Trow[0] = T0;
    Fsurf[f] = -s_k[1] * (Trow[1] - T0) / z[1];
    for (int i = 0; i <= nz; i++) {
      if (!finite_val(Trow[i])) my_flags |= kFlagNonfiniteOut;
      if (Trow[i] < R(0)) my_flags |= kFlagNegativeOut;
    }
  }
  __syncthreads();
  stage<R, false>(tile, T_out, f0, rows, w, ws);
  if (my_flags) atomicOr(flags, my_flags);
}

// One step of the prescribed-surface-temperature problem (conductionT.c).
template <class R, int NZMAX>
__global__ void __launch_bounds__(kMaxThreads)
conduction_t_kernel(int num_faces, int nz, const R* __restrict__ z, R dt,
                    const R* __restrict__ Tsurf, const R* __restrict__ Tsurfp1,
                    const R* T_in, R* T_out,
                    const R* __restrict__ ti, const R* __restrict__ rhoc,
                    const R* __restrict__ Fgeotherm, R* __restrict__ Fsurf,
                    unsigned* __restrict__ flags) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  R* sh = reinterpret_cast<R*>(smem_raw);
  const int w = nz + 1, ws = tile_stride(nz), nt = blockDim.x;
  R* s_k = coeff(sh, 0, nz);
  R* s_alpha = coeff(sh, 1, nz);
  R* s_gamma = coeff(sh, 2, nz);
  R* s_a = coeff(sh, 3, nz);
  R* s_b = coeff(sh, 4, nz);
  R* s_c = coeff(sh, 5, nz);
  R* tile = sh + 7 * w;
  Layer<R>* s_L = layers_at(sh, nz, nt);
  grid_coeffs_t<R>(nz, z, dt, ti, rhoc, s_k, s_alpha, s_gamma, s_a, s_b, s_c);
  __syncthreads();
  pack_layers<R>(nz, s_alpha, s_gamma, s_a, s_b, s_c, s_L);
  const long long f0 = (long long)blockIdx.x * nt;
  const int rows = (int)min((long long)nt, (long long)num_faces - f0);
  stage<R, true>(tile, const_cast<R*>(T_in), f0, rows, w, ws);
  __syncthreads();
  const int t = threadIdx.x;
  R* gam = tile + nt * ws + t;
  unsigned my_flags = 0;
  if (t < rows) {
    const long long f = f0 + t;
    R* Trow = tile + t * ws;
    const R ts = Tsurf[f], tsp1 = Tsurfp1[f], fg = Fgeotherm[f];
    if (!finite_val(tsp1)) my_flags |= kFlagNonfiniteIn;
    if (tsp1 < R(0)) my_flags |= kFlagNegativeIn;
    const R alpha1 = s_alpha[1], gamma1 = s_gamma[1];
    R r1 = alpha1 * Trow[2] + (R(1) - alpha1 - gamma1) * Trow[1] + gamma1 * (ts + tsp1);
    const R rhs_bottom = dt / rhoc[nz] * fg / (z[nz] - z[nz - 1]);
    if (!thomas_cn<R>(nz, Trow, r1, s_b[1], rhs_bottom, s_L, gam, nt)) {
      my_flags |= kFlagZeroPivot;
      // the reference leaves T as it was: put the pre-step row back
      const R* src = T_in + f * w;
      for (int i = 1; i <= nz; i++) Trow[i] = src[i];
    } else {
      Fsurf[f] = -s_k[1] * (Trow[1] - tsp1) / z[1];
    }
    for (int i = 1; i <= nz; i++) {
      if (!finite_val(Trow[i])) my_flags |= kFlagNonfiniteOut;
      if (Trow[i] < R(0)) my_flags |= kFlagNegativeOut;
    }
  }
  __syncthreads();
  stage<R, false>(tile, T_out, f0, rows, w, ws);
  if (my_flags) atomicOr(flags, my_flags);
}

template <class R, int NZMAX>
int launch_q(int num_faces, int nz, const R* z, R dt, const R* Qn, const R* Qnp1,
             const R* T_in, R* T_out, const R* ti, const R* rhoc, const R* emiss,
             const R* Fgeotherm, R* Fsurf, unsigned* flags, cudaStream_t s) {
  const int nt = cond_threads<R>(nz);
  const size_t sm = cond_smem<R>(nz, nt);
  auto k = conduction_q_kernel<R, NZMAX>;
  FGB_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  const unsigned grid = (unsigned)((num_faces + nt - 1) / nt);
  k<<<grid, nt, sm, s>>>(num_faces, nz, z, dt, Qn, Qnp1, T_in, T_out, ti, rhoc, emiss,
                         Fgeotherm, Fsurf, flags);
  FGB_LAUNCH_CHECK("conduction_q_kernel");
  return FGB_OK;
}

template <class R, int NZMAX>
int launch_t(int num_faces, int nz, const R* z, R dt, const R* Ts, const R* Tsp1,
             const R* T_in, R* T_out, const R* ti, const R* rhoc, const R* Fgeotherm,
             R* Fsurf, unsigned* flags, cudaStream_t s) {
  const int nt = cond_threads<R>(nz);
  const size_t sm = cond_smem<R>(nz, nt);
  auto k = conduction_t_kernel<R, NZMAX>;
  FGB_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  const unsigned grid = (unsigned)((num_faces + nt - 1) / nt);
  k<<<grid, nt, sm, s>>>(num_faces, nz, z, dt, Ts, Tsp1, T_in, T_out, ti, rhoc, Fgeotherm,
                         Fsurf, flags);
  FGB_LAUNCH_CHECK("conduction_t_kernel");
  return FGB_OK;
}

template <class R>
int check_args(int num_faces, int nz) {
  if (num_faces < 0) { set_error("num_faces must be >= 0"); return FGB_BAD_ARG; }
  if (nz < 2 || nz > 255) { set_error("nz (interior layers) must be in [2, 255], got %d", nz); return FGB_BAD_ARG; }
  if (cond_threads<R>(nz) == 0) {
    set_error("nz too large for the staged tile");
    return FGB_BAD_ARG;
  }
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
