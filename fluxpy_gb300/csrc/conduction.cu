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

// The staged temperature tile: nt rows of stride ws = (nz+1)|1 (odd, so
// that the threads of a warp reading element i of their own rows hit
// distinct banks), after 7 coefficient arrays of nz+1 (k, alpha, gamma, a,
// b, c, misc).
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
template <class R>
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

// FP32: the same step with the tridiagonal system eliminated from the bottom
// up.  Rows 2..nz do not depend on the facet except through the right-hand
// side, and only row 1 depends on the linearised radiative boundary, so
//   * the pivots beta_j and factors e_j = c_j / beta_{j+1} of rows nz..2
//     are computed once per CTA (UpRow / DownRow tables);
//   * each facet sweeps up once, y_j = r_j - e_j y_{j+1}, forming r_j from
//     the pre-step profile and overwriting it with y_j;
//   * the predictor-corrector iterations (conductionQ.c:103-172) then solve
//     row 1 alone, u_1 = (r_1 - e_1 y_2) / (b_1 - e_1 a_2), with r_1 and b_1
//     from the current linearisation temperature: a redo costs O(1), not a
//     new solve (the reference re-solves the whole system from the pre-step
//     profile, which gives the same u in exact arithmetic);
//   * one substitution down, u_j = (y_j - a_j u_{j-1}) / beta_j.
// No per-facet pivots or elimination factors, no reloads; FMAs are explicit
// (this file is compiled without contraction for the FP64 path).  The
// system is strictly diagonally dominant, so elimination in either direction
// is stable; the FP64 kernel keeps the reference's top-down order.
struct alignas(16) UpRow {
  float ga, mid, al, e;
};
struct alignas(8) DownRow {
  float a, rb;
};

// Shared layout of the FP32 kernel: the 7 coefficient arrays (padded to a
// multiple of 4 floats, so that the tile starts 16-byte aligned), the tile,
// then the UpRow and DownRow tables.
__host__ __device__ inline int cond_up_coeff_floats(int nz) { return (7 * (nz + 1) + 3) & ~3; }
__host__ __device__ inline size_t cond_up_smem(int nz, int nt) {
  const size_t base =
      sizeof(float) * ((size_t)cond_up_coeff_floats(nz) + (size_t)nt * tile_stride(nz));
  return (base + 15) / 16 * 16 + (sizeof(UpRow) + sizeof(DownRow)) * (size_t)(nz + 1);
}

// A warp's own rows [f0, f0 + rows) x w (rows <= 32) <-> its part of the
// tile: a contiguous copy in 16-byte pieces (the last few floats one by
// one) when the tile's stride is w (w odd) and the global rows are 16-byte
// aligned; otherwise element by element.  Only the warp's lanes take part,
// so no CTA barrier is needed around it.
// Loads go through cp.async (global to shared without a register round
// trip): the caller waits for them (cp.async.wait_all) before its barrier.
template <bool IN>
__device__ void stage_warp(float* tile, float* T, long long f0, int rows, int w, int ws,
                           int lane) {
  float* g = T + f0 * w;
  const int n = rows * w;
  if (ws == w && (reinterpret_cast<uintptr_t>(g) & 15) == 0 &&
      (reinterpret_cast<uintptr_t>(tile) & 15) == 0) {
    const int n4 = n >> 2;
    float4* t4 = reinterpret_cast<float4*>(tile);
    float4* g4 = reinterpret_cast<float4*>(g);
    for (int i = lane; i < n4; i += 32) {
      if (IN) {
        const unsigned sa = static_cast<unsigned>(__cvta_generic_to_shared(t4 + i));
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(g4 + i)
                     : "memory");
      } else {
        g4[i] = t4[i];
      }
    }
    if (IN) asm volatile("cp.async.commit_group;\n" ::: "memory");
    for (int i = 4 * n4 + lane; i < n; i += 32) {
      if (IN) tile[i] = g[i];
      else g[i] = tile[i];
    }
    return;
  }
  for (int q = lane; q < n; q += 32) {
    const int r = q / w, c = q - r * w;
    if (IN) tile[r * ws + c] = g[q];
    else g[q] = tile[r * ws + c];
  }
}

constexpr int kUpThreads = 128;

int cond_up_threads(int nz) {
  int best = 0, best_res = 0;
  for (int nt = 32; nt <= kUpThreads; nt += 32) {
    const size_t sm = cond_up_smem(nz, nt);
    if (sm > kSmemBudget) break;
    const int ctas = (int)((228 * 1024) / (sm + 1024));
    const int res = nt * (ctas < 2048 / nt ? ctas : 2048 / nt);
    if (res >= best_res) { best_res = res; best = nt; }
  }
  return best;
}

__global__ void __launch_bounds__(kUpThreads, 9)
conduction_q_up_kernel(int num_faces, int nz, const float* __restrict__ z, float dt,
                       const float* __restrict__ Qn, const float* __restrict__ Qnp1,
                       const float* T_in, float* T_out,
                       const float* __restrict__ ti, const float* __restrict__ rhoc,
                       const float* __restrict__ emiss, const float* __restrict__ Fgeotherm,
                       float* __restrict__ Fsurf, unsigned* __restrict__ flags) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* sh = reinterpret_cast<float*>(smem_raw);
  const int w = nz + 1, ws = tile_stride(nz), nt = blockDim.x;
  float* s_k = coeff(sh, 0, nz);
  float* s_alpha = coeff(sh, 1, nz);
  float* s_gamma = coeff(sh, 2, nz);
  float* s_a = coeff(sh, 3, nz);
  float* s_b = coeff(sh, 4, nz);
  float* s_c = coeff(sh, 5, nz);
  float* s_misc = coeff(sh, 6, nz);  // [0] k1, [1] e_1, [2] e_1 a_2, [3] zero pivot
  float* tile = sh + cond_up_coeff_floats(nz);
  const size_t base = sizeof(float) * ((size_t)cond_up_coeff_floats(nz) + (size_t)nt * ws);
  UpRow* s_up = reinterpret_cast<UpRow*>(smem_raw + (base + 15) / 16 * 16);
  DownRow* s_dn = reinterpret_cast<DownRow*>(s_up + w);

  // each warp stages its own 32 facets' profiles first (their loads are in
  // flight while the coefficients and the elimination are formed)
  const int t = threadIdx.x, lane = t & 31;
  const long long f0 = (long long)blockIdx.x * nt;
  const int rows = (int)min((long long)nt, (long long)num_faces - f0);
  const int wrow0 = t & ~31;
  const int wrows = max(0, min(32, rows - wrow0));
  float* wtile = tile + wrow0 * ws;
  stage_warp<true>(wtile, const_cast<float*>(T_in), f0 + wrow0, wrows, w, ws, lane);
  grid_coeffs_q<float>(nz, z, dt, ti, rhoc, s_k, s_alpha, s_gamma, s_a, s_b, s_c, &s_misc[0]);
  asm volatile("cp.async.wait_all;\n" ::: "memory");
  __syncthreads();
  // the rows' own coefficients, one row per thread (fields apart from the
  // e and rb that thread 0 writes below)
  for (int j = threadIdx.x + 2; j <= nz; j += nt) {
    const float al = j < nz ? s_alpha[j] : 0.0f, ga = s_gamma[j];
    s_up[j].ga = ga;
    s_up[j].mid = 1.0f - al - ga;
    s_up[j].al = al;
    s_dn[j].a = s_a[j];
  }
  if (threadIdx.x == 0) {
    // the facet-independent elimination of rows nz..2: a serial recurrence
    // (one fast reciprocal per row)
    float beta = s_b[nz], rb = __fdividef(1.0f, beta);
    bool zero = beta == 0.0f;
    s_up[nz].e = 0.0f;
    s_dn[nz].rb = rb;
#pragma unroll 4
    for (int j = nz - 1; j >= 2; j--) {
      const float e = s_c[j] * rb;
      beta = __fmaf_rn(-e, s_a[j + 1], s_b[j]);
      zero = zero || beta == 0.0f;
      rb = __fdividef(1.0f, beta);
      s_up[j].e = e;
      s_dn[j].rb = rb;
    }
    const float e1 = s_c[1] * rb;
    s_misc[1] = e1;
    s_misc[2] = e1 * s_a[2];
    s_misc[3] = zero ? 1.0f : 0.0f;
  }
  __syncthreads();

  unsigned my_flags = 0;
  if (t < rows) {
    const long long f = f0 + t;
    float* Trow = tile + t * ws;
    const float qn = Qn[f], qnp1 = Qnp1[f], em = emiss[f], fg = Fgeotherm[f];
    if (!finite_val(qnp1)) my_flags |= kFlagNonfiniteIn;
    if (qnp1 < 0.0f) my_flags |= kFlagNegativeIn;
    if (s_misc[3] != 0.0f) my_flags |= kFlagZeroPivot;
    const float rhs_bottom = dt / rhoc[nz] * fg / (z[nz] - z[nz - 1]);
    // sweep up: y_j = r_j - e_j y_{j+1}, r_j from the pre-step profile
    // (tj = T[j], tj1 = T[j+1] of the pre-step profile, in registers); row
    // nz carries the bottom flux and e_nz = 0
    float tj1 = Trow[nz], tj = Trow[nz - 1], y;
    {
      const UpRow u = s_up[nz];
      y = __fmaf_rn(u.mid, tj1, __fmaf_rn(u.ga, tj, rhs_bottom));
      Trow[nz] = y;
    }
#pragma unroll 4
    for (int j = nz - 1; j >= 2; j--) {
      const UpRow u = s_up[j];
      const float tm1 = Trow[j - 1];
      const float r = __fmaf_rn(u.al, tj1, __fmaf_rn(u.mid, tj, __fmul_rn(u.ga, tm1)));
      y = __fmaf_rn(-u.e, y, r);
      Trow[j] = y;
      tj1 = tj;
      tj = tm1;
    }
    const float t1 = tj, t2 = tj1, y2 = y;
    // predictor-corrector on row 1 alone
    const float k1 = s_misc[0], e1 = s_misc[1], e1a2 = s_misc[2];
    const float sig = Consts<float>::sigSB;
    const float alpha1 = s_alpha[1], gamma1 = s_gamma[1];
    float Tr = Trow[0], T0 = Tr, u1 = t1;
    int iter = 0;
    while (true) {
      const float arad = -3.0f * em * sig * Tr * Tr * Tr * Tr;
      const float brad = 2.0f * em * sig * Tr * Tr * Tr;
      const float inv = __fdividef(1.0f, k1 + brad);
      const float ann = (qn - arad) * inv;
      const float annp1 = (qnp1 - arad) * inv;
      const float bn = (k1 - brad) * inv;
      const float b1 = 1.0f + alpha1 + gamma1 - gamma1 * bn;
      const float r1 = gamma1 * (annp1 + ann) + (1.0f - alpha1 - gamma1 + gamma1 * bn) * t1 +
                       alpha1 * t2;
      const float beta1 = b1 - e1a2;
      if (beta1 == 0.0f) {
        my_flags |= kFlagZeroPivot;
        break;
      }
      u1 = __fdividef(r1 - e1 * y2, beta1);
      T0 = 0.5f * (annp1 + bn * u1 + u1);
      if ((T0 > 1.2f * Tr || T0 < 0.8f * Tr) && iter < 10) {
        iter++;
        Tr = sqrtf(Tr * T0);
        continue;
      }
      break;
    }
    if (iter >= 9) my_flags |= kFlagPredCorrMax;
    // substitute down: u_j = (y_j - a_j u_{j-1}) / beta_j; the output
    // checks through a running sum (NaN and infinity propagate) and minimum
    Trow[0] = T0;
    Trow[1] = u1;
    float up = u1, sum = T0 + u1, mn = fminf(T0, u1);
#pragma unroll 4
    for (int j = 2; j <= nz; j++) {
      const DownRow d = s_dn[j];
      up = __fmul_rn(__fmaf_rn(-d.a, up, Trow[j]), d.rb);
      Trow[j] = up;
      sum += up;
      mn = fminf(mn, up);
    }
    if (!finite_val(sum)) my_flags |= kFlagNonfiniteOut;
    if (mn < 0.0f) my_flags |= kFlagNegativeOut;
    Fsurf[f] = -s_k[1] * (u1 - T0) / z[1];
  }
  // the warp writes its own rows back
  __syncwarp();
  stage_warp<false>(wtile, T_out, f0 + wrow0, wrows, w, ws, lane);
  if (my_flags) atomicOr(flags, my_flags);
}

int launch_q_up(int num_faces, int nz, const float* z, float dt, const float* Qn,
                const float* Qnp1, const float* T_in, float* T_out, const float* ti,
                const float* rhoc, const float* emiss, const float* Fgeotherm, float* Fsurf,
                unsigned* flags, cudaStream_t s) {
  const int nt = cond_up_threads(nz);
  const size_t sm = cond_up_smem(nz, nt);
  FGB_CUDA_TRY(cudaFuncSetAttribute(conduction_q_up_kernel,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  const unsigned grid = (unsigned)((num_faces + nt - 1) / nt);
  conduction_q_up_kernel<<<grid, nt, sm, s>>>(num_faces, nz, z, dt, Qn, Qnp1, T_in, T_out, ti,
                                              rhoc, emiss, Fgeotherm, Fsurf, flags);
  FGB_LAUNCH_CHECK("conduction_q_up_kernel");
  return FGB_OK;
}

// One step of the prescribed-surface-temperature problem (conductionT.c).
template <class R>
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

template <class R>
int launch_q(int num_faces, int nz, const R* z, R dt, const R* Qn, const R* Qnp1,
             const R* T_in, R* T_out, const R* ti, const R* rhoc, const R* emiss,
             const R* Fgeotherm, R* Fsurf, unsigned* flags, cudaStream_t s) {
  const int nt = cond_threads<R>(nz);
  const size_t sm = cond_smem<R>(nz, nt);
  auto k = conduction_q_kernel<R>;
  FGB_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  const unsigned grid = (unsigned)((num_faces + nt - 1) / nt);
  k<<<grid, nt, sm, s>>>(num_faces, nz, z, dt, Qn, Qnp1, T_in, T_out, ti, rhoc, emiss,
                         Fgeotherm, Fsurf, flags);
  FGB_LAUNCH_CHECK("conduction_q_kernel");
  return FGB_OK;
}

template <class R>
int launch_t(int num_faces, int nz, const R* z, R dt, const R* Ts, const R* Tsp1,
             const R* T_in, R* T_out, const R* ti, const R* rhoc, const R* Fgeotherm,
             R* Fsurf, unsigned* flags, cudaStream_t s) {
  const int nt = cond_threads<R>(nz);
  const size_t sm = cond_smem<R>(nz, nt);
  auto k = conduction_t_kernel<R>;
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
  if (sizeof(R) == sizeof(float) && cond_up_threads(nz) > 0)
    return launch_q_up(num_faces, nz, reinterpret_cast<const float*>(z), (float)dt,
                       reinterpret_cast<const float*>(Qn), reinterpret_cast<const float*>(Qnp1),
                       reinterpret_cast<const float*>(T_in), reinterpret_cast<float*>(T_out),
                       reinterpret_cast<const float*>(ti), reinterpret_cast<const float*>(rhoc),
                       reinterpret_cast<const float*>(emiss),
                       reinterpret_cast<const float*>(Fgeotherm), reinterpret_cast<float*>(Fsurf),
                       flags, s);
  return launch_q<R>(num_faces, nz, z, dt, Qn, Qnp1, T_in, T_out, ti, rhoc, emiss, Fgeotherm, Fsurf, flags, s);
}

template <class R>
int dispatch_t(int num_faces, int nz, const R* z, R dt, const R* Ts, const R* Tsp1,
               const R* T_in, R* T_out, const R* ti, const R* rhoc, const R* Fgeotherm,
               R* Fsurf, unsigned* flags, void* stream) {
  int st = check_args<R>(num_faces, nz);
  if (st) return st;
  if (num_faces == 0) return FGB_OK;
  cudaStream_t s = as_stream(stream);
  return launch_t<R>(num_faces, nz, z, dt, Ts, Tsp1, T_in, T_out, ti, rhoc, Fgeotherm, Fsurf, flags, s);
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
