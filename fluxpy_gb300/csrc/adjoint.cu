// Reverse-mode pieces of the radiosity + conduction model.
//
// * conduction_q_facet_kernel: one conductionQ step (src/flux/pcc/
//   conductionQ.c:10-186, tridag.c:5-34) for every facet, with the thermal
//   inertia given per facet and layer (row stride ti_ld; 0 = one profile
//   shared by all facets).  One thread per facet; the facet's alpha/gamma
//   coefficients are formed in the reference's order of operations, so with
//   a shared profile the result is bit-identical to fgb_conduction_q_f64
//   (this file is compiled without FMA contraction).
// * conduction_q_adjoint_kernel: the transpose of that step's Jacobian
//   applied to a cotangent of the new profiles.  The step's predictor-
//   corrector passes (conductionQ.c:103-172; a redo linearises about
//   sqrt(Tr T0) of the previous pass) are replayed forwards, recording the
//   linearisation temperatures, then taken in reverse: per pass the
//   transposed tridiagonal system is solved (Thomas on M^T) and the
//   cotangents of the boundary terms, the coefficients alpha, gamma, k1/dz,
//   the pre-step profile, the fluxes and the emissivity are accumulated;
//   the coefficient cotangents are mapped to the thermal inertia at the end.
// * phaseBt_k1 / phaseAt_k1: y -> F^T y for the compressed operator, the
//   transpose of the two-phase panel product of matvec.cu: phase B^T
//   scatters each panel row's dot product with its tile's 64 y values into
//   the source vector [Zbar; Xbar] (FP64 atomics: panel rows of different
//   tiles share sources), phase A^T adds V_g Zbar_g into the columns of
//   each low-rank group.  Used by the transposed solve of the adjoint and by
//   CompressedKernelMatrix's transpose product
//   (src/flux/compressed_form_factors.py:904-913).
#include "common.cuh"

namespace fgb {
namespace {

constexpr double kSigPcc = 5.6704e-8;  // conductionQ.c:55
constexpr int kPassMax = 11;            // first pass + at most 10 redos

// Per-facet grid coefficients (conductionQ.c:69-83).  al[i], ga[i] for
// i = 1..nz (al[nz] unused); returns k1/dz and k[1].
__device__ void facet_coeffs(int nz, const double* z, double dt, const double* ti,
                             const double* rhoc, double* al, double* ga, double* kappa) {
  auto k = [&](int i) { return ti[i] * ti[i] / rhoc[i]; };
  const double dz = 2. * z[1];
  const double beta = dt / rhoc[1] / (2. * dz * dz);
  al[1] = beta * k(2);
  ga[1] = beta * k(1);
  for (int i = 2; i < nz; i++) {
    const double buf = dt / (z[i + 1] - z[i - 1]);
    al[i] = 2 * k(i + 1) * buf / (rhoc[i] + rhoc[i + 1]) / (z[i + 1] - z[i]);
    ga[i] = 2 * k(i) * buf / (rhoc[i] + rhoc[i + 1]) / (z[i] - z[i - 1]);
  }
  const double buf = dt / (z[nz] - z[nz - 1]) / (z[nz] - z[nz - 1]);
  ga[nz] = k(nz) * buf / (2 * rhoc[nz]);
  al[nz] = 0.0;
  *kappa = k(1) / dz;
}

struct PassOut {
  double T0, brad, ann, annp1, bn, b1;
  bool ok;
};

// One linearised pass about Tr (conductionQ.c:103-157): u[1..nz] and T0.
// T: the pre-step profile; gam: Thomas scratch.
__device__ PassOut cn_pass(int nz, const double* T, const double* al, const double* ga,
                           double kappa, double rb, double Tr, double qn, double qnp1,
                           double em, double* u, double* gam) {
  PassOut o;
  const double arad = -3 * em * kSigPcc * Tr * Tr * Tr * Tr;
  o.brad = 2 * em * kSigPcc * Tr * Tr * Tr;
  o.ann = (qn - arad) / (kappa + o.brad);
  o.annp1 = (qnp1 - arad) / (kappa + o.brad);
  o.bn = (kappa - o.brad) / (kappa + o.brad);
  o.b1 = 1. + al[1] + ga[1] - ga[1] * o.bn;
  const double r1 = ga[1] * (o.annp1 + o.ann) + (1. - al[1] - ga[1] + ga[1] * o.bn) * T[1] +
                    al[1] * T[2];
  double bet = o.b1;
  o.ok = bet != 0.0;
  if (!o.ok) { o.T0 = 0.0; return o; }
  u[1] = r1 / bet;
  for (int j = 2; j <= nz; j++) {
    const double rj = (j < nz)
        ? ga[j] * T[j - 1] + (1 - al[j] - ga[j]) * T[j] + al[j] * T[j + 1]
        : ga[nz] * T[nz - 1] + (1. - ga[nz]) * T[nz] + rb;
    const double aj = -ga[j];
    gam[j] = (-al[j - 1]) / bet;
    const double bj = (j == nz) ? 1. + ga[nz] : 1. + al[j] + ga[j];
    bet = bj - aj * gam[j];
    if (bet == 0.0) { o.ok = false; o.T0 = 0.0; return o; }
    u[j] = (rj - aj * u[j - 1]) / bet;
  }
  for (int j = nz - 1; j >= 1; j--) u[j] -= gam[j + 1] * u[j + 1];
  o.T0 = 0.5 * (o.annp1 + o.bn * u[1] + u[1]);
  return o;
}

__device__ inline bool redo_test(double T0, double Tr) {
  return T0 > 1.2 * Tr || T0 < 0.8 * Tr;
}

template <int NZMAX>
__global__ void __launch_bounds__(128)
conduction_q_facet_kernel(int num_faces, int nz, const double* __restrict__ z, double dt,
                          const double* __restrict__ Qn, const double* __restrict__ Qnp1,
                          const double* T_in, double* T_out, const double* __restrict__ ti,
                          long long ti_ld, const double* __restrict__ rhoc,
                          const double* __restrict__ emiss,
                          const double* __restrict__ Fgeotherm, unsigned* __restrict__ flags) {
  const long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (f >= num_faces) return;
  const int w = nz + 1;
  double T[NZMAX + 1], al[NZMAX + 1], ga[NZMAX + 1], u[NZMAX + 1], gam[NZMAX + 1];
  for (int i = 0; i < w; i++) T[i] = T_in[f * w + i];
  double kappa;
  facet_coeffs(nz, z, dt, ti + f * ti_ld, rhoc, al, ga, &kappa);
  const double qn = Qn[f], qnp1 = Qnp1[f], em = emiss[f];
  const double rb = dt / rhoc[nz] * Fgeotherm[f] / (z[nz] - z[nz - 1]);
  unsigned fl = 0;
  double Tr = T[0];
  PassOut o;
  for (int it = 0;; it++) {
    o = cn_pass(nz, T, al, ga, kappa, rb, Tr, qn, qnp1, em, u, gam);
    if (!o.ok) { fl |= kFlagZeroPivot; break; }
    if (redo_test(o.T0, Tr) && it < 10) { Tr = sqrt(Tr * o.T0); continue; }
    if (it >= 9) fl |= kFlagPredCorrMax;
    break;
  }
  if (o.ok) {
    T_out[f * w] = o.T0;
    for (int i = 1; i <= nz; i++) T_out[f * w + i] = u[i];
    for (int i = 0; i <= nz; i++) {
      const double v = T_out[f * w + i];
      if (!isfinite(v)) fl |= kFlagNonfiniteOut;
      if (v < 0.0) fl |= kFlagNegativeOut;
    }
  }
  if (fl) atomicOr(flags, fl);
}

// Cotangents in: gT_out (N x w).  Out: gT_in (N x w, overwritten; may be
// the same buffer as gT_out: each thread reads its row before writing it),
// gQn, gQnp1 (overwritten), gemiss (N) and gti (N x w, row stride w) added
// to.
template <int NZMAX>
__global__ void __launch_bounds__(128)
conduction_q_adjoint_kernel(int num_faces, int nz, const double* __restrict__ z, double dt,
                            const double* __restrict__ Qn, const double* __restrict__ Qnp1,
                            const double* __restrict__ T_in, const double* __restrict__ ti,
                            long long ti_ld, const double* __restrict__ rhoc,
                            const double* __restrict__ emiss,
                            const double* __restrict__ Fgeotherm, const double* gT_out,
                            double* gT_in, double* __restrict__ gQn,
                            double* __restrict__ gQnp1, double* __restrict__ gemiss,
                            double* __restrict__ gti, unsigned* __restrict__ flags) {
  const long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (f >= num_faces) return;
  const int w = nz + 1;
  double T[NZMAX + 1], al[NZMAX + 1], ga[NZMAX + 1], u[NZMAX + 1], wk[NZMAX + 1];
  double gr[NZMAX + 1], gTp[NZMAX + 1], gal[NZMAX + 1], gga[NZMAX + 1];
  double trs[kPassMax];
  for (int i = 0; i < w; i++) {
    T[i] = T_in[f * w + i];
    gTp[i] = 0.0;
    gal[i] = 0.0;
    gga[i] = 0.0;
  }
  const double* tif = ti + f * ti_ld;
  double kappa;
  facet_coeffs(nz, z, dt, tif, rhoc, al, ga, &kappa);
  const double qn = Qn[f], qnp1 = Qnp1[f], em = emiss[f];
  const double rb = dt / rhoc[nz] * Fgeotherm[f] / (z[nz] - z[nz - 1]);

  // replay the passes, recording the linearisation temperatures
  int npass = 0;
  {
    double Tr = T[0];
    for (int it = 0;; it++) {
      trs[it] = Tr;
      const PassOut o = cn_pass(nz, T, al, ga, kappa, rb, Tr, qn, qnp1, em, u, wk);
      if (!o.ok) {
        atomicOr(flags, (unsigned)kFlagZeroPivot);
        for (int i = 0; i < w; i++) gT_in[f * w + i] = 0.0;
        gQn[f] = 0.0;
        gQnp1[f] = 0.0;
        return;
      }
      npass = it;
      if (redo_test(o.T0, Tr) && it < 10) { Tr = sqrt(Tr * o.T0); continue; }
      break;
    }
  }

  double gkappa = 0.0, gq_n = 0.0, gq_np1 = 0.0, gem = 0.0, gTr_next = 0.0;
  for (int p = npass; p >= 0; p--) {
    const double Tr = trs[p];
    const PassOut o = cn_pass(nz, T, al, ga, kappa, rb, Tr, qn, qnp1, em, u, wk);
    double gT0;
    if (p == npass) {
      gT0 = gT_out[f * w];
      for (int i = 1; i <= nz; i++) gr[i] = gT_out[f * w + i];
    } else {
      gT0 = 0.0;
      for (int i = 1; i <= nz; i++) gr[i] = 0.0;
    }
    double gTr_carry = 0.0;
    if (p < npass) {
      // Tr_{p+1} = sqrt(Tr_p T0_p)
      const double Tr1 = trs[p + 1];
      gT0 += gTr_next * Tr1 / (2 * o.T0);
      gTr_carry = gTr_next * Tr1 / (2 * Tr);
    }
    // T0 = 0.5 (annp1 + bn u1 + u1)
    double g_annp1 = 0.5 * gT0;
    double g_bn = 0.5 * u[1] * gT0;
    gr[1] += 0.5 * (o.bn + 1) * gT0;
    // gr <- M^-T gr: M^T has sub-diagonal c_{j-1} = -al[j-1] and
    // super-diagonal a_{j+1} = -ga[j+1]; wk holds the Thomas factors
    {
      double bet = o.b1;
      gr[1] = gr[1] / bet;
      for (int j = 2; j <= nz; j++) {
        const double sub = -al[j - 1];
        wk[j] = (-ga[j]) / bet;
        const double bj = (j == nz) ? 1. + ga[nz] : 1. + al[j] + ga[j];
        bet = bj - sub * wk[j];
        gr[j] = (gr[j] - sub * gr[j - 1]) / bet;
      }
      for (int j = nz - 1; j >= 1; j--) gr[j] -= wk[j + 1] * gr[j + 1];
    }
    // matrix entries (dM = -gr u^T on the band) and the right-hand side
    {
      const double g1 = ga[1], a1 = al[1];
      const double gb = -gr[1] * u[1];
      const double gc = -gr[1] * u[2];
      gal[1] += gb - gc + gr[1] * (T[2] - T[1]);
      gga[1] += gb * (1 - o.bn) + gr[1] * ((o.annp1 + o.ann) + (o.bn - 1) * T[1]);
      g_bn += -g1 * gb + gr[1] * g1 * T[1];
      g_annp1 += gr[1] * g1;
      const double g_ann = gr[1] * g1;
      gTp[1] += gr[1] * (1. - a1 - g1 + g1 * o.bn);
      gTp[2] += gr[1] * a1;
      for (int i = 2; i < nz; i++) {
        const double gbi = -gr[i] * u[i];
        const double gai = -gr[i] * u[i - 1];
        const double gci = -gr[i] * u[i + 1];
        gal[i] += gbi - gci + gr[i] * (T[i + 1] - T[i]);
        gga[i] += gbi - gai + gr[i] * (T[i - 1] - T[i]);
        gTp[i - 1] += gr[i] * ga[i];
        gTp[i] += gr[i] * (1 - al[i] - ga[i]);
        gTp[i + 1] += gr[i] * al[i];
      }
      {
        const double gbi = -gr[nz] * u[nz];
        const double gai = -gr[nz] * u[nz - 1];
        gga[nz] += gbi - gai + gr[nz] * (T[nz - 1] - T[nz]);
        gTp[nz - 1] += gr[nz] * ga[nz];
        gTp[nz] += gr[nz] * (1 - ga[nz]);
      }
      // boundary terms -> Tr, emiss, kappa, Qn, Qnp1
      const double D = kappa + o.brad;
      gq_n += g_ann / D;
      gq_np1 += g_annp1 / D;
      const double g_arad = -(g_ann + g_annp1) / D;
      const double g_D = -(g_ann * o.ann + g_annp1 * o.annp1 + g_bn * o.bn) / D;
      gkappa += g_bn / D + g_D;
      const double g_brad = -g_bn / D + g_D;
      const double Tr2 = Tr * Tr, Tr3 = Tr2 * Tr;
      gem += g_arad * (-3 * kSigPcc * Tr3 * Tr) + g_brad * (2 * kSigPcc * Tr3);
      gTr_next = g_arad * (-12 * em * kSigPcc * Tr3) + g_brad * (6 * em * kSigPcc * Tr2) +
                 gTr_carry;
    }
  }
  gTp[0] += gTr_next;

  // alpha, gamma, kappa -> k -> ti
  const double dz = 2. * z[1];
  const double beta = dt / rhoc[1] / (2. * dz * dz);
  for (int i = 0; i < w; i++) wk[i] = 0.0;  // gk
  wk[2] += gal[1] * beta;
  wk[1] += gga[1] * beta + gkappa / dz;
  for (int i = 2; i < nz; i++) {
    const double buf = dt / (z[i + 1] - z[i - 1]);
    const double rs = rhoc[i] + rhoc[i + 1];
    wk[i + 1] += gal[i] * (2 * buf / rs / (z[i + 1] - z[i]));
    wk[i] += gga[i] * (2 * buf / rs / (z[i] - z[i - 1]));
  }
  {
    const double buf = dt / (z[nz] - z[nz - 1]) / (z[nz] - z[nz - 1]);
    wk[nz] += gga[nz] * (buf / (2 * rhoc[nz]));
  }
  for (int i = 1; i <= nz; i++) gti[f * w + i] += wk[i] * 2 * tif[i] / rhoc[i];
  for (int i = 0; i < w; i++) gT_in[f * w + i] = gTp[i];
  gQn[f] = gq_n;
  gQnp1[f] = gq_np1;
  gemiss[f] += gem;
}

// ------------------------------------------------------ F^T products ----
constexpr int kTileRows = 64;

template <class T>
__global__ void __launch_bounds__(256)
phaseBt_k1(const long long* __restrict__ t_p0, const int* __restrict__ src, long long N,
           long long num_src, const T* __restrict__ panel, const double* __restrict__ y,
           double* sbar, unsigned* __restrict__ flags) {
  __shared__ double s_y[kTileRows];
  const long long t = blockIdx.x;
  if (threadIdx.x < kTileRows) {
    const long long row = t * kTileRows + threadIdx.x;
    s_y[threadIdx.x] = row < N ? y[row] : 0.0;
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long p0 = t_p0[t], p1 = t_p0[t + 1];
  const double y0 = s_y[2 * lane], y1 = s_y[2 * lane + 1];
  for (long long l = p0 + warp; l < p1; l += 8) {
    const T* wrow = panel + l * kTileRows;
    double acc = (double)wrow[2 * lane] * y0 + (double)wrow[2 * lane + 1] * y1;
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0 && acc != 0.0) {
      const long long s = src[l];
      if (s >= 0 && s < num_src) atomicAdd(sbar + s, acc);
      else atomicOr(flags, (unsigned)kFlagIndexRange);
    }
  }
}

template <class T>
__global__ void __launch_bounds__(256)
phaseAt_k1(const int* __restrict__ a_grp, const int* __restrict__ a_j0,
           const int* __restrict__ a_j1, long long num_items, const int* __restrict__ g_c0,
           const int* __restrict__ g_kz, const int* __restrict__ g_ldv,
           const long long* __restrict__ g_voff, const long long* __restrict__ g_z0,
           const T* __restrict__ vpanel, double* sbar, long long num_zrows) {
  for (long long it = blockIdx.x; it < num_items; it += gridDim.x) {
    const int g = a_grp[it];
    const int j0 = a_j0[it], j1 = a_j1[it];
    const int kz = g_kz[g];
    const long long ldv = g_ldv[g];
    const T* vg = vpanel + g_voff[g];
    const double* zb = sbar + g_z0[g];
    double* xb = sbar + num_zrows + g_c0[g];
    for (int j = j0 + threadIdx.x; j < j1; j += blockDim.x) {
      double acc = 0.0;
      for (int r = 0; r < kz; r++) acc += (double)vg[r * ldv + j] * zb[r];
      if (acc != 0.0) atomicAdd(xb + j, acc);
    }
  }
}

int check_cond(int num_faces, int nz) {
  if (num_faces < 0) { set_error("num_faces must be >= 0"); return FGB_BAD_ARG; }
  if (nz < 2 || nz > 127) {
    set_error("nz (interior layers) must be in [2, 127] for the per-facet step and its adjoint, got %d", nz);
    return FGB_BAD_ARG;
  }
  return FGB_OK;
}

template <class T>
int rmatvec(const fgb_op_desc* d, const T* panel, const T* vpanel, const double* y,
            double* work, unsigned* flags, cudaStream_t s) {
  if (d->N < 0 || d->num_tiles < 0 || d->num_items < 0 || d->num_zrows < 0) {
    set_error("bad operator sizes");
    return FGB_BAD_ARG;
  }
  if (d->tile_rows != 0 && d->tile_rows != kTileRows) {
    set_error("the transpose product takes the 64-row panel (tile_rows 64)");
    return FGB_BAD_ARG;
  }
  const long long num_src = d->num_zrows + d->N;
  if (num_src > 0) FGB_CUDA_TRY(cudaMemsetAsync(work, 0, sizeof(double) * num_src, s));
  if (d->num_tiles > 0) {
    phaseBt_k1<T><<<(unsigned)d->num_tiles, 256, 0, s>>>(d->t_p0, d->src, d->N, num_src, panel,
                                                         y, work, flags);
    FGB_LAUNCH_CHECK("phaseBt_k1");
  }
  if (d->num_items > 0 && d->num_zrows > 0) {
    phaseAt_k1<T><<<grid_for(d->num_items, 1, 152LL * 64), 256, 0, s>>>(
        d->a_grp, d->a_j0, d->a_j1, d->num_items, d->g_c0, d->g_kz, d->g_ldv, d->g_voff,
        d->g_z0, vpanel, work, d->num_zrows);
    FGB_LAUNCH_CHECK("phaseAt_k1");
  }
  return FGB_OK;
}

}  // namespace
}  // namespace fgb

extern "C" {

int fgb_conduction_q_ti_f64(int num_faces, int nz, const double* z, double dt, const double* Qn,
                            const double* Qnp1, const double* T_in, double* T_out,
                            const double* ti, long long ti_ld, const double* rhoc,
                            const double* emiss, const double* Fgeotherm, unsigned* flags,
                            void* stream) {
  int st = fgb::check_cond(num_faces, nz);
  if (st) return st;
  if (ti_ld != 0 && ti_ld != nz + 1) {
    fgb::set_error("ti_ld must be 0 (shared profile) or nz + 1 (per facet), got %lld", ti_ld);
    return FGB_BAD_ARG;
  }
  if (num_faces == 0) return FGB_OK;
  cudaStream_t s = fgb::as_stream(stream);
  const unsigned grid = (unsigned)((num_faces + 127) / 128);
  if (nz <= 47) {
    fgb::conduction_q_facet_kernel<47><<<grid, 128, 0, s>>>(num_faces, nz, z, dt, Qn, Qnp1, T_in,
                                                            T_out, ti, ti_ld, rhoc, emiss,
                                                            Fgeotherm, flags);
  } else {
    fgb::conduction_q_facet_kernel<127><<<grid, 128, 0, s>>>(num_faces, nz, z, dt, Qn, Qnp1,
                                                             T_in, T_out, ti, ti_ld, rhoc, emiss,
                                                             Fgeotherm, flags);
  }
  FGB_LAUNCH_CHECK("conduction_q_facet_kernel");
  return FGB_OK;
}

int fgb_conduction_q_adjoint_f64(int num_faces, int nz, const double* z, double dt,
                                 const double* Qn, const double* Qnp1, const double* T_in,
                                 const double* ti, long long ti_ld, const double* rhoc,
                                 const double* emiss, const double* Fgeotherm,
                                 const double* gT_out, double* gT_in, double* gQn,
                                 double* gQnp1, double* gemiss, double* gti, unsigned* flags,
                                 void* stream) {
  int st = fgb::check_cond(num_faces, nz);
  if (st) return st;
  if (ti_ld != 0 && ti_ld != nz + 1) {
    fgb::set_error("ti_ld must be 0 (shared profile) or nz + 1 (per facet), got %lld", ti_ld);
    return FGB_BAD_ARG;
  }
  if (num_faces == 0) return FGB_OK;
  cudaStream_t s = fgb::as_stream(stream);
  const unsigned grid = (unsigned)((num_faces + 127) / 128);
  if (nz <= 47) {
    fgb::conduction_q_adjoint_kernel<47><<<grid, 128, 0, s>>>(
        num_faces, nz, z, dt, Qn, Qnp1, T_in, ti, ti_ld, rhoc, emiss, Fgeotherm, gT_out, gT_in,
        gQn, gQnp1, gemiss, gti, flags);
  } else {
    fgb::conduction_q_adjoint_kernel<127><<<grid, 128, 0, s>>>(
        num_faces, nz, z, dt, Qn, Qnp1, T_in, ti, ti_ld, rhoc, emiss, Fgeotherm, gT_out, gT_in,
        gQn, gQnp1, gemiss, gti, flags);
  }
  FGB_LAUNCH_CHECK("conduction_q_adjoint_kernel");
  return FGB_OK;
}

int fgb_rmatvec_f64(const fgb_op_desc* d, const double* panel, const double* vpanel,
                    const double* y, double* work, unsigned* flags, void* stream) {
  return fgb::rmatvec<double>(d, panel, vpanel, y, work, flags, fgb::as_stream(stream));
}

int fgb_rmatvec_f32_f64(const fgb_op_desc* d, const float* panel, const float* vpanel,
                        const double* y, double* work, unsigned* flags, void* stream) {
  return fgb::rmatvec<float>(d, panel, vpanel, y, work, flags, fgb::as_stream(stream));
}

}  // extern "C"
