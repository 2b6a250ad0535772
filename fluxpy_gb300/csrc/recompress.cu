// FP64 rank truncation of the low-rank factors (the reference's SVD
// truncation, src/flux/linalg.py:20-51 applied at
// src/flux/compressed_form_factors.py:388-405: keep sigma_i with
// sigma_i / sigma_0 > tol).
//
// A block is stored as U V^T with U (m x k), V (n x k) in FP32 (the pool
// holds U^T, k x m, then V^T, k x n, each row contiguous).  Its singular
// values are found without forming the block:
//   1. Gram matrices G_u = U^T U and G_v = V^T V in FP64 (FP32 products are
//      exact in FP64; sums in FP64);
//   2. G_u = W diag(lam) W^T by cyclic Jacobi (FP64, shared memory);
//      L = W diag(sqrt(lam)) is a square root, U = Q L^T with Q orthonormal
//      (an orthogonalisation of U equivalent to its QR factorisation);
//   3. S = L^T G_v L = C C^T for the core C = L^T V^T, whose singular values
//      are the block's: S = Y diag(sigma^2) Y^T by cyclic Jacobi again;
//   4. r = #{sigma_i > tol sigma_0}; the truncated block is U' V'^T with
//      U' = U W diag(lam^-1/2) Y_r diag(sigma_r)   (= Q Y_r Sigma_r, orthogonal
//      columns scaled by sigma) and V' = V L Y_r diag(1/sigma_r) (orthonormal),
//      applied to the FP32 factors with FP64 sums and stored in FP32.
// Eigenvalues of G_u below 1e-14 lam_max (directions U does not span to
// working precision) are dropped.  Singular values come out accurate to
// ~1e-8 sigma_0 (S is formed in FP64), far below any truncation tolerance
// the compression uses.
//
// One CTA per block, persistent CTAs taking blocks from a queue; two
// instantiations by the largest rank they hold (KM = 32 and 64), so small
// blocks run many CTAs per SM.  Blocks of rank 0 or 1 and of rank above 64
// are copied unchanged.
#include "common.cuh"

#include <algorithm>

namespace fgb {
namespace {

constexpr int kRcThreads = 256;
constexpr int kChunk = 32;            // factor positions staged per step
constexpr double kDropRel = 1e-14;    // eigenvalues of G_u dropped below this * max
constexpr int kMaxSweeps = 40;

struct RcArgs {
  const float* pool_in;
  const long long* off_in;
  const int* rank_in;
  const int* m;
  const int* n;
  long long nblocks;
  float tol;
  float* pool_out;
  long long capacity;
  unsigned long long* used;
  int* rank_out;
  long long* off_out;
  int* queue;
  unsigned* flags;
};

// Block-wide sum of doubles (kRcThreads threads).
__device__ __forceinline__ double rc_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  double t = 0.0;
  for (int i = 0; i < kRcThreads / 32; i++) t += red[i];
  __syncthreads();
  return t;
}

// G (kp x kp, leading dimension KM) = X X^T for X = rows 0..k-1 of a k x len
// FP32 matrix (row stride len), FP64 sums; rows/cols k..kp-1 set to zero.
template <int KM>
__device__ void gram(const float* X, int k, int kp, long long len, double* G, float* stage) {
  constexpr int kPairsPerThread = (KM * (KM + 1) / 2 + kRcThreads - 1) / kRcThreads;
  const int tid = threadIdx.x;
  const int npairs = k * (k + 1) / 2;
  int pi[kPairsPerThread], pj[kPairsPerThread];
  double acc[kPairsPerThread];
#pragma unroll
  for (int u = 0; u < kPairsPerThread; u++) {
    const int e = tid + u * kRcThreads;
    int i = 0, j = 0;
    if (e < npairs) {
      // row i holds pairs (i, i..k-1): start index i k - i (i - 1) / 2
      int r = 0, base = 0;
      while (base + (k - r) <= e) { base += k - r; r++; }
      i = r;
      j = r + (e - base);
    }
    pi[u] = i;
    pj[u] = e < npairs ? j : -1;
    acc[u] = 0.0;
  }
  for (long long p0 = 0; p0 < len; p0 += kChunk) {
    const int w = (int)min((long long)kChunk, len - p0);
    __syncthreads();
    for (int q = tid; q < k * kChunk; q += kRcThreads) {
      const int i = q / kChunk, pp = q % kChunk;
      stage[i * (kChunk + 1) + pp] = pp < w ? X[(long long)i * len + p0 + pp] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < kPairsPerThread; u++) {
      if (pj[u] < 0) continue;
      const float* a = stage + pi[u] * (kChunk + 1);
      const float* b = stage + pj[u] * (kChunk + 1);
      double s = 0.0;
#pragma unroll 8
      for (int pp = 0; pp < kChunk; pp++) s += (double)a[pp] * (double)b[pp];
      acc[u] += s;
    }
  }
  __syncthreads();
  for (int q = tid; q < kp * kp; q += kRcThreads) G[(q / kp) * KM + q % kp] = 0.0;
  __syncthreads();
#pragma unroll
  for (int u = 0; u < kPairsPerThread; u++) {
    if (pj[u] < 0) continue;
    G[pi[u] * KM + pj[u]] = acc[u];
    G[pj[u] * KM + pi[u]] = acc[u];
  }
  __syncthreads();
}

// Cyclic Jacobi eigen-decomposition of the symmetric kp x kp matrix A (kp
// even, leading dimension KM) in place: on return A is diagonal to working
// precision (the eigenvalues) and V holds the eigenvectors as columns.
// Each round applies kp/2 disjoint rotations (round-robin pairing), rows
// then columns.  Returns false if it did not converge in kMaxSweeps.
template <int KM>
__device__ bool jacobi_eigh(double* A, double* V, int kp, double* rot, double* red) {
  const int tid = threadIdx.x;
  const int half = kp / 2;
  for (int q = tid; q < kp * kp; q += kRcThreads) {
    const int i = q / kp, j = q % kp;
    V[i * KM + j] = i == j ? 1.0 : 0.0;
  }
  __syncthreads();
  bool converged = false;
  for (int sweep = 0; sweep < kMaxSweeps; sweep++) {
    double off = 0.0, dg = 0.0;
    for (int q = tid; q < kp * kp; q += kRcThreads) {
      const int i = q / kp, j = q % kp;
      const double v = A[i * KM + j];
      if (i == j) dg += v * v; else off += v * v;
    }
    off = rc_sum(off, red);
    dg = rc_sum(dg, red);
    if (off <= 1e-30 * dg || off == 0.0) { converged = true; break; }
    for (int t = 0; t < kp - 1; t++) {
      if (tid < half) {
        auto pos = [&](int j) { return j == 0 ? 0 : 1 + (j - 1 + t) % (kp - 1); };
        int p = pos(tid), q = pos(kp - 1 - tid);
        if (p > q) { const int x = p; p = q; q = x; }
        const double app = A[p * KM + p], aqq = A[q * KM + q], apq = A[p * KM + q];
        double c = 1.0, s = 0.0;
        if (apq != 0.0 && fabs(apq) > 1e-300) {
          const double tau = (aqq - app) / (2.0 * apq);
          const double tt = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + hypot(1.0, tau));
          c = 1.0 / sqrt(1.0 + tt * tt);
          s = tt * c;
        }
        rot[4 * tid + 0] = (double)p;
        rot[4 * tid + 1] = (double)q;
        rot[4 * tid + 2] = c;
        rot[4 * tid + 3] = s;
      }
      __syncthreads();
      // rows p, q  <-  J^T A
      for (int e = tid; e < half * kp; e += kRcThreads) {
        const int r = e / kp, j = e % kp;
        const int p = (int)rot[4 * r], q = (int)rot[4 * r + 1];
        const double c = rot[4 * r + 2], s = rot[4 * r + 3];
        const double ap = A[p * KM + j], aq = A[q * KM + j];
        A[p * KM + j] = c * ap - s * aq;
        A[q * KM + j] = s * ap + c * aq;
      }
      __syncthreads();
      // columns p, q  <-  A J, and V J
      for (int e = tid; e < half * kp; e += kRcThreads) {
        const int r = e / kp, i = e % kp;
        const int p = (int)rot[4 * r], q = (int)rot[4 * r + 1];
        const double c = rot[4 * r + 2], s = rot[4 * r + 3];
        const double ap = A[i * KM + p], aq = A[i * KM + q];
        A[i * KM + p] = c * ap - s * aq;
        A[i * KM + q] = s * ap + c * aq;
        const double vp = V[i * KM + p], vq = V[i * KM + q];
        V[i * KM + p] = c * vp - s * vq;
        V[i * KM + q] = s * vp + c * vq;
      }
      __syncthreads();
    }
  }
  return converged;
}

// out (r x len, FP32, row stride len) = T^T X for X = k x len FP32 (row
// stride len) and T (k x r, leading dimension KM) in FP64.
template <int KM>
__device__ void apply_transform(const float* X, int k, long long len, const double* T, int r,
                                float* out, float* stage) {
  const int tid = threadIdx.x;
  for (long long p0 = 0; p0 < len; p0 += kChunk) {
    const int w = (int)min((long long)kChunk, len - p0);
    __syncthreads();
    for (int q = tid; q < k * kChunk; q += kRcThreads) {
      const int i = q / kChunk, pp = q % kChunk;
      stage[i * (kChunk + 1) + pp] = pp < w ? X[(long long)i * len + p0 + pp] : 0.f;
    }
    __syncthreads();
    for (int q = tid; q < r * kChunk; q += kRcThreads) {
      const int l = q / kChunk, pp = q % kChunk;
      if (pp >= w) continue;
      double s = 0.0;
      for (int i = 0; i < k; i++) s += T[i * KM + l] * (double)stage[i * (kChunk + 1) + pp];
      out[(long long)l * len + p0 + pp] = (float)s;
    }
  }
  __syncthreads();
}

template <int KM>
__global__ void __launch_bounds__(kRcThreads)
recompress_kernel(RcArgs a, int k_lo, int k_hi, int queue_slot) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* G = reinterpret_cast<double*>(smem_raw);   // G_u, then Y (eigenvectors of S)
  double* W = G + KM * KM;                           // eigenvectors of G_u, then T_v
  double* H = W + KM * KM;                           // G_v, then S, then T_u
  double* L = H + KM * KM;                           // L = W sqrt(lam)
  double* lam = L + KM * KM;                         // KM
  double* sig2 = lam + KM;                           // KM
  double* rot = sig2 + KM;                           // 4 * KM / 2
  double* red = rot + 2 * KM;                        // kRcThreads / 32
  int* ord = reinterpret_cast<int*>(red + kRcThreads / 32);   // KM
  float* stage = reinterpret_cast<float*>(ord + KM);          // KM * (kChunk + 1)
  __shared__ long long s_blk;
  __shared__ unsigned long long s_off;
  __shared__ int s_r;
  const int tid = threadIdx.x;

  while (true) {
    if (tid == 0) s_blk = atomicAdd(a.queue + queue_slot, 1);
    __syncthreads();
    const long long b = s_blk;
    __syncthreads();
    if (b >= a.nblocks) break;
    const int k = a.rank_in[b];
    const bool copy_through = (k <= 1 || k > 64);
    // the small instantiation also copies the blocks nobody truncates
    if (copy_through ? (KM != 32) : (k < k_lo || k > k_hi)) continue;
    const long long m = a.m[b], n = a.n[b];
    const float* Ut = a.pool_in + a.off_in[b];
    const float* Vt = Ut + (long long)k * m;
    if (k <= 0) {
      // zero blocks stay zero; failure codes pass through
      if (tid == 0) { a.rank_out[b] = k; a.off_out[b] = k == 0 ? a.off_in[b] : -1; }
      continue;
    }
    if (copy_through) {
      if (tid == 0) {
        const unsigned long long need = (unsigned long long)k * (unsigned long long)(m + n);
        const unsigned long long off = atomicAdd(a.used, need);
        s_off = off + need > (unsigned long long)a.capacity ? ~0ull : off;
      }
      __syncthreads();
      const unsigned long long off = s_off;
      if (off == ~0ull) {
        if (tid == 0) { atomicOr(a.flags, kFlagRankCap); a.rank_out[b] = -2; a.off_out[b] = -1; }
        continue;
      }
      const long long total = (long long)k * (m + n);
      for (long long q = tid; q < total; q += kRcThreads) a.pool_out[off + q] = Ut[q];
      if (tid == 0) { a.rank_out[b] = k; a.off_out[b] = (long long)off; }
      if (k > 64 && tid == 0) atomicOr(a.flags, kFlagIndexRange);
      continue;
    }
    const int kp = k + (k & 1);
    // 1. Gram matrices (FP64)
    gram<KM>(Ut, k, kp, m, G, stage);
    gram<KM>(Vt, k, kp, n, H, stage);
    // 2. G_u = W diag(lam) W^T
    const bool ok1 = jacobi_eigh<KM>(G, W, kp, rot, red);
    for (int i = tid; i < kp; i += kRcThreads) lam[i] = G[i * KM + i];
    __syncthreads();
    double lmax = 0.0;
    for (int i = 0; i < kp; i++) lmax = fmax(lmax, lam[i]);
    // L = W diag(sqrt(lam)), dropped directions zero
    for (int q = tid; q < kp * kp; q += kRcThreads) {
      const int i = q / kp, j = q % kp;
      const double l = lam[j];
      L[i * KM + j] = l > kDropRel * lmax ? W[i * KM + j] * sqrt(l) : 0.0;
    }
    __syncthreads();
    // 3. S = L^T G_v L: M = G_v L into G, then S = L^T M into H
    for (int q = tid; q < kp * kp; q += kRcThreads) {
      const int i = q / kp, j = q % kp;
      double s = 0.0;
      for (int t = 0; t < kp; t++) s += H[i * KM + t] * L[t * KM + j];
      G[i * KM + j] = s;
    }
    __syncthreads();
    for (int q = tid; q < kp * kp; q += kRcThreads) {
      const int i = q / kp, j = q % kp;
      double s = 0.0;
      for (int t = 0; t < kp; t++) s += L[t * KM + i] * G[t * KM + j];
      H[i * KM + j] = s;
    }
    __syncthreads();
    // symmetrise (rounding) before the second decomposition
    for (int q = tid; q < kp * kp; q += kRcThreads) {
      const int i = q / kp, j = q % kp;
      if (i < j) {
        const double v = 0.5 * (H[i * KM + j] + H[j * KM + i]);
        H[i * KM + j] = v;
        H[j * KM + i] = v;
      }
    }
    __syncthreads();
    const bool ok2 = jacobi_eigh<KM>(H, G, kp, rot, red);   // Y in G
    for (int i = tid; i < kp; i += kRcThreads) sig2[i] = fmax(H[i * KM + i], 0.0);
    __syncthreads();
    // descending order of sigma^2 (ties by index)
    for (int i = tid; i < kp; i += kRcThreads) {
      int rk = 0;
      for (int j = 0; j < kp; j++)
        rk += (sig2[j] > sig2[i]) || (sig2[j] == sig2[i] && j < i);
      ord[rk] = i;
    }
    __syncthreads();
    // 4. truncation rank
    if (tid == 0) {
      const double s0 = sqrt(sig2[ord[0]]);
      int r = 0;
      if (s0 > 0.0) {
        const double cut = (double)a.tol * s0;
        while (r < k && sqrt(sig2[ord[r]]) > cut) r++;
      }
      s_r = r;
      if (!(ok1 && ok2)) atomicOr(a.flags, kFlagNoConverge);
    }
    __syncthreads();
    const int r = s_r;
    // T_u = W diag(lam^-1/2) Y_r diag(sigma_r) into H (S no longer needed)
    // T_v = L Y_r diag(1/sigma_r) into W (after T_u, which still reads W)
    for (int q = tid; q < kp * r; q += kRcThreads) {
      const int i = q / r, l = q % r;
      const int c = ord[l];
      const double sg = sqrt(sig2[c]);
      double s = 0.0;
      for (int j = 0; j < kp; j++) {
        const double lj = lam[j];
        if (lj > kDropRel * lmax) s += W[i * KM + j] * G[j * KM + c] / sqrt(lj);
      }
      H[i * KM + l] = s * sg;
    }
    __syncthreads();
    for (int q = tid; q < kp * r; q += kRcThreads) {
      const int i = q / r, l = q % r;
      const int c = ord[l];
      const double sg = sqrt(sig2[c]);
      double s = 0.0;
      for (int j = 0; j < kp; j++) s += L[i * KM + j] * G[j * KM + c];
      W[i * KM + l] = s / sg;
    }
    __syncthreads();
    // outputs: U'^T (r x m) then V'^T (r x n)
    if (tid == 0) {
      const unsigned long long need = (unsigned long long)r * (unsigned long long)(m + n);
      const unsigned long long off = need ? atomicAdd(a.used, need) : 0ull;
      s_off = off + need > (unsigned long long)a.capacity ? ~0ull : off;
    }
    __syncthreads();
    const unsigned long long off = s_off;
    if (off == ~0ull) {
      if (tid == 0) { atomicOr(a.flags, kFlagRankCap); a.rank_out[b] = -2; a.off_out[b] = -1; }
      continue;
    }
    apply_transform<KM>(Ut, k, m, H, r, a.pool_out + off, stage);
    apply_transform<KM>(Vt, k, n, W, r, a.pool_out + off + (unsigned long long)r * m, stage);
    if (tid == 0) { a.rank_out[b] = r; a.off_out[b] = (long long)off; }
    __syncthreads();
  }
}

template <int KM>
constexpr size_t rc_smem() {
  return sizeof(double) * (4 * KM * KM + 2 * KM + 2 * KM + kRcThreads / 32) + sizeof(int) * KM +
         sizeof(float) * KM * (kChunk + 1);
}

}  // namespace
}  // namespace fgb

extern "C" {

int fgb_recompress_f32(const float* pool_in, const long long* off_in, const int* rank_in,
                       const int* m, const int* n, long long nblocks, float tol, float* pool_out,
                       long long pool_capacity, unsigned long long* pool_used, int* rank_out,
                       long long* off_out, int* queue, unsigned* flags, void* stream) {
  if (nblocks < 0 || !(tol >= 0.0f) || pool_capacity < 0) {
    fgb::set_error("bad recompression arguments");
    return FGB_BAD_ARG;
  }
  if (nblocks == 0) return FGB_OK;
  if (!pool_in || !off_in || !rank_in || !m || !n || !pool_out || !pool_used || !rank_out ||
      !off_out || !queue || !flags) {
    fgb::set_error("fgb_recompress_f32: null pointer");
    return FGB_BAD_ARG;
  }
  fgb::RcArgs a{pool_in, off_in, rank_in, m, n, nblocks, tol, pool_out, pool_capacity,
                pool_used, rank_out, off_out, queue, flags};
  cudaStream_t s = fgb::as_stream(stream);
  constexpr size_t sm32 = fgb::rc_smem<32>();
  constexpr size_t sm64 = fgb::rc_smem<64>();
  static bool attr_set = false;
  if (!attr_set) {
    FGB_CUDA_TRY(cudaFuncSetAttribute(fgb::recompress_kernel<64>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm64));
    FGB_CUDA_TRY(cudaFuncSetAttribute(fgb::recompress_kernel<32>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm32));
    attr_set = true;
  }
  const unsigned g32 = (unsigned)std::min<long long>(nblocks, (long long)fgb::kNumSMs * 6);
  const unsigned g64 = (unsigned)std::min<long long>(nblocks, (long long)fgb::kNumSMs);
  fgb::recompress_kernel<64><<<g64, fgb::kRcThreads, sm64, s>>>(a, 33, 64, 0);
  FGB_LAUNCH_CHECK("recompress_kernel<64>");
  fgb::recompress_kernel<32><<<g32, fgb::kRcThreads, sm32, s>>>(a, 2, 32, 1);
  FGB_LAUNCH_CHECK("recompress_kernel<32>");
  return FGB_OK;
}

}  // extern "C"
