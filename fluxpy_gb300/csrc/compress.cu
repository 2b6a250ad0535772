// Batched adaptive cross approximation (ACA) of admissible form-factor
// blocks, replacing the reference's assemble-then-ARPACK compression
// (src/flux/compressed_form_factors.py:345-405 -> src/flux/linalg.py:8-51):
// the reference evaluates every entry of a block and truncates its SVD at
// sigma_i / sigma_0 <= tol; here only O(k (m + n)) entries of an admissible
// block are evaluated (each with its visibility ray), and the rank-k factors
// U V^T are built by partially pivoted ACA (Bebendorf, "Approximation of
// boundary element matrices", Numer. Math. 86, 2000) with the Frobenius
// stopping test |u_k| |v_k| <= tol |S_k|_F.  Because visibility makes blocks
// patchy (a few rows or columns may carry all of a block's mass), the test
// is confirmed by a Monte Carlo estimate of the residual's Frobenius norm
// from `nsample` random entries, (m n / S) sum R_ij^2 <= tol^2 |S_k|_F^2; if
// it fails, the row of the worst sample becomes the next pivot row.
// A block whose rank would reach its cap (storage no smaller than half the
// dense block, or rmax) is reported as failed (rank -1) and is subdivided by
// the host.  Two more outcomes guard against visibility-made sparsity:
//  * a sampled block accepted with k > 0 terms whose nonzeros, estimated
//    from the random samples, would take no more bytes stored exactly than
//    its factors (2 nnz <= k (m + n): the reference's choice between a CSR
//    and an SVD block by bytes) is reported as failed too: such blocks are
//    scattered visible pairs that partial pivoting misses, and their
//    children are approximated again (small ones with every entry known);
//  * a block whose every entry is known is reported as "store exactly"
//    (rank -3) when the near-field panel rows its nonzeros need (one
//    64-weight row per 64-row tile and column that holds a nonzero) take no
//    more weights than the factors.
// A sampled block is accepted as zero only after kZeroRounds rounds of
// samples without a nonzero entry.
//
// One CTA per block (persistent CTAs take blocks from a queue, largest
// first).  The residual row/column, U and V live in a per-CTA FP32 scratch
// slice of global memory (L2-resident for the small blocks that dominate);
// norms and Gram products are accumulated in FP64.  Finished factors are
// copied to a pool with a 64-bit bump allocator: block b gets U^T (k x m)
// followed by V^T (k x n), row l contiguous.
#include "common.cuh"
#include "ffentry.cuh"

#include <climits>
#include <mutex>

#include <cuda.h>  // CUcontext and the driver types, resolved at run time

namespace fgb {
BvhView view_of(const void* handle);

namespace {

constexpr int kAcaThreads = 256;
// sampling rounds that must all find nothing before a block is zero
constexpr int kZeroRounds = 4;

struct AcaArgs {
  BvhView bvh;
  const long long* perm;
  long long nblocks;
  const int* r0;
  const int* m;
  const int* c0;
  const int* n;
  int sem;
  float tol;
  int rmax;
  int nsample;
  long long exact_max;
  float* dense_scratch;
  float* scratch;
  long long per_cta;
  long long mmax, nmax;
  float* pool;
  long long pool_capacity;
  unsigned long long* pool_used;
  int* rank_out;
  long long* off_out;
  int* queue;
  unsigned* flags;
};

template <class R>
struct EntryCtx {
  const R* P;
  const R* N;
  const R* A;
  R eps;
};

template <class R>
__device__ __forceinline__ float entry(const AcaArgs& a, const EntryCtx<R>& e, long long fi,
                                       long long fj, bool* of) {
  bool kept = false, ne = false;
  R v = ff_entry<R>(a.bvh, e.P, e.N, e.A, fi, fj, e.eps, a.sem, &kept, &ne, of);
  return (float)v;
}

// Block-wide reductions (kAcaThreads threads).
__device__ __forceinline__ double block_sum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x < 32) {
    t = threadIdx.x < (kAcaThreads / 32) ? sh[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (threadIdx.x == 0) sh[0] = t;
  }
  __syncthreads();
  t = sh[0];
  __syncthreads();
  return t;
}

// argmax of |v| over candidates (idx >= 0); returns (value, index).
__device__ __forceinline__ void block_argmax(float v, int idx, float* shv, int* shi, float* out_v,
                                             int* out_i) {
  float a = idx >= 0 ? fabsf(v) : -1.0f;
  for (int o = 16; o > 0; o >>= 1) {
    float a2 = __shfl_xor_sync(0xffffffffu, a, o);
    int i2 = __shfl_xor_sync(0xffffffffu, idx, o);
    float v2 = __shfl_xor_sync(0xffffffffu, v, o);
    if (a2 > a || (a2 == a && i2 >= 0 && (idx < 0 || i2 < idx))) { a = a2; idx = i2; v = v2; }
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) { shv[w] = a; shi[w] = idx; shv[8 + w] = v; }
  __syncthreads();
  if (threadIdx.x < 32) {
    float aa = threadIdx.x < 8 ? shv[threadIdx.x] : -1.0f;
    int ii = threadIdx.x < 8 ? shi[threadIdx.x] : -1;
    float vv = threadIdx.x < 8 ? shv[8 + threadIdx.x] : 0.0f;
    for (int o = 16; o > 0; o >>= 1) {
      float a2 = __shfl_xor_sync(0xffffffffu, aa, o);
      int i2 = __shfl_xor_sync(0xffffffffu, ii, o);
      float v2 = __shfl_xor_sync(0xffffffffu, vv, o);
      if (a2 > aa || (a2 == aa && i2 >= 0 && (ii < 0 || i2 < ii))) { aa = a2; ii = i2; vv = v2; }
    }
    if (threadIdx.x == 0) { shv[16] = vv; shi[16] = ii; }
  }
  __syncthreads();
  *out_v = shv[16];
  *out_i = shi[16];
  __syncthreads();
}

template <class R>
__global__ void __launch_bounds__(kAcaThreads)
aca_kernel(AcaArgs a, EntryCtx<R> e) {
  __shared__ double sh_d[32];
  __shared__ float sh_v[32];
  __shared__ int sh_i[32];
  __shared__ int s_block;
  __shared__ double s_dot[2][128];
  const int tid = threadIdx.x;
  float* U = a.scratch + (long long)blockIdx.x * a.per_cta;  // [rmax][mmax]
  float* V = U + (long long)a.rmax * a.mmax;                  // [rmax][nmax]
  float* rowbuf = V + (long long)a.rmax * a.nmax;             // [nmax]
  float* used_r = rowbuf + a.nmax;                            // [mmax]
  float* used_c = used_r + a.mmax;                            // [nmax]
  bool overflow = false;

  while (true) {
    if (tid == 0) s_block = atomicAdd(a.queue, 1);
    __syncthreads();
    const long long b = s_block;
    __syncthreads();
    if (b >= a.nblocks) break;
    const int m = a.m[b], n = a.n[b];
    const long long r0 = a.r0[b], c0 = a.c0[b];
    const long long* prow = a.perm + r0;
    const long long* pcol = a.perm + c0;
    for (int i = tid; i < m; i += kAcaThreads) used_r[i] = 0.f;
    for (int j = tid; j < n; j += kAcaThreads) used_c[j] = 0.f;
    long long cap = ((long long)m * n) / (2LL * (m + n));
    int kmax = (int)min((long long)a.rmax, max(cap, 1LL));
    int k = 0;
    double normS2 = 0.0;
    const unsigned bseed = 0x9e3779b9u ^ (unsigned)(b * 2654435761ull);
    int istar = m / 2;
    bool failed = false;
    bool store_exact = false;
    int rounds = 0;
    bool verify = false;
    double hits = 0.0, samples = 0.0;   // random samples and their nonzero entries
    const int max_rounds = 4 * a.rmax + 8;
    __syncthreads();
    if ((long long)m * n <= a.exact_max) {
      // ---- small block: evaluate every entry once, then cross approximation
      // with full pivoting on the exact residual (exact Frobenius control)
      float* Rm = a.dense_scratch + (long long)blockIdx.x * a.exact_max;
      const long long mn = (long long)m * n;
      double a2 = 0.0;
      float pv = 0.f;
      int pq = -1;
      for (long long q = tid; q < mn; q += kAcaThreads) {
        const int i = (int)(q / n), j = (int)(q % n);
        const float val = entry<R>(a, e, prow[i], pcol[j], &overflow);
        Rm[q] = val;
        a2 += (double)val * val;
        if (pq < 0 || fabsf(val) > fabsf(pv)) { pv = val; pq = (int)q; }
      }
      a2 = block_sum(a2, sh_d);
      // near-field panel rows the exact block would need: (64-row tile,
      // column) pairs that hold a nonzero
      double prows = 0.0;
      {
        const long long t_first = r0 >> 6;
        const int ntile = (int)(((r0 + m - 1) >> 6) - t_first + 1);
        for (long long q = tid; q < (long long)ntile * n; q += kAcaThreads) {
          const int t = (int)(q / n), j = (int)(q % n);
          const long long i0 = max(0LL, ((t_first + t) << 6) - r0);
          const long long i1 = min((long long)m, ((t_first + t + 1) << 6) - r0);
          bool any = false;
          for (long long i = i0; i < i1 && !any; i++) any = Rm[i * n + j] != 0.f;
          prows += any ? 1.0 : 0.0;
        }
      }
      prows = block_sum(prows, sh_d);
      double res2 = a2;
      while (res2 > (double)a.tol * a.tol * a2) {
        float piv;
        int qs;
        block_argmax(pv, pq, sh_v, sh_i, &piv, &qs);
        if (qs < 0 || piv == 0.0f) break;
        if (k >= kmax) { failed = true; break; }
        const int is = qs / n, js = qs % n;
        const float inv = 1.0f / piv;
        for (int i = tid; i < m; i += kAcaThreads) U[(long long)k * a.mmax + i] = Rm[(long long)i * n + js];
        for (int j = tid; j < n; j += kAcaThreads) V[(long long)k * a.nmax + j] = Rm[(long long)is * n + j] * inv;
        __syncthreads();
        double r2 = 0.0;
        pv = 0.f;
        pq = -1;
        for (long long q = tid; q < mn; q += kAcaThreads) {
          const int i = (int)(q / n), j = (int)(q % n);
          const float val = Rm[q] - U[(long long)k * a.mmax + i] * V[(long long)k * a.nmax + j];
          Rm[q] = val;
          r2 += (double)val * val;
          if (pq < 0 || fabsf(val) > fabsf(pv)) { pv = val; pq = (int)q; }
        }
        res2 = block_sum(r2, sh_d);
        k++;
      }
      if (!failed && k > 0 && 64.0 * prows <= (double)k * (double)(m + n)) store_exact = true;
    } else
    while (true) {
      if (!verify) {
        // ---- partially pivoted row step at istar
        const long long fi = prow[istar];
        float lmax_v = 0.f;
        int lmax_i = -1;
        double rr = 0.0;
        for (int j = tid; j < n; j += kAcaThreads) {
          float val = entry<R>(a, e, fi, pcol[j], &overflow);
          for (int l = 0; l < k; l++) val -= U[(long long)l * a.mmax + istar] * V[(long long)l * a.nmax + j];
          rowbuf[j] = val;
          rr += (double)val * val;
          if (lmax_i < 0 || fabsf(val) > fabsf(lmax_v)) { lmax_v = val; lmax_i = j; }
        }
        if (tid == 0) used_r[istar] = 1.f;
        float piv;
        int jstar;
        block_argmax(lmax_v, lmax_i, sh_v, sh_i, &piv, &jstar);
        rr = block_sum(rr, sh_d);
        // The pivot is the row's largest residual over all columns, so the
        // new v has |v| <= 1.  A row whose largest residual sits on an
        // already used column holds FP32 rounding noise only (the residual
        // of pivot columns is zero up to rounding): treat it as negligible,
        // as any row whose residual norm would add less than (tol/4)^2 of
        // |S|_F^2 when repeated over all m rows.
        const bool negligible = jstar < 0 || piv == 0.0f || used_c[jstar] != 0.f ||
                                (normS2 > 0.0 && (double)m * rr <= 0.0625 * (double)a.tol * a.tol * normS2);
        if (negligible) { verify = true; continue; }
        if (k >= kmax) { failed = true; break; }
        // new term: v = row / pivot, u = residual column jstar
        const float inv = 1.0f / piv;
        for (int j = tid; j < n; j += kAcaThreads) V[(long long)k * a.nmax + j] = rowbuf[j] * inv;
        __syncthreads();
        const long long fj = pcol[jstar];
        double uu = 0.0;
        float umax_v = 0.f;
        int umax_i = -1;
        for (int i = tid; i < m; i += kAcaThreads) {
          float val = entry<R>(a, e, prow[i], fj, &overflow);
          for (int l = 0; l < k; l++) val -= V[(long long)l * a.nmax + jstar] * U[(long long)l * a.mmax + i];
          U[(long long)k * a.mmax + i] = val;
          uu += (double)val * val;
          if (used_r[i] == 0.f && (umax_i < 0 || fabsf(val) > fabsf(umax_v))) { umax_v = val; umax_i = i; }
        }
        if (tid == 0) used_c[jstar] = 1.f;
        double vv = 0.0;
        for (int j = tid; j < n; j += kAcaThreads) {
          float v = V[(long long)k * a.nmax + j];
          vv += (double)v * v;
        }
        uu = block_sum(uu, sh_d);
        vv = block_sum(vv, sh_d);
        // cross terms 2 sum_l (u.U_l)(v.V_l), one warp per l
        const int w = tid >> 5, ln = tid & 31;
        for (int l = w; l < k; l += kAcaThreads / 32) {
          double du = 0.0, dv = 0.0;
          for (int i = ln; i < m; i += 32)
            du += (double)U[(long long)k * a.mmax + i] * U[(long long)l * a.mmax + i];
          for (int j = ln; j < n; j += 32)
            dv += (double)V[(long long)k * a.nmax + j] * V[(long long)l * a.nmax + j];
          for (int o = 16; o > 0; o >>= 1) {
            du += __shfl_xor_sync(0xffffffffu, du, o);
            dv += __shfl_xor_sync(0xffffffffu, dv, o);
          }
          if (ln == 0) { s_dot[0][l] = du; s_dot[1][l] = dv; }
        }
        __syncthreads();
        if (tid == 0) {
          double cross = 0.0;
          for (int l = 0; l < k; l++) cross += s_dot[0][l] * s_dot[1][l];
          sh_d[31] = cross;
        }
        __syncthreads();
        const double cross = sh_d[31];
        __syncthreads();
        normS2 += uu * vv + 2.0 * cross;
        if (normS2 < 0.0) normS2 = 0.0;
        k++;
        float nxt_v;
        int nxt_i;
        block_argmax(umax_v, umax_i, sh_v, sh_i, &nxt_v, &nxt_i);
        if (sqrt(uu * vv) <= (double)a.tol * sqrt(normS2) || nxt_i < 0) verify = true;
        else istar = nxt_i;
        continue;
      }
      // ---- verification: Monte Carlo estimate of |R|_F^2 from nsample random entries
      if (++rounds > max_rounds) { failed = true; break; }
      double rs = 0.0, nzr = 0.0;
      float wmax_v = 0.f;
      int wmax_i = -1;
      bool any_nz = false;
      for (int q = tid; q < a.nsample; q += kAcaThreads) {
        unsigned h = bseed ^ (unsigned)(rounds * 0x85ebca6bu) ^ (unsigned)(q * 0xc2b2ae35u);
        h ^= h >> 16; h *= 0x7feb352du; h ^= h >> 15; h *= 0x846ca68bu; h ^= h >> 16;
        const int i = (int)(h % (unsigned)m);
        unsigned h2 = h * 0x9e3779b1u + 0x7f4a7c15u;
        h2 ^= h2 >> 13; h2 *= 0x5bd1e995u; h2 ^= h2 >> 15;
        const int j = (int)(h2 % (unsigned)n);
        const float raw = entry<R>(a, e, prow[i], pcol[j], &overflow);
        float val = raw;
        for (int l = 0; l < k; l++) val -= U[(long long)l * a.mmax + i] * V[(long long)l * a.nmax + j];
        rs += (double)val * val;
        nzr += raw != 0.f ? 1.0 : 0.0;
        if (val != 0.f) any_nz = true;
        if (used_r[i] == 0.f && (wmax_i < 0 || fabsf(val) > fabsf(wmax_v))) { wmax_v = val; wmax_i = i; }
      }
      rs = block_sum(rs, sh_d);
      hits += block_sum(nzr, sh_d);
      samples += (double)a.nsample;
      const int nz = __syncthreads_or(any_nz);
      float wv;
      int wi;
      block_argmax(wmax_v, wmax_i, sh_v, sh_i, &wv, &wi);
      const double est = rs * ((double)m * (double)n / (double)a.nsample);
      const bool ok = (normS2 > 0.0) ? (est <= (double)a.tol * a.tol * normS2) : (nz == 0);
      // a zero block needs kZeroRounds empty rounds (fresh samples each)
      if (ok && normS2 == 0.0 && rounds < kZeroRounds) continue;
      if (ok) {
        // scattered visible pairs: cheaper stored exactly than as factors,
        // and what partial pivoting misses; approximate the children again
        if (k > 0 && 2.0 * (hits / samples) * (double)m * (double)n <= (double)k * (double)(m + n))
          failed = true;
        break;
      }
      if (wi < 0 || wv == 0.0f) {
        // the worst sample sits on an already used row: fall back to any unused row
        int cand = -1;
        for (int c = 0; c < m; c++)
          if (used_r[c] == 0.f) { cand = c; break; }
        __syncthreads();
        if (cand < 0) { failed = true; break; }
        istar = cand;
      } else {
        istar = wi;
      }
      verify = false;
    }
    __syncthreads();
    // factors must be finite (a degenerate pivot would show up here)
    {
      bool bad = false;
      for (int l = 0; l < k && !failed; l++) {
        for (int i = tid; i < m; i += kAcaThreads)
          if (!isfinite(U[(long long)l * a.mmax + i])) bad = true;
        for (int j = tid; j < n; j += kAcaThreads)
          if (!isfinite(V[(long long)l * a.nmax + j])) bad = true;
      }
      if (__syncthreads_or(bad)) failed = true;
    }
    if (failed || store_exact) {
      if (tid == 0) { a.rank_out[b] = failed ? -1 : -3; a.off_out[b] = -1; }
      continue;
    }
    // copy out U^T (k x m) then V^T (k x n)
    __shared__ unsigned long long s_off;
    if (tid == 0) {
      unsigned long long need = (unsigned long long)k * (unsigned long long)(m + n);
      unsigned long long off = need ? atomicAdd(a.pool_used, need) : 0ull;
      if (off + need > (unsigned long long)a.pool_capacity) {
        atomicOr(a.flags, kFlagRankCap);
        s_off = ~0ull;
      } else {
        s_off = off;
      }
    }
    __syncthreads();
    const unsigned long long off = s_off;
    if (off == ~0ull) {
      if (tid == 0) { a.rank_out[b] = -2; a.off_out[b] = -1; }
      continue;
    }
    float* dst = a.pool + off;
    for (int l = 0; l < k; l++)
      for (int i = tid; i < m; i += kAcaThreads) dst[(long long)l * m + i] = U[(long long)l * a.mmax + i];
    dst += (long long)k * m;
    for (int l = 0; l < k; l++)
      for (int j = tid; j < n; j += kAcaThreads) dst[(long long)l * n + j] = V[(long long)l * a.nmax + j];
    if (tid == 0) { a.rank_out[b] = k; a.off_out[b] = (long long)off; }
    __syncthreads();
  }
  if (overflow) atomicOr(a.flags, kFlagStackOverflow);
}

}  // namespace
}  // namespace fgb

extern "C" {

int fgb_aca_scratch_floats(int rmax, long long mmax, long long nmax, long long* per_cta) {
  // block sides are int in the kernel: bounding them also keeps the product
  // below 2^40 (no overflow)
  if (rmax < 1 || rmax > 128 || mmax < 1 || nmax < 1 || mmax > INT_MAX || nmax > INT_MAX) {
    fgb::set_error("bad ACA sizes (rmax in [1,128], block sides in [1, 2^31))");
    return FGB_BAD_ARG;
  }
  if (!per_cta) { fgb::set_error("null output"); return FGB_BAD_ARG; }
  *per_cta = (long long)rmax * (mmax + nmax) + 2 * (mmax + nmax);
  return FGB_OK;
}

}  // extern "C"

namespace fgb {
namespace {
// Scratch of fgb_aca_f64_static, the entry point for callers that cannot
// allocate device memory (their allocator owns the device, or they call
// from a region where cudaMalloc is not allowed): one file-scope device
// array per device (the module's static data), sized for small batches.
// In host code the array's name is not a device address: the address is
// looked up with cudaGetSymbolAddress by the first call on each device
// (before any stream capture), with that device current.
constexpr long long kAcaStaticFloats = 8LL << 20;   // 32 MiB
static __device__ __align__(256) float g_aca_static_scratch[kAcaStaticFloats];
static __device__ __align__(256) int g_aca_static_queue[64];

struct StaticAcaSlot {
  unsigned long long ctx_id = 0;   // context the addresses belong to
  float* scratch = nullptr;
  int* queue = nullptr;
};
std::mutex g_aca_static_mutex;
StaticAcaSlot g_aca_static_slots[64];

// The symbol addresses of the current device, looked up once per context:
// a context created after cudaDeviceReset loads the module again, possibly
// elsewhere, so the cached addresses are keyed by the context's unique id.
// The two driver calls are resolved through the runtime
// (cudaGetDriverEntryPoint), so the library does not link libcuda itself.
using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

int current_context_id(unsigned long long* id) {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPoint("cuCtxGetCurrent", &f, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<CtxGetCurrentFn>(f);
    f = nullptr;
    if (cudaGetDriverEntryPoint("cuCtxGetId", &f, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<CtxGetIdFn>(f);
  });
  CUcontext ctx = nullptr;
  if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx ||
      get_id(ctx, id) != CUDA_SUCCESS) {
    set_error("fgb_aca_f64_static: no current CUDA context");
    return FGB_CUDA_ERR;
  }
  return FGB_OK;
}

int static_aca_slot(StaticAcaSlot* out) {
  int dev = 0;
  FGB_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) { set_error("device index out of range"); return FGB_BAD_ARG; }
  // make the runtime's context current (a no-op when it already is)
  FGB_CUDA_TRY(cudaFree(nullptr));
  unsigned long long id = 0;
  int st = current_context_id(&id);
  if (st) return st;
  std::lock_guard<std::mutex> lock(g_aca_static_mutex);
  StaticAcaSlot& s = g_aca_static_slots[dev];
  if (!s.scratch || s.ctx_id != id) {
    void* p = nullptr;
    void* q = nullptr;
    FGB_CUDA_TRY(cudaGetSymbolAddress(&p, g_aca_static_scratch));
    FGB_CUDA_TRY(cudaGetSymbolAddress(&q, g_aca_static_queue));
    s.scratch = static_cast<float*>(p);
    s.queue = static_cast<int*>(q);
    s.ctx_id = id;
  }
  *out = s;
  return FGB_OK;
}
}  // namespace
}  // namespace fgb

extern "C" {

int fgb_aca_f64(const void* bvh, const double* P, const double* N, const double* A,
                const long long* perm, long long nblocks, const int* r0, const int* m,
                const int* c0, const int* n, long long mmax, long long nmax, double eps,
                int semantics, float tol, int rmax, int nsample, long long exact_max,
                float* dense_scratch, float* scratch, int num_ctas,
                float* pool, long long pool_capacity, unsigned long long* pool_used,
                int* rank_out, long long* off_out, int* queue, unsigned* flags, void* stream) {
  if (!bvh || nblocks < 0 || num_ctas < 1) { fgb::set_error("bad ACA arguments"); return FGB_BAD_ARG; }
  if (rmax < 1 || rmax > 128) { fgb::set_error("rmax must be in [1, 128]"); return FGB_BAD_ARG; }
  if (nblocks == 0) return FGB_OK;
  long long per_cta;
  int st = fgb_aca_scratch_floats(rmax, mmax, nmax, &per_cta);
  if (st) return st;
  fgb::AcaArgs a;
  a.bvh = fgb::view_of(bvh);
  a.perm = perm;
  a.nblocks = nblocks;
  a.r0 = r0; a.m = m; a.c0 = c0; a.n = n;
  a.sem = semantics;
  a.tol = tol;
  a.rmax = rmax;
  a.nsample = nsample < 32 ? 32 : nsample;
  a.exact_max = dense_scratch ? exact_max : 0;
  a.dense_scratch = dense_scratch;
  a.scratch = scratch;
  a.per_cta = per_cta;
  a.mmax = mmax; a.nmax = nmax;
  a.pool = pool;
  a.pool_capacity = pool_capacity;
  a.pool_used = pool_used;
  a.rank_out = rank_out;
  a.off_out = off_out;
  a.queue = queue;
  a.flags = flags;
  fgb::EntryCtx<double> e{P, N, A, eps};
  fgb::aca_kernel<double><<<num_ctas, fgb::kAcaThreads, 0, fgb::as_stream(stream)>>>(a, e);
  FGB_LAUNCH_CHECK("aca_kernel");
  return FGB_OK;
}

int fgb_aca_f64_static(const void* bvh, const double* P, const double* N, const double* A,
                       const long long* perm, long long nblocks, const int* r0, const int* m,
                       const int* c0, const int* n, long long mmax, long long nmax, double eps,
                       int semantics, float tol, int rmax, int nsample, long long exact_max,
                       int num_ctas, float* pool, long long pool_capacity,
                       unsigned long long* pool_used, int* rank_out, long long* off_out,
                       unsigned* flags, void* stream) {
  if (!bvh || nblocks < 0 || num_ctas < 1) { fgb::set_error("bad ACA arguments"); return FGB_BAD_ARG; }
  if (nblocks == 0) return FGB_OK;
  long long per_cta;
  int st = fgb_aca_scratch_floats(rmax, mmax, nmax, &per_cta);
  if (st) return st;
  if (exact_max < 0) exact_max = 0;
  // per CTA: the factor scratch slice, then (blocks with m n <= exact_max)
  // the dense block.  Each term is bounded before the sum and the division
  // replaces the product, so no size wraps around.
  const long long cap = fgb::kAcaStaticFloats;
  if (per_cta > cap || exact_max > cap || per_cta + exact_max > cap / num_ctas) {
    fgb::set_error("fgb_aca_f64_static: %d CTAs x (%lld + %lld) floats of scratch "
                   "(rmax %d, mmax %lld, nmax %lld, exact_max %lld) exceed the static scratch "
                   "of %lld floats: use fewer CTAs, smaller blocks or fgb_aca_f64",
                   num_ctas, per_cta, exact_max, rmax, mmax, nmax, exact_max, cap);
    return FGB_BAD_ARG;
  }
  fgb::StaticAcaSlot slot;
  if ((st = fgb::static_aca_slot(&slot))) return st;
  cudaStream_t s = fgb::as_stream(stream);
  // the work queue must start at zero for every call
  FGB_CUDA_TRY(cudaMemsetAsync(slot.queue, 0, sizeof(int), s));
  float* scratch = slot.scratch;
  float* dense = exact_max > 0 ? slot.scratch + (long long)num_ctas * per_cta : nullptr;
  return fgb_aca_f64(bvh, P, N, A, perm, nblocks, r0, m, c0, n, mmax, nmax, eps, semantics, tol,
                     rmax, nsample, exact_max, dense, scratch, num_ctas, pool, pool_capacity,
                     pool_used, rank_out, off_out, slot.queue, flags, stream);
}

}  // extern "C"
