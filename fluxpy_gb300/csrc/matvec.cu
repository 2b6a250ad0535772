// Block matvec of the compressed form-factor operator.
//
// Replaces the recursive Python matvec of CompressedFormFactorMatrix
// (src/flux/compressed_form_factors.py:805 -> FormFactorBlockMatrix._matmat
// :407-414 -> leaf blocks: dense :175, CSR :193, SVD :247-251).
//
// Layout (built by the host, all in HBM; "permuted" = cluster order, where
// every block's rows and columns are contiguous ranges):
//   block b: rows [r0, r0+m), cols [c0, c0+n), "inner size" k
//     LR (rank-k factors):  W = U^T (k x m) at wpool + woff, Vt (k x n) at
//                           vpool + voff, Z rows [zoff, zoff+k)
//     DENSE (exact leaf):   W = D^T (n x m, i.e. column j of D contiguous),
//                           k = n, no Vt / Z
//   Phase A (LR blocks only): Z[zoff+l, :] = sum_j Vt[l, j] X[c0+j, :],
//     over work items (block, j0, j1) so that long blocks are split; items
//     that do not own their whole block accumulate with atomics.
//   Phase B: row tiles of kTileRows rows; tile t lists the blocks that
//     overlap it.  Y[i, :] = sum_blocks sum_l W[l, i-r0] S[l, :] with
//     S = Z[zoff..] (LR) or X[c0..] (DENSE).  Every Y row is written by one
//     CTA exactly once: no atomics, no separate zeroing.
// X and Y are (N x K) row-major, K = 1 for the single-RHS path.
#include "common.cuh"

#include <cuda_bf16.h>

namespace fgb {
namespace {

constexpr int kTileRows = 64;

struct OpView {
  const int* r0;
  const int* m;
  const int* c0;
  const int* n;
  const int* k;
  const long long* woff;
  const long long* voff;
  const long long* zoff;
  // phase A items
  const int* a_blk;
  const int* a_j0;
  const int* a_j1;
  const unsigned char* a_excl;  // 1: the item covers its whole block
  long long num_items;
  // phase B tiles
  const long long* t_ptr;
  const int* t_blk;
  long long num_tiles;
  long long N;
};

// ------------------------------------------------------------ K = 1 ----
template <class T, class V>
__global__ void phaseA_k1(OpView op, const T* __restrict__ vpool, const V* __restrict__ x,
                          V* __restrict__ z) {
  const int lane = threadIdx.x & 31;
  const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long it = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5; it < op.num_items;
       it += warps) {
    const int b = op.a_blk[it];
    const int j0 = op.a_j0[it], j1 = op.a_j1[it];
    const int n = op.n[b], k = op.k[b];
    const V* xb = x + op.c0[b];
    const T* vt = vpool + op.voff[b];
    V* zb = z + op.zoff[b];
    const bool excl = op.a_excl[it];
    for (int l = 0; l < k; l++) {
      const T* row = vt + (long long)l * n;
      V s = V(0);
      for (int j = j0 + lane; j < j1; j += 32) s += (V)row[j] * __ldg(xb + j);
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0) {
        if (excl) zb[l] = s;
        else atomicAdd(zb + l, s);
      }
    }
  }
}

// Phase B, K = 1: one CTA (8 warps) per 64-row tile.  Warp w takes blocks
// w, w+8, ... of the tile's list; lane L accumulates rows L and L+32 of the
// tile; the 8 warp partials are summed in a fixed order (deterministic).
constexpr int kB1Warps = 8;

template <class T, class V>
__global__ void __launch_bounds__(kB1Warps * 32)
phaseB_k1(OpView op, const T* __restrict__ wpool, const V* __restrict__ x,
          const V* __restrict__ z, V* __restrict__ y, const V* __restrict__ add_vec,
          V alpha) {
  __shared__ V s_part[kB1Warps][kTileRows];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long t = blockIdx.x;
  const long long t0 = t * kTileRows;
  V acc0 = V(0), acc1 = V(0);
  for (long long q = op.t_ptr[t] + warp; q < op.t_ptr[t + 1]; q += kB1Warps) {
    const int b = op.t_blk[q];
    const long long r0 = op.r0[b];
    const int m = op.m[b], k = op.k[b];
    const bool lr = op.zoff[b] >= 0;
    const V* src = lr ? z + op.zoff[b] : x + op.c0[b];
    const T* w = wpool + op.woff[b];
    const long long i0 = t0 + lane, i1 = t0 + lane + 32;
    const bool in0 = i0 >= r0 && i0 < r0 + m, in1 = i1 >= r0 && i1 < r0 + m;
    const T* w0 = w + (i0 - r0);
    const T* w1 = w + (i1 - r0);
    int l = 0;
    for (; l + 4 <= k; l += 4) {
      const V s0 = __ldg(src + l), s1 = __ldg(src + l + 1), s2 = __ldg(src + l + 2),
              s3 = __ldg(src + l + 3);
      if (in0) {
        acc0 += (V)w0[(long long)l * m] * s0 + (V)w0[(long long)(l + 1) * m] * s1 +
                (V)w0[(long long)(l + 2) * m] * s2 + (V)w0[(long long)(l + 3) * m] * s3;
      }
      if (in1) {
        acc1 += (V)w1[(long long)l * m] * s0 + (V)w1[(long long)(l + 1) * m] * s1 +
                (V)w1[(long long)(l + 2) * m] * s2 + (V)w1[(long long)(l + 3) * m] * s3;
      }
    }
    for (; l < k; l++) {
      const V sv = __ldg(src + l);
      if (in0) acc0 += (V)w0[(long long)l * m] * sv;
      if (in1) acc1 += (V)w1[(long long)l * m] * sv;
    }
  }
  s_part[warp][lane] = acc0;
  s_part[warp][lane + 32] = acc1;
  __syncthreads();
  if (threadIdx.x < kTileRows) {
    V sum = V(0);
#pragma unroll
    for (int wv = 0; wv < kB1Warps; wv++) sum += s_part[wv][threadIdx.x];
    const long long i = t0 + threadIdx.x;
    if (i < op.N) y[i] = add_vec ? add_vec[i] + alpha * sum : sum;
  }
}

// ------------------------------------------------- K RHS, FP32 FFMA ----
// Phase A: CTA per (item, 64-column K tile); Z block (k x 64) accumulated
// in registers: thread (ty, tx) owns rows l = ty + 16 r, columns tx*4..+4.
constexpr int kKT = 64;   // K columns per CTA
constexpr int kJC = 32;   // reduction chunk

__global__ void __launch_bounds__(256)
phaseA_kn_f32(OpView op, const float* __restrict__ vpool, const float* __restrict__ X,
              float* __restrict__ Z, int K) {
  __shared__ float s_v[64][kJC + 1];
  __shared__ float s_x[kJC][kKT];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int nkt = (K + kKT - 1) / kKT;
  const long long it = blockIdx.x / nkt;
  const int c_base = (int)(blockIdx.x % nkt) * kKT;
  const int b = op.a_blk[it];
  const int j0 = op.a_j0[it], j1 = op.a_j1[it];
  const int n = op.n[b], k = op.k[b];
  const long long c0 = op.c0[b];
  const float* vt = vpool + op.voff[b];
  float acc[4][4];
#pragma unroll
  for (int r = 0; r < 4; r++)
#pragma unroll
    for (int c = 0; c < 4; c++) acc[r][c] = 0.f;
  for (int jc = j0; jc < j1; jc += kJC) {
    __syncthreads();
    for (int q = threadIdx.x; q < 64 * kJC; q += 256) {
      int l = q / kJC, j = q % kJC;
      s_v[l][j] = (l < k && jc + j < j1) ? vt[(long long)l * n + jc + j] : 0.f;
    }
    for (int q = threadIdx.x; q < kJC * kKT; q += 256) {
      int j = q / kKT, c = q % kKT;
      s_x[j][c] = (jc + j < j1 && c_base + c < K) ? X[(c0 + jc + j) * (long long)K + c_base + c] : 0.f;
    }
    __syncthreads();
#pragma unroll 4
    for (int j = 0; j < kJC; j++) {
      float xv[4];
#pragma unroll
      for (int c = 0; c < 4; c++) xv[c] = s_x[j][tx * 4 + c];
#pragma unroll
      for (int r = 0; r < 4; r++) {
        float v = s_v[ty + 16 * r][j];
#pragma unroll
        for (int c = 0; c < 4; c++) acc[r][c] += v * xv[c];
      }
    }
  }
  const bool excl = op.a_excl[it];
  float* zb = Z + op.zoff[b] * (long long)K;
#pragma unroll
  for (int r = 0; r < 4; r++) {
    int l = ty + 16 * r;
    if (l >= k) continue;
#pragma unroll
    for (int c = 0; c < 4; c++) {
      int col = c_base + tx * 4 + c;
      if (col >= K) continue;
      if (excl) zb[(long long)l * K + col] = acc[r][c];
      else atomicAdd(zb + (long long)l * K + col, acc[r][c]);
    }
  }
}

// Phase B: CTA per (row tile of 64, 64 columns); thread owns 4 rows x 4 cols.
__global__ void __launch_bounds__(256)
phaseB_kn_f32(OpView op, const float* __restrict__ wpool, const float* __restrict__ X,
              const float* __restrict__ Z, float* __restrict__ Y, int K,
              const float* __restrict__ add_mat, float alpha) {
  __shared__ float s_w[kJC][kTileRows + 1];
  __shared__ float s_s[kJC][kKT];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int nkt = (K + kKT - 1) / kKT;
  const long long t = blockIdx.x / nkt;
  const long long t0 = t * kTileRows;
  const int c_base = (int)(blockIdx.x % nkt) * kKT;
  float acc[4][4];
#pragma unroll
  for (int r = 0; r < 4; r++)
#pragma unroll
    for (int c = 0; c < 4; c++) acc[r][c] = 0.f;
  for (long long q = op.t_ptr[t]; q < op.t_ptr[t + 1]; q++) {
    const int b = op.t_blk[q];
    const long long r0 = op.r0[b];
    const int m = op.m[b], k = op.k[b];
    const bool lr = op.zoff[b] >= 0;
    const float* src = lr ? Z + op.zoff[b] * (long long)K : X + (long long)op.c0[b] * K;
    const float* w = wpool + op.woff[b];
    const long long lo = max(t0, r0), hi = min(t0 + kTileRows, r0 + (long long)m);
    for (int l0 = 0; l0 < k; l0 += kJC) {
      __syncthreads();
      for (int e = threadIdx.x; e < kJC * kTileRows; e += 256) {
        int l = e / kTileRows, ri = e % kTileRows;
        long long i = t0 + ri;
        s_w[l][ri] = (l0 + l < k && i >= lo && i < hi) ? w[(long long)(l0 + l) * m + (i - r0)] : 0.f;
      }
      for (int e = threadIdx.x; e < kJC * kKT; e += 256) {
        int l = e / kKT, c = e % kKT;
        s_s[l][c] = (l0 + l < k && c_base + c < K) ? src[(long long)(l0 + l) * K + c_base + c] : 0.f;
      }
      __syncthreads();
#pragma unroll 4
      for (int l = 0; l < kJC; l++) {
        float sv[4];
#pragma unroll
        for (int c = 0; c < 4; c++) sv[c] = s_s[l][tx * 4 + c];
#pragma unroll
        for (int r = 0; r < 4; r++) {
          float wv = s_w[l][ty + 16 * r];
#pragma unroll
          for (int c = 0; c < 4; c++) acc[r][c] += wv * sv[c];
        }
      }
    }
  }
#pragma unroll
  for (int r = 0; r < 4; r++) {
    long long i = t0 + ty + 16 * r;
    if (i >= op.N) continue;
#pragma unroll
    for (int c = 0; c < 4; c++) {
      int col = c_base + tx * 4 + c;
      if (col >= K) continue;
      float v = acc[r][c];
      if (add_mat) v = add_mat[i * K + col] + alpha * v;
      Y[i * K + col] = v;
    }
  }
}

// ------------------------------------------ K RHS, BF16 tensor cores ----
// mma.sync.m16n8k16 (bf16 x bf16 -> fp32).  Fragments are loaded from shared
// memory with ldmatrix (.trans where the operand is stored k-major).
// CTA: 4 warps, tile 64 x 128 (Phase A: rows = factor rows l <= 64, warp w
// owns columns 32w..32w+31; Phase B: rows = Y rows, warp w owns rows
// 16w..16w+15 and all 128 columns), reduction chunk 32.
constexpr int kBT = 128;     // columns per CTA
constexpr int kBK = 32;      // reduction chunk
constexpr int kAPad = 40;    // smem row length (elements) for 32-wide rows
constexpr int kBPad = 136;   // smem row length for 128-wide rows
constexpr int kMPad = 72;    // smem row length for 64-wide rows

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void ldm_x4(unsigned addr, unsigned& r0, unsigned& r1, unsigned& r2,
                                       unsigned& r3) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3) : "r"(addr));
}
__device__ __forceinline__ void ldm_x4_t(unsigned addr, unsigned& r0, unsigned& r1, unsigned& r2,
                                         unsigned& r3) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3) : "r"(addr));
}
__device__ __forceinline__ void mma_bf16(float* c, unsigned a0, unsigned a1, unsigned a2,
                                         unsigned a3, unsigned b0, unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// Phase A: Z[zoff + l, c] (+)= sum_j Vt[l, j] X[c0 + j, c]
__global__ void __launch_bounds__(128)
phaseA_kn_bf16(OpView op, const __nv_bfloat16* __restrict__ vpool,
               const __nv_bfloat16* __restrict__ X, long long ldx, float* __restrict__ Z,
               long long ldz, int K) {
  __shared__ __align__(16) __nv_bfloat16 s_a[64][kAPad];
  __shared__ __align__(16) __nv_bfloat16 s_b[kBK][kBPad];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nkt = (K + kBT - 1) / kBT;
  const int c_base = (int)(blockIdx.x % nkt) * kBT;
  const long long it = blockIdx.x / nkt;
  const int b = op.a_blk[it];
  const int j0 = op.a_j0[it], j1 = op.a_j1[it];
  const int n = op.n[b], k = op.k[b];
  const long long c0 = op.c0[b];
  const __nv_bfloat16* vt = vpool + op.voff[b];
  const __nv_bfloat16 zero = __float2bfloat16(0.f);
  float acc[4][4][4];
#pragma unroll
  for (int mt = 0; mt < 4; mt++)
#pragma unroll
    for (int nt = 0; nt < 4; nt++)
#pragma unroll
      for (int e = 0; e < 4; e++) acc[mt][nt][e] = 0.f;
  const int mtiles = (k + 15) >> 4;
  for (int jc = j0; jc < j1; jc += kBK) {
    __syncthreads();
    for (int q = threadIdx.x; q < 64 * kBK; q += 128) {
      int l = q / kBK, j = q % kBK;
      s_a[l][j] = (l < k && jc + j < j1) ? vt[(long long)l * n + jc + j] : zero;
    }
    for (int q = threadIdx.x; q < kBK * (kBT / 8); q += 128) {
      int j = q / (kBT / 8), c8 = (q % (kBT / 8)) * 8;
      uint4 v = make_uint4(0, 0, 0, 0);
      if (jc + j < j1 && c_base + c8 < K)
        v = *reinterpret_cast<const uint4*>(X + (c0 + jc + j) * ldx + c_base + c8);
      *reinterpret_cast<uint4*>(&s_b[j][c8]) = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kBK; kk += 16) {
      unsigned bf[4][2];
#pragma unroll
      for (int np = 0; np < 2; np++) {
        // two n8 tiles per ldmatrix.x4.trans: matrices (k 0-7, n), (k 8-15, n), (k 0-7, n+8), (k 8-15, n+8)
        const int mi = lane >> 3, r = lane & 7;
        const int krow = kk + r + ((mi & 1) ? 8 : 0);
        const int ncol = warp * 32 + np * 16 + ((mi & 2) ? 8 : 0);
        ldm_x4_t(smem_u32(&s_b[krow][ncol]), bf[2 * np][0], bf[2 * np][1], bf[2 * np + 1][0],
                 bf[2 * np + 1][1]);
      }
#pragma unroll
      for (int mt = 0; mt < 4; mt++) {
        if (mt >= mtiles) break;
        unsigned a0, a1, a2, a3;
        const int mi = lane >> 3, r = lane & 7;
        const int row = mt * 16 + r + ((mi & 1) ? 8 : 0);
        const int col = kk + ((mi & 2) ? 8 : 0);
        ldm_x4(smem_u32(&s_a[row][col]), a0, a1, a2, a3);
#pragma unroll
        for (int nt = 0; nt < 4; nt++) mma_bf16(acc[mt][nt], a0, a1, a2, a3, bf[nt][0], bf[nt][1]);
      }
    }
  }
  const bool excl = op.a_excl[it];
  float* zb = Z + op.zoff[b] * ldz;
  const int g = lane >> 2, tg = lane & 3;
#pragma unroll
  for (int mt = 0; mt < 4; mt++) {
#pragma unroll
    for (int nt = 0; nt < 4; nt++) {
#pragma unroll
      for (int e = 0; e < 4; e++) {
        int l = mt * 16 + g + ((e & 2) ? 8 : 0);
        int col = c_base + warp * 32 + nt * 8 + tg * 2 + (e & 1);
        if (l < k && col < K) {
          if (excl) zb[(long long)l * ldz + col] = acc[mt][nt][e];
          else atomicAdd(zb + (long long)l * ldz + col, acc[mt][nt][e]);
        }
      }
    }
  }
}

__global__ void f32_to_bf16_kernel(const float* __restrict__ in, __nv_bfloat16* __restrict__ out,
                                   long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    out[i] = __float2bfloat16(in[i]);
}

// Phase B: Y[i, c] = (add[i, c] + alpha *) sum_blocks sum_l W[l, i - r0] S[l, c]
__global__ void __launch_bounds__(128)
phaseB_kn_bf16(OpView op, const __nv_bfloat16* __restrict__ wpool,
               const __nv_bfloat16* __restrict__ X, long long ldx,
               const __nv_bfloat16* __restrict__ Zb, long long ldz, float* __restrict__ Y,
               long long ldy, int K, const float* __restrict__ add_mat, long long ld_add,
               float alpha) {
  __shared__ __align__(16) __nv_bfloat16 s_w[kBK][kMPad];   // [l][row]
  __shared__ __align__(16) __nv_bfloat16 s_s[kBK][kBPad];   // [l][col]
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nkt = (K + kBT - 1) / kBT;
  const int c_base = (int)(blockIdx.x % nkt) * kBT;
  const long long t = blockIdx.x / nkt;
  const long long t0 = t * kTileRows;
  const __nv_bfloat16 zero = __float2bfloat16(0.f);
  float acc[16][4];
#pragma unroll
  for (int nt = 0; nt < 16; nt++)
#pragma unroll
    for (int e = 0; e < 4; e++) acc[nt][e] = 0.f;
  for (long long q = op.t_ptr[t]; q < op.t_ptr[t + 1]; q++) {
    const int b = op.t_blk[q];
    const long long r0 = op.r0[b];
    const int m = op.m[b], k = op.k[b];
    const bool lr = op.zoff[b] >= 0;
    const __nv_bfloat16* src = lr ? Zb + op.zoff[b] * ldz : X + (long long)op.c0[b] * ldx;
    const long long lds = lr ? ldz : ldx;
    const __nv_bfloat16* w = wpool + op.woff[b];
    const long long lo = max(t0, r0), hi = min(t0 + kTileRows, r0 + (long long)m);
    for (int l0 = 0; l0 < k; l0 += kBK) {
      __syncthreads();
      for (int e = threadIdx.x; e < kBK * kTileRows; e += 128) {
        int l = e / kTileRows, ri = e % kTileRows;
        long long i = t0 + ri;
        s_w[l][ri] = (l0 + l < k && i >= lo && i < hi) ? w[(long long)(l0 + l) * m + (i - r0)] : zero;
      }
      for (int e = threadIdx.x; e < kBK * (kBT / 8); e += 128) {
        int l = e / (kBT / 8), c8 = (e % (kBT / 8)) * 8;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (l0 + l < k && c_base + c8 < K)
          v = *reinterpret_cast<const uint4*>(src + (long long)(l0 + l) * lds + c_base + c8);
        *reinterpret_cast<uint4*>(&s_s[l][c8]) = v;
      }
      __syncthreads();
#pragma unroll
      for (int kk = 0; kk < kBK; kk += 16) {
        unsigned a0, a1, a2, a3;
        {
          // A = W^T (rows x l) stored [l][row]: ldmatrix.x4.trans
          const int mi = lane >> 3, r = lane & 7;
          const int lrow = kk + r + ((mi & 2) ? 8 : 0);
          const int rcol = warp * 16 + ((mi & 1) ? 8 : 0);
          ldm_x4_t(smem_u32(&s_w[lrow][rcol]), a0, a1, a2, a3);
        }
#pragma unroll
        for (int np = 0; np < 8; np++) {
          unsigned b0, b1, b2, b3;
          const int mi = lane >> 3, r = lane & 7;
          const int krow = kk + r + ((mi & 1) ? 8 : 0);
          const int ncol = np * 16 + ((mi & 2) ? 8 : 0);
          ldm_x4_t(smem_u32(&s_s[krow][ncol]), b0, b1, b2, b3);
          mma_bf16(acc[2 * np], a0, a1, a2, a3, b0, b1);
          mma_bf16(acc[2 * np + 1], a0, a1, a2, a3, b2, b3);
        }
      }
    }
  }
  const int g = lane >> 2, tg = lane & 3;
#pragma unroll
  for (int nt = 0; nt < 16; nt++) {
#pragma unroll
    for (int e = 0; e < 4; e++) {
      long long i = t0 + warp * 16 + g + ((e & 2) ? 8 : 0);
      int col = c_base + nt * 8 + tg * 2 + (e & 1);
      if (i < op.N && col < K) {
        float v = acc[nt][e];
        if (add_mat) v = add_mat[i * ld_add + col] + alpha * v;
        Y[i * ldy + col] = v;
      }
    }
  }
}

int check_op(const OpView& op) {
  if (op.N < 0 || op.num_tiles < 0 || op.num_items < 0) { set_error("bad operator sizes"); return FGB_BAD_ARG; }
  return FGB_OK;
}

}  // namespace
}  // namespace fgb


namespace fgb {
namespace {
OpView to_view(const fgb_op_desc* d) {
  OpView v;
  v.r0 = d->r0; v.m = d->m; v.c0 = d->c0; v.n = d->n; v.k = d->k;
  v.woff = d->woff; v.voff = d->voff; v.zoff = d->zoff;
  v.a_blk = d->a_blk; v.a_j0 = d->a_j0; v.a_j1 = d->a_j1; v.a_excl = d->a_excl;
  v.num_items = d->num_items;
  v.t_ptr = d->t_ptr; v.t_blk = d->t_blk; v.num_tiles = d->num_tiles;
  v.N = d->N;
  return v;
}
}  // namespace
}  // namespace fgb

extern "C" {

/*
 * y = F x (+ optional y = add + alpha * F x), single right-hand side, FP32
 * factors.  x, y, add: N floats in cluster (permuted) order.  z: scratch of
 * num_zrows floats (phase A output); it is fully overwritten for blocks
 * processed by one item and must be zeroed by the caller when some block
 * is split into several items (fgb_op_desc.a_excl == 0 somewhere): pass
 * zero_z != 0 to have it zeroed here.
 */
int fgb_matvec_f32(const fgb_op_desc* d, const float* wpool, const float* vpool, const float* x,
                   float* z, float* y, const float* add, float alpha, int zero_z, void* stream) {
  fgb::OpView op = fgb::to_view(d);
  int st = fgb::check_op(op);
  if (st) return st;
  cudaStream_t s = fgb::as_stream(stream);
  if (zero_z && d->num_zrows > 0) FGB_CUDA_TRY(cudaMemsetAsync(z, 0, sizeof(float) * d->num_zrows, s));
  if (op.num_items > 0) {
    fgb::phaseA_k1<float, float><<<fgb::grid_for(op.num_items * 32, 256, 152LL * 64), 256, 0, s>>>(op, vpool, x, z);
    FGB_LAUNCH_CHECK("phaseA_k1");
  }
  if (op.num_tiles > 0) {
    fgb::phaseB_k1<float, float><<<(unsigned)op.num_tiles, fgb::kB1Warps * 32, 0, s>>>(op, wpool, x, z, y, add, alpha);
    FGB_LAUNCH_CHECK("phaseB_k1");
  }
  return FGB_OK;
}

/* Same with FP64 factors and FP64 vectors (reference-precision path). */
int fgb_matvec_f64(const fgb_op_desc* d, const double* wpool, const double* vpool, const double* x,
                   double* z, double* y, const double* add, double alpha, int zero_z,
                   void* stream) {
  fgb::OpView op = fgb::to_view(d);
  int st = fgb::check_op(op);
  if (st) return st;
  cudaStream_t s = fgb::as_stream(stream);
  if (zero_z && d->num_zrows > 0) FGB_CUDA_TRY(cudaMemsetAsync(z, 0, sizeof(double) * d->num_zrows, s));
  if (op.num_items > 0) {
    fgb::phaseA_k1<double, double><<<fgb::grid_for(op.num_items * 32, 256, 152LL * 64), 256, 0, s>>>(op, vpool, x, z);
    FGB_LAUNCH_CHECK("phaseA_k1");
  }
  if (op.num_tiles > 0) {
    fgb::phaseB_k1<double, double><<<(unsigned)op.num_tiles, fgb::kB1Warps * 32, 0, s>>>(op, wpool, x, z, y, add, alpha);
    FGB_LAUNCH_CHECK("phaseB_k1");
  }
  return FGB_OK;
}

/*
 * Y = F X (+ add + alpha F X) for K right-hand sides, FP32 factors and FP32
 * CUDA-core arithmetic.  X, Y, add: N x K row-major; Z: num_zrows x K.
 */
int fgb_matmat_f32(const fgb_op_desc* d, const float* wpool, const float* vpool, const float* X,
                   float* Z, float* Y, int K, const float* add, float alpha, int zero_z,
                   int phases, void* stream) {
  fgb::OpView op = fgb::to_view(d);
  int st = fgb::check_op(op);
  if (st) return st;
  if (K < 1) { fgb::set_error("K must be >= 1"); return FGB_BAD_ARG; }
  cudaStream_t s = fgb::as_stream(stream);
  if ((phases & 1) && zero_z && d->num_zrows > 0)
    FGB_CUDA_TRY(cudaMemsetAsync(Z, 0, sizeof(float) * d->num_zrows * (size_t)K, s));
  unsigned ky = (unsigned)((K + fgb::kKT - 1) / fgb::kKT);
  if ((phases & 1) && op.num_items > 0) {
    dim3 g((unsigned)(op.num_items * ky));
    fgb::phaseA_kn_f32<<<g, 256, 0, s>>>(op, vpool, X, Z, K);
    FGB_LAUNCH_CHECK("phaseA_kn_f32");
  }
  if ((phases & 2) && op.num_tiles > 0) {
    dim3 g((unsigned)(op.num_tiles * ky));
    fgb::phaseB_kn_f32<<<g, 256, 0, s>>>(op, wpool, X, Z, Y, K, add, alpha);
    FGB_LAUNCH_CHECK("phaseB_kn_f32");
  }
  return FGB_OK;
}

/*
 * Y = F X (+ add + alpha F X) for K right-hand sides on the tensor cores:
 * BF16 factors and BF16 X, FP32 accumulation, FP32 Y.  X: N x K bf16
 * (row stride K, K a multiple of 8), Z: num_zrows x K fp32 scratch, Zb: the
 * same in bf16, Y / add: N x K fp32.
 */
int fgb_matmat_bf16(const fgb_op_desc* d, const void* wpool, const void* vpool, const void* X,
                    float* Z, void* Zb, float* Y, int K, const float* add, float alpha,
                    int zero_z, int phases, void* stream) {
  fgb::OpView op = fgb::to_view(d);
  int st = fgb::check_op(op);
  if (st) return st;
  if (K < 8 || (K % 8) != 0) { fgb::set_error("K must be a positive multiple of 8"); return FGB_BAD_ARG; }
  if ((reinterpret_cast<uintptr_t>(X) & 15) || (reinterpret_cast<uintptr_t>(Zb) & 15)) {
    fgb::set_error("X and Zb must be 16-byte aligned");
    return FGB_BAD_ARG;
  }
  cudaStream_t s = fgb::as_stream(stream);
  const __nv_bfloat16* w = static_cast<const __nv_bfloat16*>(wpool);
  const __nv_bfloat16* v = static_cast<const __nv_bfloat16*>(vpool);
  const __nv_bfloat16* x = static_cast<const __nv_bfloat16*>(X);
  __nv_bfloat16* zb = static_cast<__nv_bfloat16*>(Zb);
  unsigned kx = (unsigned)((K + fgb::kBT - 1) / fgb::kBT);
  if ((phases & 1) && op.num_items > 0) {
    if (zero_z) FGB_CUDA_TRY(cudaMemsetAsync(Z, 0, sizeof(float) * d->num_zrows * (size_t)K, s));
    dim3 g((unsigned)(op.num_items * kx));
    fgb::phaseA_kn_bf16<<<g, 128, 0, s>>>(op, v, x, K, Z, K, K);
    FGB_LAUNCH_CHECK("phaseA_kn_bf16");
    long long nz = d->num_zrows * (long long)K;
    fgb::f32_to_bf16_kernel<<<fgb::grid_for(nz, 256), 256, 0, s>>>(Z, zb, nz);
    FGB_LAUNCH_CHECK("f32_to_bf16_kernel");
  }
  if ((phases & 2) && op.num_tiles > 0) {
    dim3 g((unsigned)(op.num_tiles * kx));
    fgb::phaseB_kn_bf16<<<g, 128, 0, s>>>(op, w, x, K, zb, K, Y, K, K, add, K, alpha);
    FGB_LAUNCH_CHECK("phaseB_kn_bf16");
  }
  return FGB_OK;
}

}  // extern "C"
