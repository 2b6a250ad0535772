// Block matvec of the compressed form-factor operator.
//
// Replaces the recursive Python matvec of CompressedFormFactorMatrix
// (src/flux/compressed_form_factors.py:805 -> FormFactorBlockMatrix._matmat
// :407-414 -> leaf blocks: dense :175, CSR :193, SVD :247-251).
//
// Everything is in cluster order, where each block's rows and columns are
// contiguous ranges.  The operator is F ~= sum_LR U_b V_b^T + sum_dense D_b.
// It is applied in two phases, each a dense "gather-GEMM" over panels built
// once at setup (no per-block loops in the hot kernels):
//
//   Phase A (low-rank blocks, grouped by their column range):
//     group g = all LR blocks with columns [c0, c0+n): their V^T rows
//     stacked into one panel Vg (kz x n, row stride ldv = n rounded up to 8);
//     Z[z0 + r, :] = sum_j Vg[r, j] X[c0 + j, :]   for r < kz
//     Work items (g, j0, j1) split long groups; items that do not cover the
//     whole group accumulate with atomics into a zeroed Z.
//
//   Phase B (row tiles of 64 rows):
//     tile t owns panel rows [p0, p1) (a multiple of 32 rows); panel row l
//     holds 64 weights W[l, i] for the tile's rows i and a source index
//     src[l]: a row of Z (src < num_zrows: U^T rows of an LR block) or a row
//     of X (src - num_zrows: D^T rows of an exact dense block, i.e. its
//     columns).  Y[t0 + i, :] = sum_l W[l, i] S[src[l], :].
//     Padding rows have zero weights and src 0.
// Every Y row is written once by the CTA of its tile: deterministic, no
// atomics in phase B.
#include "common.cuh"

#include <cuda_bf16.h>

namespace fgb {
namespace {

constexpr int kTileRows = 64;

struct PanelView {
  // phase A
  const int* g_c0;
  const int* g_n;
  const int* g_kz;
  const int* g_ldv;
  const long long* g_voff;
  const long long* g_z0;
  const int* a_grp;
  const int* a_j0;
  const int* a_j1;
  const unsigned char* a_excl;
  long long num_items;
  const long long* a_woff;  // first 64-row work slice of each item
  long long num_work;
  // phase B
  const long long* t_p0;  // num_tiles + 1 panel row offsets
  const int* src;         // per panel row
  long long num_tiles;
  int tile_rows;
  long long N;
  long long num_zrows;
};

// ------------------------------------------------------------ K = 1 ----
// Phase A: one CTA per work slice (item, 64 stacked V^T rows); the item's
// x segment (at most ITEM_COLS = 2048 values) is staged in shared memory and
// warp w computes the dot products of rows w, w + 8, ... (coalesced, 4-wide
// loads along the row), reduced with shuffles in a fixed order.
constexpr int kItemColsMax = 2048;

template <class T> struct Vec4;
template <> struct Vec4<float> { using type = float4; };
template <> struct Vec4<double> { using type = double4_32a; };

template <class T, class V>
__global__ void __launch_bounds__(256)
phaseA_k1(PanelView op, const T* __restrict__ vpanel, const V* __restrict__ x,
          V* __restrict__ z) {
  __shared__ __align__(16) V s_x[kItemColsMax];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (long long unit = blockIdx.x; unit < op.num_work; unit += gridDim.x) {
    long long lo = 0, hi = op.num_items - 1;
    while (lo < hi) {
      const long long mid = (lo + hi + 1) >> 1;
      if (op.a_woff[mid] <= unit) lo = mid; else hi = mid - 1;
    }
    const long long it = lo;
    const int s = (int)(unit - op.a_woff[it]);
    const int g = op.a_grp[it];
    const int j0 = op.a_j0[it], j1 = op.a_j1[it];
    const int n = j1 - j0;
    const int kz = op.g_kz[g], ldv = op.g_ldv[g];
    const bool excl = op.a_excl[it];
    __syncthreads();
    const V* xb = x + op.g_c0[g] + j0;
    // items are at most kItemColsMax columns wide (the host splits groups);
    // a wider one would read x from global memory directly
    const bool staged = n <= kItemColsMax;
    if (staged)
      for (int j = threadIdx.x; j < n; j += blockDim.x) s_x[j] = __ldg(xb + j);
    __syncthreads();
    const V* xs = staged ? s_x : xb;
    const T* vg = vpanel + op.g_voff[g] + j0;
    V* zg = z + op.g_z0[g];
    const int r_end = min(kz, (s + 1) * 64);
    for (int r = s * 64 + warp; r < r_end; r += 8) {
      const T* row = vg + (long long)r * ldv;   // 32-byte aligned: ldv % 8 == 0, j0 % 2048 == 0
      V acc = V(0);
      const int n4 = n & ~3;
      for (int j = lane * 4; j < n4; j += 128) {
        const typename Vec4<T>::type w = *reinterpret_cast<const typename Vec4<T>::type*>(row + j);
        acc += (V)w.x * xs[j] + (V)w.y * xs[j + 1] + (V)w.z * xs[j + 2] + (V)w.w * xs[j + 3];
      }
      for (int j = n4 + lane; j < n; j += 32) acc += (V)row[j] * xs[j];
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
      if (lane == 0) {
        if (excl) zg[r] = acc;
        else atomicAdd(zg + r, acc);
      }
    }
  }
}

// Phase B: one CTA per tile; warp w accumulates panel rows p0 + w, p0 + w + 8,
// ... for the tile's rows 2 lane and 2 lane + 1 (each panel row read as one
// 256-byte (FP32) line per warp), eight rows in flight per warp; the eight
// warps' partial sums are added in a fixed order.
template <class T> struct Vec2;
template <> struct Vec2<float> { using type = float2; };
template <> struct Vec2<double> { using type = double2; };

template <class T, class V>
__global__ void __launch_bounds__(256)
phaseB_k1(PanelView op, const T* __restrict__ panel, const V* __restrict__ x,
          const V* __restrict__ z, V* __restrict__ y, const V* __restrict__ add_vec, V alpha) {
  __shared__ V s_part[8][kTileRows];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long t = blockIdx.x;
  const long long p0 = op.t_p0[t], p1 = op.t_p0[t + 1];
  const long long nz = op.num_zrows;
  using T2 = typename Vec2<T>::type;
  V a0 = V(0), a1 = V(0);
  auto src_val = [&](long long l) -> V {
    const int sidx = __ldg(op.src + l);
    return sidx < nz ? __ldg(z + sidx) : __ldg(x + (sidx - nz));
  };
  long long l = p0 + warp;
  for (; l + 56 < p1; l += 64) {
    V v[8];
    T2 w[8];
#pragma unroll
    for (int u = 0; u < 8; u++) {
      w[u] = __ldg(reinterpret_cast<const T2*>(panel + (l + 8 * u) * kTileRows) + lane);
      v[u] = src_val(l + 8 * u);
    }
#pragma unroll
    for (int u = 0; u < 8; u++) {
      a0 += (V)w[u].x * v[u];
      a1 += (V)w[u].y * v[u];
    }
  }
  for (; l < p1; l += 8) {
    const T2 w = __ldg(reinterpret_cast<const T2*>(panel + l * kTileRows) + lane);
    const V v = src_val(l);
    a0 += (V)w.x * v;
    a1 += (V)w.y * v;
  }
  s_part[warp][2 * lane] = a0;
  s_part[warp][2 * lane + 1] = a1;
  __syncthreads();
  if (threadIdx.x < kTileRows) {
    const int i = threadIdx.x;
    const V sum = ((s_part[0][i] + s_part[1][i]) + (s_part[2][i] + s_part[3][i])) +
                  ((s_part[4][i] + s_part[5][i]) + (s_part[6][i] + s_part[7][i]));
    const long long row = t * kTileRows + i;
    if (row < op.N) y[row] = add_vec ? add_vec[row] + alpha * sum : sum;
  }
}

// ------------------------------------------------- async-copy helpers ----
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
// 16-byte async copy; src_size 0 zero-fills (the address must still be valid)
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem, bool pred) {
  const unsigned s = smem_u32(smem);
  const int n = pred ? 16 : 0;
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(n));
}
// 4-byte async copy (zero-fill when !pred)
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem, bool pred) {
  const unsigned s = smem_u32(smem);
  const int n = pred ? 4 : 0;
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(s), "l"(gmem), "r"(n));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

// ------------------------------------------------- K RHS, FP32 FFMA ----
// s += x with Kahan compensation c (the _rn intrinsics keep the compiler
// from re-associating the compensation away).
__device__ __forceinline__ void kahan_add(float& s, float& c, float x) {
  const float y = __fsub_rn(x, c);
  const float t = __fadd_rn(s, y);
  c = __fsub_rn(__fsub_rn(t, s), y);
  s = t;
}

constexpr int kB32Cols = 128;   // K columns per CTA (FP32 K-column kernels)
constexpr int kB32Chunk = 32;   // reduction rows per stage

// Phase A: CTA per (work slice = item x 64 stacked V^T rows, 128 columns),
// 256 threads; thread (ty, tx) owns rows 8 ty .. + 7 and columns 4 tx .. + 3.
// Per chunk of 32 group columns j the 64 x 32 slab of V^T is staged
// transposed (s_v[j][row], two broadcast 16-byte reads per thread and j)
// and the 32 X rows c0 + j with cp.async; Kahan-compensated chunk sums.
__global__ void __launch_bounds__(256, 2)
phaseA_kn_f32(PanelView op, const float* __restrict__ vpanel, const float* __restrict__ X,
              long long ldx, float* __restrict__ Z, long long ldz, int K) {
  __shared__ __align__(16) float s_v[kB32Chunk][68];   // padded: 4-way store conflicts
  __shared__ __align__(16) float s_x[kB32Chunk][kB32Cols];
  const int tid = threadIdx.x, ty = tid >> 5, tx = tid & 31;
  const int nkt = (K + kB32Cols - 1) / kB32Cols;
  const long long unit = blockIdx.x / nkt;
  const int c_base = (int)(blockIdx.x % nkt) * kB32Cols;
  long long lo = 0, hi = op.num_items - 1;
  while (lo < hi) {
    const long long mid = (lo + hi + 1) >> 1;
    if (op.a_woff[mid] <= unit) lo = mid; else hi = mid - 1;
  }
  const long long it = lo;
  const int sl = (int)(unit - op.a_woff[it]);
  const int g = op.a_grp[it];
  const int kz = op.g_kz[g];
  const int r_base = sl * 64;
  const int j0 = op.a_j0[it], j1 = op.a_j1[it];
  const int ldv = op.g_ldv[g];
  const long long c0 = op.g_c0[g];
  const float* vg = vpanel + op.g_voff[g];
  const bool vec = (K % 4) == 0 && (ldx % 4) == 0 && (ldz % 4) == 0;
  float acc[8][4], comp[8][4];
#pragma unroll
  for (int r = 0; r < 8; r++)
#pragma unroll
    for (int c = 0; c < 4; c++) { acc[r][c] = 0.f; comp[r][c] = 0.f; }
  for (int jc = j0; jc < j1; jc += kB32Chunk) {
    __syncthreads();
    // V^T slab: 64 rows x 32 columns, read along the rows in 16-byte pieces
    // (a warp covers 4 rows x 128 bytes; rows are 32-byte aligned: ldv % 8
    // == 0, jc % 32 == 0), stored transposed
#pragma unroll
    for (int q = 0; q < 2; q++) {
      const int p = tid + q * 256;          // 512 pieces
      const int r = p >> 3, j = (p & 7) * 4;
      const int row = r_base + r;
      float v[4] = {0.f, 0.f, 0.f, 0.f};
      if (row < kz) {
        const float* src = vg + (long long)row * ldv + jc + j;
        if (jc + j + 3 < j1) {
          const float4 f = *reinterpret_cast<const float4*>(src);
          v[0] = f.x; v[1] = f.y; v[2] = f.z; v[3] = f.w;
        } else {
#pragma unroll
          for (int e = 0; e < 4; e++)
            if (jc + j + e < j1) v[e] = src[e];
        }
      }
#pragma unroll
      for (int e = 0; e < 4; e++) s_v[j + e][r] = v[e];
    }
    // X rows c0 + jc .. + 31, 128 columns
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int j = ty + 8 * q;
      const bool okr = jc + j < j1;
      const float* xrow = X + (c0 + (okr ? jc + j : 0)) * ldx;
      const int c = c_base + tx * 4;
      if (vec) {
        const bool ok = okr && c < K;
        cp_async16(&s_x[j][tx * 4], ok ? xrow + c : xrow, ok);
      } else {
#pragma unroll
        for (int e = 0; e < 4; e++) {
          const bool ok = okr && c + e < K;
          cp_async4(&s_x[j][tx * 4 + e], ok ? xrow + c + e : xrow, ok);
        }
      }
    }
    cp_async_commit();
    cp_async_wait<0>();
    __syncthreads();
    float part[8][4];
#pragma unroll
    for (int r = 0; r < 8; r++)
#pragma unroll
      for (int c = 0; c < 4; c++) part[r][c] = 0.f;
#pragma unroll 8
    for (int j = 0; j < kB32Chunk; j++) {
      const float4 v0 = *reinterpret_cast<const float4*>(&s_v[j][ty * 8]);
      const float4 v1 = *reinterpret_cast<const float4*>(&s_v[j][ty * 8 + 4]);
      const float4 xv = *reinterpret_cast<const float4*>(&s_x[j][tx * 4]);
      const float w[8] = {v0.x, v0.y, v0.z, v0.w, v1.x, v1.y, v1.z, v1.w};
      const float x4[4] = {xv.x, xv.y, xv.z, xv.w};
#pragma unroll
      for (int r = 0; r < 8; r++)
#pragma unroll
        for (int c = 0; c < 4; c++) part[r][c] = fmaf(w[r], x4[c], part[r][c]);
    }
#pragma unroll
    for (int r = 0; r < 8; r++)
#pragma unroll
      for (int c = 0; c < 4; c++) kahan_add(acc[r][c], comp[r][c], part[r][c]);
  }
  const bool excl = op.a_excl[it];
  float* zg = Z + op.g_z0[g] * ldz;
  const int col = c_base + tx * 4;
#pragma unroll
  for (int r = 0; r < 8; r++) {
    const int row = r_base + ty * 8 + r;
    if (row >= kz) continue;
#pragma unroll
    for (int c = 0; c < 4; c++) {
      if (col + c >= K) continue;
      float* dst = zg + (long long)row * ldz + col + c;
      if (excl) *dst = acc[r][c];
      else atomicAdd(dst, acc[r][c]);
    }
  }
}

// Phase B: CTA per (tile, 128 columns), 256 threads; thread (ty, tx) =
// (tid / 32, tid % 32) owns rows 8 ty .. 8 ty + 7 and columns 4 tx .. 4 tx + 3
// (32 accumulators).  Per panel row a thread reads its 8 weights as two
// broadcast 16-byte shared loads and its 4 sources as one, for 32 FMAs.
// Chunks of 32 panel rows are double-buffered with cp.async; the chunk's
// partial sums are added to the running sums with Kahan compensation.
__global__ void __launch_bounds__(256, 2)
phaseB_kn_f32(PanelView op, const float* __restrict__ panel, const float* __restrict__ X,
              long long ldx, const float* __restrict__ Z, long long ldz, float* __restrict__ Y,
              long long ldy, int K, const float* __restrict__ add_mat, long long ld_add,
              float alpha) {
  __shared__ __align__(16) float s_w[2][kB32Chunk][kTileRows];
  __shared__ __align__(16) float s_s[2][kB32Chunk][kB32Cols];
  const int tid = threadIdx.x, ty = tid >> 5, tx = tid & 31;
  const int nkt = (K + kB32Cols - 1) / kB32Cols;
  const long long t = blockIdx.x / nkt;
  const int c_base = (int)(blockIdx.x % nkt) * kB32Cols;
  const long long p0 = op.t_p0[t], p1 = op.t_p0[t + 1];
  const bool vec = (K % 4) == 0 && (ldx % 4) == 0 && (ldz % 4) == 0 && (ldy % 4) == 0;
  float acc[8][4], comp[8][4];
#pragma unroll
  for (int r = 0; r < 8; r++)
#pragma unroll
    for (int c = 0; c < 4; c++) { acc[r][c] = 0.f; comp[r][c] = 0.f; }
  auto load = [&](int buf, long long l0) {
    // W: 32 rows x 64 floats = 512 16-byte pieces (2 per thread)
#pragma unroll
    for (int q = 0; q < 2; q++) {
      const int e = tid + q * 256;
      const int l = e >> 4, i4 = (e & 15) * 4;
      cp_async16(&s_w[buf][l][i4], panel + (l0 + l) * kTileRows + i4, true);
    }
    // S: 32 gathered rows x 128 floats = 1024 pieces (4 per thread); rows
    // l = tid / 32 + 8 q, piece tx (16-byte copies when rows are 16-byte
    // aligned, K % 4 == 0; 4-byte copies otherwise)
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int l = ty + 8 * q;
      const int sidx = op.src[l0 + l];
      const float* srow = sidx < op.num_zrows ? Z + (long long)sidx * ldz
                                              : X + (long long)(sidx - op.num_zrows) * ldx;
      const int c = c_base + tx * 4;
      if (vec) {
        const bool ok = c < K;
        cp_async16(&s_s[buf][l][tx * 4], ok ? srow + c : srow, ok);
      } else {
#pragma unroll
        for (int e = 0; e < 4; e++) {
          const bool ok = c + e < K;
          cp_async4(&s_s[buf][l][tx * 4 + e], ok ? srow + c + e : srow, ok);
        }
      }
    }
    cp_async_commit();
  };
  int buf = 0;
  if (p0 < p1) load(0, p0);
  for (long long l0 = p0; l0 < p1; l0 += kB32Chunk) {
    if (l0 + kB32Chunk < p1) {
      load(buf ^ 1, l0 + kB32Chunk);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    float part[8][4];
#pragma unroll
    for (int r = 0; r < 8; r++)
#pragma unroll
      for (int c = 0; c < 4; c++) part[r][c] = 0.f;
#pragma unroll 8
    for (int l = 0; l < kB32Chunk; l++) {
      const float4 w0 = *reinterpret_cast<const float4*>(&s_w[buf][l][ty * 8]);
      const float4 w1 = *reinterpret_cast<const float4*>(&s_w[buf][l][ty * 8 + 4]);
      const float4 sv = *reinterpret_cast<const float4*>(&s_s[buf][l][tx * 4]);
      const float w[8] = {w0.x, w0.y, w0.z, w0.w, w1.x, w1.y, w1.z, w1.w};
      const float x4[4] = {sv.x, sv.y, sv.z, sv.w};
#pragma unroll
      for (int r = 0; r < 8; r++)
#pragma unroll
        for (int c = 0; c < 4; c++) part[r][c] = fmaf(w[r], x4[c], part[r][c]);
    }
#pragma unroll
    for (int r = 0; r < 8; r++)
#pragma unroll
      for (int c = 0; c < 4; c++) kahan_add(acc[r][c], comp[r][c], part[r][c]);
    __syncthreads();
    buf ^= 1;
  }
  const int col = c_base + tx * 4;
  if (col < K) {
#pragma unroll
    for (int r = 0; r < 8; r++) {
      const long long i = t * kTileRows + ty * 8 + r;
      if (i >= op.N) continue;
      float v[4];
#pragma unroll
      for (int c = 0; c < 4; c++) {
        v[c] = acc[r][c];
        if (add_mat) v[c] = add_mat[i * ld_add + col + c] + alpha * v[c];
      }
      if (vec && col + 4 <= K) {
        *reinterpret_cast<float4*>(Y + i * ldy + col) = make_float4(v[0], v[1], v[2], v[3]);
      } else {
        for (int c = 0; c < 4 && col + c < K; c++) Y[i * ldy + col + c] = v[c];
      }
    }
  }
}

// ------------------------------- K RHS, FP32 panels, FP64 arithmetic ----
// The FP32-stored operator applied to FP64 right-hand sides with FP64
// products and sums (the FP32 weights are exact in FP64): FP64 residuals of
// many columns at once.  Same work split as the FP32 kernels above, with 64
// columns per CTA (thread (ty, tx) owns rows 8 ty .. + 7 and columns
// 2 tx, 2 tx + 1) so that the staged FP64 rows fit the same shared memory.
constexpr int kB64Cols = 64;

__device__ __forceinline__ void cp_async8(void* smem, const void* gmem, bool pred) {
  const unsigned s = smem_u32(smem);
  const int n = pred ? 8 : 0;
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(s), "l"(gmem), "r"(n));
}

__global__ void __launch_bounds__(256, 2)
phaseA_kn_w32d(PanelView op, const float* __restrict__ vpanel, const double* __restrict__ X,
               long long ldx, double* __restrict__ Z, long long ldz, int K) {
  __shared__ __align__(16) float s_v[kB32Chunk][68];
  __shared__ __align__(16) double s_x[kB32Chunk][kB64Cols];
  const int tid = threadIdx.x, ty = tid >> 5, tx = tid & 31;
  const int nkt = (K + kB64Cols - 1) / kB64Cols;
  const long long unit = blockIdx.x / nkt;
  const int c_base = (int)(blockIdx.x % nkt) * kB64Cols;
  long long lo = 0, hi = op.num_items - 1;
  while (lo < hi) {
    const long long mid = (lo + hi + 1) >> 1;
    if (op.a_woff[mid] <= unit) lo = mid; else hi = mid - 1;
  }
  const long long it = lo;
  const int sl = (int)(unit - op.a_woff[it]);
  const int g = op.a_grp[it];
  const int kz = op.g_kz[g];
  const int r_base = sl * 64;
  const int j0 = op.a_j0[it], j1 = op.a_j1[it];
  const int ldv = op.g_ldv[g];
  const long long c0 = op.g_c0[g];
  const float* vg = vpanel + op.g_voff[g];
  const bool vec = (K % 2) == 0 && (ldx % 2) == 0;
  double acc[8][2];
#pragma unroll
  for (int r = 0; r < 8; r++) { acc[r][0] = 0.0; acc[r][1] = 0.0; }
  for (int jc = j0; jc < j1; jc += kB32Chunk) {
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 2; q++) {
      const int p = tid + q * 256;
      const int r = p >> 3, j = (p & 7) * 4;
      const int row = r_base + r;
      float v[4] = {0.f, 0.f, 0.f, 0.f};
      if (row < kz) {
        const float* src = vg + (long long)row * ldv + jc + j;
        if (jc + j + 3 < j1) {
          const float4 f = *reinterpret_cast<const float4*>(src);
          v[0] = f.x; v[1] = f.y; v[2] = f.z; v[3] = f.w;
        } else {
#pragma unroll
          for (int e = 0; e < 4; e++)
            if (jc + j + e < j1) v[e] = src[e];
        }
      }
#pragma unroll
      for (int e = 0; e < 4; e++) s_v[j + e][r] = v[e];
    }
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int j = ty + 8 * q;
      const bool okr = jc + j < j1;
      const double* xrow = X + (c0 + (okr ? jc + j : 0)) * ldx;
      const int c = c_base + tx * 2;
      if (vec) {
        const bool ok = okr && c < K;
        cp_async16(&s_x[j][tx * 2], ok ? xrow + c : xrow, ok);
      } else {
#pragma unroll
        for (int e = 0; e < 2; e++) {
          const bool ok = okr && c + e < K;
          cp_async8(&s_x[j][tx * 2 + e], ok ? xrow + c + e : xrow, ok);
        }
      }
    }
    cp_async_commit();
    cp_async_wait<0>();
    __syncthreads();
#pragma unroll 4
    for (int j = 0; j < kB32Chunk; j++) {
      const float4 v0 = *reinterpret_cast<const float4*>(&s_v[j][ty * 8]);
      const float4 v1 = *reinterpret_cast<const float4*>(&s_v[j][ty * 8 + 4]);
      const double2 xv = *reinterpret_cast<const double2*>(&s_x[j][tx * 2]);
      const float w[8] = {v0.x, v0.y, v0.z, v0.w, v1.x, v1.y, v1.z, v1.w};
#pragma unroll
      for (int r = 0; r < 8; r++) {
        acc[r][0] = fma((double)w[r], xv.x, acc[r][0]);
        acc[r][1] = fma((double)w[r], xv.y, acc[r][1]);
      }
    }
  }
  const bool excl = op.a_excl[it];
  double* zg = Z + op.g_z0[g] * ldz;
  const int col = c_base + tx * 2;
#pragma unroll
  for (int r = 0; r < 8; r++) {
    const int row = r_base + ty * 8 + r;
    if (row >= kz) continue;
#pragma unroll
    for (int c = 0; c < 2; c++) {
      if (col + c >= K) continue;
      double* dst = zg + (long long)row * ldz + col + c;
      if (excl) *dst = acc[r][c];
      else atomicAdd(dst, acc[r][c]);
    }
  }
}

__global__ void __launch_bounds__(256, 2)
phaseB_kn_w32d(PanelView op, const float* __restrict__ panel, const double* __restrict__ X,
               long long ldx, const double* __restrict__ Z, long long ldz, double* __restrict__ Y,
               long long ldy, int K, const double* __restrict__ add_mat, long long ld_add,
               double alpha) {
  __shared__ __align__(16) float s_w[2][kB32Chunk][kTileRows];
  __shared__ __align__(16) double s_s[2][kB32Chunk][kB64Cols];
  const int tid = threadIdx.x, ty = tid >> 5, tx = tid & 31;
  const int nkt = (K + kB64Cols - 1) / kB64Cols;
  const long long t = blockIdx.x / nkt;
  const int c_base = (int)(blockIdx.x % nkt) * kB64Cols;
  const long long p0 = op.t_p0[t], p1 = op.t_p0[t + 1];
  const bool vec = (K % 2) == 0 && (ldx % 2) == 0 && (ldz % 2) == 0;
  double acc[8][2];
#pragma unroll
  for (int r = 0; r < 8; r++) { acc[r][0] = 0.0; acc[r][1] = 0.0; }
  auto load = [&](int buf, long long l0) {
#pragma unroll
    for (int q = 0; q < 2; q++) {
      const int e = tid + q * 256;
      const int l = e >> 4, i4 = (e & 15) * 4;
      cp_async16(&s_w[buf][l][i4], panel + (l0 + l) * kTileRows + i4, true);
    }
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int l = ty + 8 * q;
      const int sidx = op.src[l0 + l];
      const double* srow = sidx < op.num_zrows ? Z + (long long)sidx * ldz
                                               : X + (long long)(sidx - op.num_zrows) * ldx;
      const int c = c_base + tx * 2;
      if (vec) {
        const bool ok = c < K;
        cp_async16(&s_s[buf][l][tx * 2], ok ? srow + c : srow, ok);
      } else {
#pragma unroll
        for (int e = 0; e < 2; e++) {
          const bool ok = c + e < K;
          cp_async8(&s_s[buf][l][tx * 2 + e], ok ? srow + c + e : srow, ok);
        }
      }
    }
    cp_async_commit();
  };
  int buf = 0;
  if (p0 < p1) load(0, p0);
  for (long long l0 = p0; l0 < p1; l0 += kB32Chunk) {
    if (l0 + kB32Chunk < p1) {
      load(buf ^ 1, l0 + kB32Chunk);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
#pragma unroll 4
    for (int l = 0; l < kB32Chunk; l++) {
      const float4 w0 = *reinterpret_cast<const float4*>(&s_w[buf][l][ty * 8]);
      const float4 w1 = *reinterpret_cast<const float4*>(&s_w[buf][l][ty * 8 + 4]);
      const double2 sv = *reinterpret_cast<const double2*>(&s_s[buf][l][tx * 2]);
      const float w[8] = {w0.x, w0.y, w0.z, w0.w, w1.x, w1.y, w1.z, w1.w};
#pragma unroll
      for (int r = 0; r < 8; r++) {
        acc[r][0] = fma((double)w[r], sv.x, acc[r][0]);
        acc[r][1] = fma((double)w[r], sv.y, acc[r][1]);
      }
    }
    __syncthreads();
    buf ^= 1;
  }
  const int col = c_base + tx * 2;
#pragma unroll
  for (int r = 0; r < 8; r++) {
    const long long i = t * kTileRows + ty * 8 + r;
    if (i >= op.N) continue;
#pragma unroll
    for (int c = 0; c < 2; c++) {
      if (col + c >= K) continue;
      double v = acc[r][c];
      if (add_mat) v = add_mat[i * ld_add + col + c] + alpha * v;
      Y[i * ldy + col + c] = v;
    }
  }
}

// ------------------------------------------ K RHS, BF16 tensor cores ----
// mma.sync.m16n8k16 (bf16 x bf16 -> fp32).  Fragments come from shared
// memory through ldmatrix (.trans where the operand is stored k-major).
// CTA: 4 warps, tile 64 x 128, reduction chunk 32, double-buffered cp.async.
constexpr int kBT = 128;     // columns per CTA
constexpr int kBK = 32;      // reduction chunk
constexpr int kAPad = 40;    // smem row length (elements) for 32-wide rows
constexpr int kBPad = 136;   // smem row length for 128-wide rows
constexpr int kMPad = 72;    // smem row length for 64-wide rows

// Phase A: Z[z0 + r, c] (+)= sum_j Vg[r, j] X[c0 + j, c], r in a 64-row slice.
__global__ void __launch_bounds__(128)
phaseA_kn_bf16(PanelView op, const __nv_bfloat16* __restrict__ vpanel,
               const __nv_bfloat16* __restrict__ X, long long ldx, float* __restrict__ Z,
               long long ldz, int K, int mt_per_item) {
  __shared__ __align__(16) __nv_bfloat16 s_a[2][64][kAPad];
  __shared__ __align__(16) __nv_bfloat16 s_b[2][kBK][kBPad];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nkt = (K + kBT - 1) / kBT;
  long long bid = blockIdx.x;
  const int c_base = (int)(bid % nkt) * kBT;
  bid /= nkt;
  const int mt = (int)(bid % mt_per_item);
  const long long it = bid / mt_per_item;
  const int g = op.a_grp[it];
  const int kz = op.g_kz[g];
  const int r_base = mt * 64;
  if (r_base >= kz) return;
  const int j0 = op.a_j0[it], j1 = op.a_j1[it];
  const int ldv = op.g_ldv[g];
  const long long c0 = op.g_c0[g];
  const __nv_bfloat16* vg = vpanel + op.g_voff[g] + (long long)r_base * ldv;
  const int rows = min(64, kz - r_base);
  float acc[4][4][4];
#pragma unroll
  for (int m2 = 0; m2 < 4; m2++)
#pragma unroll
    for (int nt = 0; nt < 4; nt++)
#pragma unroll
      for (int e = 0; e < 4; e++) acc[m2][nt][e] = 0.f;
  const int mtiles = (rows + 15) >> 4;
  auto load = [&](int buf, int jc) {
    // A: 64 panel rows x 32 columns (rows padded to ldv % 8 == 0: 16-byte aligned)
    for (int q = threadIdx.x; q < 64 * (kBK / 8); q += 128) {
      int r = q / (kBK / 8), j8 = (q % (kBK / 8)) * 8;
      bool ok = r < rows && jc + j8 < j1;
      const __nv_bfloat16* src = vg + (ok ? (long long)r * ldv + jc + j8 : 0);
      cp_async16(&s_a[buf][r][j8], src, ok);
    }
    for (int q = threadIdx.x; q < kBK * (kBT / 8); q += 128) {
      int j = q / (kBT / 8), c8 = (q % (kBT / 8)) * 8;
      bool ok = jc + j < j1 && c_base + c8 < K;
      const __nv_bfloat16* src = X + (ok ? (c0 + jc + j) * ldx + c_base + c8 : 0);
      cp_async16(&s_b[buf][j][c8], src, ok);
    }
    cp_async_commit();
  };
  int buf = 0;
  load(0, j0);
  for (int jc = j0; jc < j1; jc += kBK) {
    if (jc + kBK < j1) {
      load(buf ^ 1, jc + kBK);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    // A columns beyond j1 were zero-filled; X rows beyond j1 too.  The panel
    // pads each row to a multiple of 8 with zeros, so 8-wide A chunks that
    // start before j1 and end after it read zero weights.
#pragma unroll
    for (int kk = 0; kk < kBK; kk += 16) {
      unsigned bf[4][2];
#pragma unroll
      for (int np = 0; np < 2; np++) {
        const int mi = lane >> 3, r = lane & 7;
        const int krow = kk + r + ((mi & 1) ? 8 : 0);
        const int ncol = warp * 32 + np * 16 + ((mi & 2) ? 8 : 0);
        ldm_x4_t(smem_u32(&s_b[buf][krow][ncol]), bf[2 * np][0], bf[2 * np][1], bf[2 * np + 1][0],
                 bf[2 * np + 1][1]);
      }
#pragma unroll
      for (int m2 = 0; m2 < 4; m2++) {
        if (m2 >= mtiles) break;
        unsigned a0, a1, a2, a3;
        const int mi = lane >> 3, r = lane & 7;
        const int row = m2 * 16 + r + ((mi & 1) ? 8 : 0);
        const int col = kk + ((mi & 2) ? 8 : 0);
        ldm_x4(smem_u32(&s_a[buf][row][col]), a0, a1, a2, a3);
#pragma unroll
        for (int nt = 0; nt < 4; nt++) mma_bf16(acc[m2][nt], a0, a1, a2, a3, bf[nt][0], bf[nt][1]);
      }
    }
    __syncthreads();
    buf ^= 1;
  }
  const bool excl = op.a_excl[it];
  float* zg = Z + (op.g_z0[g] + r_base) * ldz;
  const int gq = lane >> 2, tg = lane & 3;
#pragma unroll
  for (int m2 = 0; m2 < 4; m2++) {
#pragma unroll
    for (int nt = 0; nt < 4; nt++) {
#pragma unroll
      for (int e = 0; e < 4; e++) {
        int r = m2 * 16 + gq + ((e & 2) ? 8 : 0);
        int col = c_base + warp * 32 + nt * 8 + tg * 2 + (e & 1);
        if (r < rows && col < K) {
          if (excl) zg[(long long)r * ldz + col] = acc[m2][nt][e];
          else atomicAdd(zg + (long long)r * ldz + col, acc[m2][nt][e]);
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

// Phase B: Y[t0 + i, c] = (add + alpha *) sum_l W[l, i] S[src[l], c]
__global__ void __launch_bounds__(128)
phaseB_kn_bf16(PanelView op, const __nv_bfloat16* __restrict__ panel,
               const __nv_bfloat16* __restrict__ X, long long ldx,
               const __nv_bfloat16* __restrict__ Zb, long long ldz, float* __restrict__ Y,
               long long ldy, int K, const float* __restrict__ add_mat, long long ld_add,
               float alpha) {
  __shared__ __align__(16) __nv_bfloat16 s_w[2][kBK][kMPad];   // [l][row]
  __shared__ __align__(16) __nv_bfloat16 s_s[2][kBK][kBPad];   // [l][col]
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nkt = (K + kBT - 1) / kBT;
  const int c_base = (int)(blockIdx.x % nkt) * kBT;
  const long long t = blockIdx.x / nkt;
  const long long p0 = op.t_p0[t], p1 = op.t_p0[t + 1];
  float acc[16][4];
#pragma unroll
  for (int nt = 0; nt < 16; nt++)
#pragma unroll
    for (int e = 0; e < 4; e++) acc[nt][e] = 0.f;
  auto load = [&](int buf, long long l0) {
    // W: 32 panel rows x 64 weights (128 B each, contiguous)
    for (int q = threadIdx.x; q < kBK * (kTileRows / 8); q += 128) {
      int l = q / (kTileRows / 8), i8 = (q % (kTileRows / 8)) * 8;
      cp_async16(&s_w[buf][l][i8], panel + (l0 + l) * kTileRows + i8, true);
    }
    // S: 32 gathered rows x 128 columns
    for (int q = threadIdx.x; q < kBK * (kBT / 8); q += 128) {
      int l = q / (kBT / 8), c8 = (q % (kBT / 8)) * 8;
      const int sidx = op.src[l0 + l];
      const __nv_bfloat16* srow = sidx < op.num_zrows ? Zb + (long long)sidx * ldz
                                                      : X + (long long)(sidx - op.num_zrows) * ldx;
      const bool ok = c_base + c8 < K;
      cp_async16(&s_s[buf][l][c8], ok ? srow + c_base + c8 : srow, ok);
    }
    cp_async_commit();
  };
  int buf = 0;
  if (p0 < p1) load(0, p0);
  for (long long l0 = p0; l0 < p1; l0 += kBK) {
    if (l0 + kBK < p1) {
      load(buf ^ 1, l0 + kBK);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kBK; kk += 16) {
      unsigned a0, a1, a2, a3;
      {
        const int mi = lane >> 3, r = lane & 7;
        const int lrow = kk + r + ((mi & 2) ? 8 : 0);
        const int rcol = warp * 16 + ((mi & 1) ? 8 : 0);
        ldm_x4_t(smem_u32(&s_w[buf][lrow][rcol]), a0, a1, a2, a3);
      }
#pragma unroll
      for (int np = 0; np < 8; np++) {
        unsigned b0, b1, b2, b3;
        const int mi = lane >> 3, r = lane & 7;
        const int krow = kk + r + ((mi & 1) ? 8 : 0);
        const int ncol = np * 16 + ((mi & 2) ? 8 : 0);
        ldm_x4_t(smem_u32(&s_s[buf][krow][ncol]), b0, b1, b2, b3);
        mma_bf16(acc[2 * np], a0, a1, a2, a3, b0, b1);
        mma_bf16(acc[2 * np + 1], a0, a1, a2, a3, b2, b3);
      }
    }
    __syncthreads();
    buf ^= 1;
  }
  const int gq = lane >> 2, tg = lane & 3;
#pragma unroll
  for (int nt = 0; nt < 16; nt++) {
#pragma unroll
    for (int e = 0; e < 4; e++) {
      long long i = t * kTileRows + warp * 16 + gq + ((e & 2) ? 8 : 0);
      int col = c_base + nt * 8 + tg * 2 + (e & 1);
      if (i < op.N && col < K) {
        float v = acc[nt][e];
        if (add_mat) v = add_mat[i * ld_add + col] + alpha * v;
        Y[i * ldy + col] = v;
      }
    }
  }
}

// -------------------------------------------------------------- setup ----
// Phase-B panels: panel row p (of pair q) = 64 weights from row l of the
// pair's source matrix (row length m, first operator row r0) for the tile's
// rows t0 .. t0+63 (zero outside [r0, r0+m)).  One warp per panel row.
template <class TI, class TO>
__global__ void build_panel_kernel(const TI* __restrict__ pool, long long num_rows,
                                   const long long* __restrict__ pair_p0,
                                   const long long* __restrict__ pair_w,
                                   const int* __restrict__ pair_m,
                                   const long long* __restrict__ pair_shift,
                                   const int* __restrict__ pair_k, long long num_pairs,
                                   TO* __restrict__ panel) {
  const int lane = threadIdx.x & 31;
  const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long p = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5; p < num_rows;
       p += warps) {
    long long lo = 0, hi = num_pairs - 1;
    while (lo < hi) {
      long long mid = (lo + hi + 1) >> 1;
      if (pair_p0[mid] <= p) lo = mid; else hi = mid - 1;
    }
    const long long l = p - pair_p0[lo];
    TO* out = panel + p * kTileRows;
    if (l >= pair_k[lo]) {  // padding row
      out[lane] = TO(0.f);
      out[lane + 32] = TO(0.f);
      continue;
    }
    const int m = pair_m[lo];
    const long long shift = pair_shift[lo];  // t0 - r0
    const TI* w = pool + pair_w[lo] + l * (long long)m;
    for (int i = lane; i < kTileRows; i += 32) {
      const long long s = shift + i;
      out[i] = (s >= 0 && s < m) ? (TO)w[s] : TO(0.f);
    }
  }
}

// Phase-A panels: row r of the stacked panel = one V^T row of a member block
// (length n, row stride (n + 7) & ~7, zero-padded).
template <class TI, class TO>
__global__ void build_vpanel_kernel(const TI* __restrict__ pool, long long num_rows,
                                    const long long* __restrict__ row_src,
                                    const long long* __restrict__ row_dst,
                                    const int* __restrict__ row_n, TO* __restrict__ vpanel) {
  const int lane = threadIdx.x & 31;
  const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long r = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5; r < num_rows;
       r += warps) {
    const TI* src = pool + row_src[r];
    TO* dst = vpanel + row_dst[r];
    const int n = row_n[r];
    const int ld = (n + 7) & ~7;
    for (int j = lane; j < ld; j += 32) dst[j] = j < n ? (TO)src[j] : TO(0.f);
  }
}

int check_op(const PanelView& op) {
  if (op.N < 0 || op.num_tiles < 0 || op.num_items < 0 || op.num_zrows < 0) {
    set_error("bad operator sizes");
    return FGB_BAD_ARG;
  }
  if (op.tile_rows != 0 && op.tile_rows != kTileRows) {
    set_error("these kernels take the 64-row panel (tile_rows 64)");
    return FGB_BAD_ARG;
  }
  return FGB_OK;
}

PanelView to_view(const fgb_op_desc* d) {
  PanelView v;
  v.g_c0 = d->g_c0; v.g_n = d->g_n; v.g_kz = d->g_kz; v.g_ldv = d->g_ldv;
  v.g_voff = d->g_voff; v.g_z0 = d->g_z0;
  v.a_grp = d->a_grp; v.a_j0 = d->a_j0; v.a_j1 = d->a_j1; v.a_excl = d->a_excl;
  v.num_items = d->num_items;
  v.a_woff = d->a_woff; v.num_work = d->num_work;
  v.t_p0 = d->t_p0; v.src = d->src; v.num_tiles = d->num_tiles;
  v.tile_rows = d->tile_rows;
  v.N = d->N;
  v.num_zrows = d->num_zrows;
  return v;
}

}  // namespace
}  // namespace fgb

extern "C" {

int fgb_matvec_f32(const fgb_op_desc* d, const float* panel, const float* vpanel, const float* x,
                   float* z, float* y, const float* add, float alpha, int zero_z, void* stream) {
  fgb::PanelView op = fgb::to_view(d);
  int st = fgb::check_op(op);
  if (st) return st;
  cudaStream_t s = fgb::as_stream(stream);
  if (zero_z && d->num_zrows > 0) FGB_CUDA_TRY(cudaMemsetAsync(z, 0, sizeof(float) * d->num_zrows, s));
  if (op.num_items > 0) {
    fgb::phaseA_k1<float, float><<<fgb::grid_for(op.num_work, 1, 152LL * 64), 256, 0, s>>>(op, vpanel, x, z);
    FGB_LAUNCH_CHECK("phaseA_k1");
  }
  if (op.num_tiles > 0) {
    fgb::phaseB_k1<float, float><<<(unsigned)op.num_tiles, 256, 0, s>>>(op, panel, x, z, y, add, alpha);
    FGB_LAUNCH_CHECK("phaseB_k1");
  }
  return FGB_OK;
}

int fgb_matvec_f64(const fgb_op_desc* d, const double* panel, const double* vpanel,
                   const double* x, double* z, double* y, const double* add, double alpha,
                   int zero_z, void* stream) {
  fgb::PanelView op = fgb::to_view(d);
  int st = fgb::check_op(op);
  if (st) return st;
  cudaStream_t s = fgb::as_stream(stream);
  if (zero_z && d->num_zrows > 0) FGB_CUDA_TRY(cudaMemsetAsync(z, 0, sizeof(double) * d->num_zrows, s));
  if (op.num_items > 0) {
    fgb::phaseA_k1<double, double><<<fgb::grid_for(op.num_work, 1, 152LL * 64), 256, 0, s>>>(op, vpanel, x, z);
    FGB_LAUNCH_CHECK("phaseA_k1");
  }
  if (op.num_tiles > 0) {
    fgb::phaseB_k1<double, double><<<(unsigned)op.num_tiles, 256, 0, s>>>(op, panel, x, z, y, add, alpha);
    FGB_LAUNCH_CHECK("phaseB_k1");
  }
  return FGB_OK;
}

/* FP32 panels, FP64 vectors and accumulation (residual checks). */
int fgb_matvec_f32_f64(const fgb_op_desc* d, const float* panel, const float* vpanel,
                       const double* x, double* z, double* y, const double* add, double alpha,
                       int zero_z, void* stream) {
  fgb::PanelView op = fgb::to_view(d);
  int st = fgb::check_op(op);
  if (st) return st;
  cudaStream_t s = fgb::as_stream(stream);
  if (zero_z && d->num_zrows > 0) FGB_CUDA_TRY(cudaMemsetAsync(z, 0, sizeof(double) * d->num_zrows, s));
  if (op.num_items > 0) {
    fgb::phaseA_k1<float, double><<<fgb::grid_for(op.num_work, 1, 152LL * 64), 256, 0, s>>>(op, vpanel, x, z);
    FGB_LAUNCH_CHECK("phaseA_k1");
  }
  if (op.num_tiles > 0) {
    fgb::phaseB_k1<float, double><<<(unsigned)op.num_tiles, 256, 0, s>>>(op, panel, x, z, y, add, alpha);
    FGB_LAUNCH_CHECK("phaseB_k1");
  }
  return FGB_OK;
}

int fgb_matmat_f32(const fgb_op_desc* d, const float* panel, const float* vpanel, const float* X,
                   float* Z, float* Y, int K, const float* add, float alpha, int zero_z,
                   int phases, void* stream) {
  fgb::PanelView op = fgb::to_view(d);
  int st = fgb::check_op(op);
  if (st) return st;
  if (K < 1) { fgb::set_error("K must be >= 1"); return FGB_BAD_ARG; }
  cudaStream_t s = fgb::as_stream(stream);
  if ((phases & 1) && op.num_items > 0) {
    if (zero_z && d->num_zrows > 0)
      FGB_CUDA_TRY(cudaMemsetAsync(Z, 0, sizeof(float) * d->num_zrows * (size_t)K, s));
    const long long kb = (K + fgb::kB32Cols - 1) / fgb::kB32Cols;
    fgb::phaseA_kn_f32<<<(unsigned)(op.num_work * kb), 256, 0, s>>>(op, vpanel, X, K, Z, K, K);
    FGB_LAUNCH_CHECK("phaseA_kn_f32");
  }
  if ((phases & 2) && op.num_tiles > 0) {
    const unsigned kb = (unsigned)((K + fgb::kB32Cols - 1) / fgb::kB32Cols);
    fgb::phaseB_kn_f32<<<(unsigned)(op.num_tiles * kb), 256, 0, s>>>(op, panel, X, K, Z, K, Y, K, K,
                                                                      add, K, alpha);
    FGB_LAUNCH_CHECK("phaseB_kn_f32");
  }
  return FGB_OK;
}

int fgb_matmat_f32_f64(const fgb_op_desc* d, const float* panel, const float* vpanel,
                       const double* X, double* Z, double* Y, int K, const double* add,
                       double alpha, int zero_z, void* stream) {
  fgb::PanelView op = fgb::to_view(d);
  int st = fgb::check_op(op);
  if (st) return st;
  if (K < 1) { fgb::set_error("K must be >= 1"); return FGB_BAD_ARG; }
  if (op.tile_rows != fgb::kTileRows) {
    fgb::set_error("fgb_matmat_f32_f64 needs the 64-row panel");
    return FGB_BAD_ARG;
  }
  cudaStream_t s = fgb::as_stream(stream);
  const long long kb = (K + fgb::kB64Cols - 1) / fgb::kB64Cols;
  if (op.num_items > 0) {
    if (zero_z && d->num_zrows > 0)
      FGB_CUDA_TRY(cudaMemsetAsync(Z, 0, sizeof(double) * d->num_zrows * (size_t)K, s));
    fgb::phaseA_kn_w32d<<<(unsigned)(op.num_work * kb), 256, 0, s>>>(op, vpanel, X, K, Z, K, K);
    FGB_LAUNCH_CHECK("phaseA_kn_w32d");
  }
  if (op.num_tiles > 0) {
    fgb::phaseB_kn_w32d<<<(unsigned)(op.num_tiles * kb), 256, 0, s>>>(op, panel, X, K, Z, K, Y, K,
                                                                       K, add, K, alpha);
    FGB_LAUNCH_CHECK("phaseB_kn_w32d");
  }
  return FGB_OK;
}

int fgb_matmat_bf16(const fgb_op_desc* d, const void* panel, const void* vpanel, const void* X,
                    float* Z, void* Zb, float* Y, int K, const float* add, float alpha,
                    int zero_z, int phases, void* stream) {
  fgb::PanelView op = fgb::to_view(d);
  int st = fgb::check_op(op);
  if (st) return st;
  if (K < 8 || (K % 8) != 0) { fgb::set_error("K must be a positive multiple of 8"); return FGB_BAD_ARG; }
  if ((reinterpret_cast<uintptr_t>(X) & 15) || (reinterpret_cast<uintptr_t>(Zb) & 15) ||
      (reinterpret_cast<uintptr_t>(panel) & 15) || (reinterpret_cast<uintptr_t>(vpanel) & 15)) {
    fgb::set_error("X, Zb and the panels must be 16-byte aligned");
    return FGB_BAD_ARG;
  }
  cudaStream_t s = fgb::as_stream(stream);
  const __nv_bfloat16* w = static_cast<const __nv_bfloat16*>(panel);
  const __nv_bfloat16* v = static_cast<const __nv_bfloat16*>(vpanel);
  const __nv_bfloat16* x = static_cast<const __nv_bfloat16*>(X);
  __nv_bfloat16* zb = static_cast<__nv_bfloat16*>(Zb);
  unsigned kx = (unsigned)((K + fgb::kBT - 1) / fgb::kBT);
  if ((phases & 1) && op.num_items > 0) {
    if (zero_z) FGB_CUDA_TRY(cudaMemsetAsync(Z, 0, sizeof(float) * d->num_zrows * (size_t)K, s));
    const int mt = d->max_group_tiles;
    fgb::phaseA_kn_bf16<<<(unsigned)(op.num_items * mt * kx), 128, 0, s>>>(op, v, x, K, Z, K, K, mt);
    FGB_LAUNCH_CHECK("phaseA_kn_bf16");
    long long nz = d->num_zrows * (long long)K;
    fgb::f32_to_bf16_kernel<<<fgb::grid_for(nz, 256), 256, 0, s>>>(Z, zb, nz);
    FGB_LAUNCH_CHECK("f32_to_bf16_kernel");
  }
  if ((phases & 2) && op.num_tiles > 0) {
    fgb::phaseB_kn_bf16<<<(unsigned)(op.num_tiles * kx), 128, 0, s>>>(op, w, x, K, zb, K, Y, K, K,
                                                                       add, K, alpha);
    FGB_LAUNCH_CHECK("phaseB_kn_bf16");
  }
  return FGB_OK;
}

#define FGB_PANEL_BUILD(NAME, TI, TO)                                                         \
  int NAME(const TI* pool, long long num_rows, const long long* pair_p0,                     \
           const long long* pair_w, const int* pair_m, const long long* pair_shift,          \
           const int* pair_k, long long num_pairs, void* panel, void* stream) {              \
    if (num_rows <= 0) return FGB_OK;                                                         \
    fgb::build_panel_kernel<TI, TO><<<fgb::grid_for(num_rows * 32, 256, 152LL * 64), 256, 0, \
                                       fgb::as_stream(stream)>>>(                             \
        pool, num_rows, pair_p0, pair_w, pair_m, pair_shift, pair_k, num_pairs,              \
        static_cast<TO*>(panel));                                                             \
    FGB_LAUNCH_CHECK("build_panel_kernel");                                                  \
    return FGB_OK;                                                                            \
  }
FGB_PANEL_BUILD(fgb_build_panel_f32_f32, float, float)
FGB_PANEL_BUILD(fgb_build_panel_f32_bf16, float, __nv_bfloat16)
FGB_PANEL_BUILD(fgb_build_panel_f64_f64, double, double)
FGB_PANEL_BUILD(fgb_build_panel_f64_f32, double, float)
FGB_PANEL_BUILD(fgb_build_panel_f64_bf16, double, __nv_bfloat16)

#define FGB_VPANEL_BUILD(NAME, TI, TO)                                                          \
  int NAME(const TI* pool, long long num_rows, const long long* row_src,                       \
           const long long* row_dst, const int* row_n, void* vpanel, void* stream) {           \
    if (num_rows <= 0) return FGB_OK;                                                           \
    fgb::build_vpanel_kernel<TI, TO><<<fgb::grid_for(num_rows * 32, 256, 152LL * 64), 256, 0,  \
                                        fgb::as_stream(stream)>>>(                              \
        pool, num_rows, row_src, row_dst, row_n, static_cast<TO*>(vpanel));                     \
    FGB_LAUNCH_CHECK("build_vpanel_kernel");                                                   \
    return FGB_OK;                                                                              \
  }
FGB_VPANEL_BUILD(fgb_build_vpanel_f32_f32, float, float)
FGB_VPANEL_BUILD(fgb_build_vpanel_f32_bf16, float, __nv_bfloat16)
FGB_VPANEL_BUILD(fgb_build_vpanel_f64_f64, double, double)
FGB_VPANEL_BUILD(fgb_build_vpanel_f64_f32, double, float)
FGB_VPANEL_BUILD(fgb_build_vpanel_f64_bf16, double, __nv_bfloat16)

}  // extern "C"
