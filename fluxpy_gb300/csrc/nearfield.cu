// Near-field (exact leaf) panels of the compressed operator, built directly
// from the sparse output of the form-factor pair kernel (formfactor.cu), so
// that no dense copy of the exact leaves ever exists.
//
// For an exact leaf q (cluster rows [r0, r0+m), columns [c0, c0+n)) the
// pair kernel leaves a visible-pair bitmask (m rows x wpr 32-bit words, at
// word_off[q]) and CSR rows (row_off[q] + i) with values.  For every 64-row
// tile t that overlaps the leaf, the phase-B panel gets one row per column j
// that is nonzero for at least one of the tile's rows (column compaction):
//   1. fgb_nf_pair_masks: OR of the tile's row masks -> pair mask + count;
//   2. fgb_nf_enumerate:  one row descriptor (pair, column) per set bit, in
//                         column order, at the pair's first descriptor slot;
//                         the host then merges the descriptors of a tile that
//                         gather the same source column into one panel row;
//   3. fgb_nf_fill_*:     each descriptor writes its leaf's rows of its panel
//                         row: value (i, j) looked up in the CSR by the rank of
//                         bit j in row i's mask.
#include "common.cuh"

#include <cuda_bf16.h>

namespace fgb {
namespace {

constexpr int kTile = 64;

struct NfPairs {
  const int* q;            // exact leaf of the pair
  const long long* t0;     // first row (cluster order) of the pair's tile
  const long long* moff;   // offset of the pair's mask words
  long long num_pairs;
};

struct NfLeaves {
  const long long* r0;
  const int* m;
  const int* wpr;          // words per row
  const long long* word_off;
  const long long* row_off;
};

template <class TO> __device__ __forceinline__ TO to_out(double v) { return (TO)v; }
template <> __device__ __forceinline__ __nv_bfloat16 to_out<__nv_bfloat16>(double v) {
  return __float2bfloat16((float)v);
}

__device__ __forceinline__ long long find_pair(const long long* off, long long n, long long x) {
  long long lo = 0, hi = n - 1;
  while (lo < hi) {
    long long mid = (lo + hi + 1) >> 1;
    if (off[mid] <= x) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// One thread per (pair, mask word).
__global__ void nf_pair_masks_kernel(NfPairs P, NfLeaves L, const unsigned* __restrict__ bits,
                                     long long total_words, unsigned* __restrict__ mask,
                                     int* __restrict__ count) {
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total_words;
       g += (long long)gridDim.x * blockDim.x) {
    const long long p = find_pair(P.moff, P.num_pairs, g);
    const long long w = g - P.moff[p];
    const int q = P.q[p];
    const long long r0 = L.r0[q];
    const int m = L.m[q], wpr = L.wpr[q];
    const long long lo = max(P.t0[p], r0), hi = min(P.t0[p] + kTile, r0 + (long long)m);
    unsigned acc = 0u;
    for (long long r = lo; r < hi; r++) acc |= bits[L.word_off[q] + (r - r0) * wpr + w];
    mask[g] = acc;
    if (acc) atomicAdd(&count[p], __popc(acc));
  }
}

// One warp per pair: row descriptors (pair, column) for every set bit, in
// column order, starting at desc_off[p].
__global__ void nf_enumerate_kernel(NfPairs P, NfLeaves L, const unsigned* __restrict__ mask,
                                    const long long* __restrict__ desc_off,
                                    int* __restrict__ desc_pair, int* __restrict__ desc_col) {
  const int lane = threadIdx.x & 31;
  const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long p = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5; p < P.num_pairs;
       p += warps) {
    const int wpr = L.wpr[P.q[p]];
    long long pos = desc_off[p];
    for (int w0 = 0; w0 < wpr; w0 += 32) {
      const int w = w0 + lane;
      const unsigned word = w < wpr ? mask[P.moff[p] + w] : 0u;
      const int c = __popc(word);
      int incl = c;
      for (int o = 1; o < 32; o <<= 1) {
        int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
      }
      const int excl = incl - c;
      unsigned wb = word;
      int k = 0;
      while (wb) {
        const int b = __ffs(wb) - 1;
        wb &= wb - 1;
        desc_pair[pos + excl + k] = (int)p;
        desc_col[pos + excl + k] = w * 32 + b;
        k++;
      }
      pos += __shfl_sync(0xffffffffu, incl, 31);
    }
  }
}

// One warp per descriptor: 64 weights of column col for the pair's tile.
template <class TI, class TO>
__global__ void nf_fill_kernel(NfPairs P, NfLeaves L, const unsigned* __restrict__ bits,
                               const long long* __restrict__ indptr, const TI* __restrict__ data,
                               const int* __restrict__ desc_pair, const int* __restrict__ desc_col,
                               const long long* __restrict__ desc_row, long long num_desc,
                               TO* __restrict__ panel) {
  const int lane = threadIdx.x & 31;
  const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long d = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5; d < num_desc;
       d += warps) {
    const long long p = desc_pair[d];
    const int col = desc_col[d];
    const int q = P.q[p];
    const long long r0 = L.r0[q];
    const int m = L.m[q], wpr = L.wpr[q];
    const long long t0 = P.t0[p];
    TO* out = panel + desc_row[d] * kTile;
    const int cw = col >> 5;
    const unsigned below = (1u << (col & 31)) - 1u;
    // only the leaf's own rows are written: descriptors of other leaves may
    // share this panel row (the same column, disjoint rows); the rest of
    // the row was zeroed when the panel was built
    for (int i = lane; i < kTile; i += 32) {
      const long long r = t0 + i;
      if (r < r0 || r >= r0 + m) continue;
      TI v = TI(0);
      const unsigned* rb = bits + L.word_off[q] + (r - r0) * wpr;
      const unsigned word = rb[cw];
      if ((word >> (col & 31)) & 1u) {
        int rank = __popc(word & below);
        for (int w = 0; w < cw; w++) rank += __popc(rb[w]);
        v = data[indptr[L.row_off[q] + (r - r0)] + rank];
      }
      out[i] = to_out<TO>((double)v);
    }
  }
}

}  // namespace
}  // namespace fgb

extern "C" {

int fgb_nf_pair_masks(const int* pair_q, const long long* pair_t0, const long long* pair_moff,
                      long long num_pairs, long long total_words, const long long* leaf_r0,
                      const int* leaf_m, const int* leaf_wpr, const long long* leaf_word_off,
                      const long long* leaf_row_off, const unsigned* bits, unsigned* mask,
                      int* count, void* stream) {
  if (num_pairs < 0 || total_words < 0) { fgb::set_error("bad sizes"); return FGB_BAD_ARG; }
  if (total_words == 0) return FGB_OK;
  fgb::NfPairs P{pair_q, pair_t0, pair_moff, num_pairs};
  fgb::NfLeaves L{leaf_r0, leaf_m, leaf_wpr, leaf_word_off, leaf_row_off};
  fgb::nf_pair_masks_kernel<<<fgb::grid_for(total_words, 256), 256, 0, fgb::as_stream(stream)>>>(
      P, L, bits, total_words, mask, count);
  FGB_LAUNCH_CHECK("nf_pair_masks_kernel");
  return FGB_OK;
}

int fgb_nf_enumerate(const int* pair_q, const long long* pair_t0, const long long* pair_moff,
                     long long num_pairs, const int* leaf_wpr, const unsigned* mask,
                     const long long* desc_off, int* desc_pair, int* desc_col, void* stream) {
  if (num_pairs <= 0) return FGB_OK;
  fgb::NfPairs P{pair_q, pair_t0, pair_moff, num_pairs};
  fgb::NfLeaves L{nullptr, nullptr, leaf_wpr, nullptr, nullptr};
  fgb::nf_enumerate_kernel<<<fgb::grid_for(num_pairs * 32, 256, 152LL * 64), 256, 0,
                             fgb::as_stream(stream)>>>(P, L, mask, desc_off, desc_pair, desc_col);
  FGB_LAUNCH_CHECK("nf_enumerate_kernel");
  return FGB_OK;
}

#define FGB_NF_FILL(NAME, TI, TO)                                                                \
  int NAME(const int* pair_q, const long long* pair_t0, long long num_pairs,                    \
           const long long* leaf_r0, const int* leaf_m, const int* leaf_wpr,                    \
           const long long* leaf_word_off, const long long* leaf_row_off, const unsigned* bits, \
           const long long* indptr, const TI* data, const int* desc_pair, const int* desc_col,  \
           const long long* desc_row, long long num_desc, void* panel, void* stream) {          \
    if (num_desc <= 0) return FGB_OK;                                                            \
    fgb::NfPairs P{pair_q, pair_t0, nullptr, num_pairs};                                          \
    fgb::NfLeaves L{leaf_r0, leaf_m, leaf_wpr, leaf_word_off, leaf_row_off};                      \
    fgb::nf_fill_kernel<TI, TO><<<fgb::grid_for(num_desc * 32, 256, 152LL * 64), 256, 0,          \
                                   fgb::as_stream(stream)>>>(P, L, bits, indptr, data, desc_pair, \
                                                             desc_col, desc_row, num_desc,        \
                                                             static_cast<TO*>(panel));            \
    FGB_LAUNCH_CHECK("nf_fill_kernel");                                                          \
    return FGB_OK;                                                                                \
  }
FGB_NF_FILL(fgb_nf_fill_f32_f32, float, float)
FGB_NF_FILL(fgb_nf_fill_f32_bf16, float, __nv_bfloat16)
FGB_NF_FILL(fgb_nf_fill_f64_f64, double, double)
FGB_NF_FILL(fgb_nf_fill_f64_f32, double, float)
FGB_NF_FILL(fgb_nf_fill_f64_bf16, double, __nv_bfloat16)

}  // extern "C"
