// Fused form-factor pair kernel -> CSR (replaces the Python row loop of
// get_form_factor_matrix, src/flux/form_factors.py:45-72).
//
// Work is described by tiles: tile t covers rows I[row0 .. row0+nrows) and
// columns J[col0 .. col0+ncols).  get_form_factor_matrix is one tile; the
// compressed operator's near-field blocks are many tiles.
//
// Pass 1 (fgb_ff_count_*): one warp per 32 columns of one tile row: each
//   lane evaluates the orientation numerator, threshold and visibility ray
//   of one pair; the ballot of visible-and-kept pairs is stored as one
//   32-bit word of a bitmask and its popcount added to the row's count.
// Pass 2 (fgb_ff_fill_*): one warp per tile row walks the row's bitmask
//   words, recomputes the value of each set bit (no ray) and writes CSR
//   entries in column order at indptr[row] + rank of the bit.
// The caller scans the counts into indptr between the passes.
#include "common.cuh"
#include "ffentry.cuh"

namespace fgb {
BvhView view_of(const void* handle);

namespace {

struct TileArgs {
  const long long* row0;
  const long long* nrows;
  const long long* col0;
  const long long* ncols;
  const long long* word_off;  // exclusive prefix of nrows * ceil(ncols/32), length T+1
  const long long* row_off;   // exclusive prefix of nrows, length T+1
  long long T;
};

__device__ __forceinline__ long long find_tile(const long long* off, long long T, long long x) {
  long long lo = 0, hi = T - 1;
  while (lo < hi) {
    long long mid = (lo + hi + 1) >> 1;
    if (off[mid] <= x) lo = mid; else hi = mid - 1;
  }
  return lo;
}

template <class R>
__global__ void ff_count_kernel(BvhView b, const R* __restrict__ P, const R* __restrict__ N,
                                const R* __restrict__ A, const long long* __restrict__ I,
                                const long long* __restrict__ J, TileArgs ta, R eps, int sem,
                                unsigned* __restrict__ bits, int* __restrict__ row_cnt,
                                unsigned long long* __restrict__ stats,
                                unsigned* __restrict__ flags) {
  const int lane = threadIdx.x & 31;
  const long long warps_total = (long long)gridDim.x * (blockDim.x >> 5);
  const long long W = ta.word_off[ta.T];
  for (long long w = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5; w < W; w += warps_total) {
    long long t = find_tile(ta.word_off, ta.T, w);
    long long ncols = ta.ncols[t];
    long long wpr = (ncols + 31) >> 5;
    long long local = w - ta.word_off[t];
    long long r = local / wpr, wc = local % wpr;
    long long col = wc * 32 + lane;
    bool vis = false, kept = false, ne = false, of = false;
    if (col < ncols) {
      long long i = I[ta.row0[t] + r];
      long long j = J[ta.col0[t] + col];
      // an entry is stored whenever the pair is kept and visible
      // (form_factors.py:50-70)
      if (i != j) {
        R num = ff_num(P, N, i, j);
        if (fabs(num) > eps) {
          kept = true;
          vis = pair_visible<R>(b, P, (int)i, (int)j, sem, &ne, &of);
        }
      }
    }
    unsigned word = __ballot_sync(0xffffffffu, vis);
    unsigned kept_w = __ballot_sync(0xffffffffu, kept);
    unsigned ne_w = __ballot_sync(0xffffffffu, ne);
    if (of) atomicOr(flags, kFlagStackOverflow);
    if (lane == 0) {
      bits[w] = word;
      if (word) atomicAdd(&row_cnt[ta.row_off[t] + r], __popc(word));
      if (kept_w) atomicAdd(&stats[0], (unsigned long long)__popc(kept_w));
      if (ne_w) atomicAdd(&stats[1], (unsigned long long)__popc(ne_w));
    }
  }
}

template <class R, class IDX, class RO>
__global__ void ff_fill_kernel(const R* __restrict__ P, const R* __restrict__ A,
                               const R* __restrict__ N, const long long* __restrict__ I,
                               const long long* __restrict__ J, TileArgs ta,
                               const unsigned* __restrict__ bits,
                               const long long* __restrict__ indptr, IDX* __restrict__ indices,
                               RO* __restrict__ data) {
  const int lane = threadIdx.x & 31;
  const long long warps_total = (long long)gridDim.x * (blockDim.x >> 5);
  const long long rows_total = ta.row_off[ta.T];
  const unsigned lt = (1u << lane) - 1u;
  for (long long g = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5; g < rows_total;
       g += warps_total) {
    long long t = find_tile(ta.row_off, ta.T, g);
    long long r = g - ta.row_off[t];
    long long ncols = ta.ncols[t];
    long long wpr = (ncols + 31) >> 5;
    const unsigned* rb = bits + ta.word_off[t] + r * wpr;
    long long pos = indptr[g];
    long long i = I[ta.row0[t] + r];
    for (long long wc = 0; wc < wpr; wc++) {
      unsigned word = rb[wc];
      if (!word) continue;
      if ((word >> lane) & 1u) {
        long long col = wc * 32 + lane;
        long long j = J[ta.col0[t] + col];
        R num = ff_num(P, N, i, j);
        long long q = pos + __popc(word & lt);
        indices[q] = (IDX)col;
        data[q] = (RO)ff_value(P, A, i, j, num);
      }
      pos += __popc(word);
    }
  }
}

int check_tiles(const void* bvh, long long T) {
  if (!bvh) { set_error("null BVH handle"); return FGB_BAD_ARG; }
  if (T < 1) { set_error("need at least one tile"); return FGB_BAD_ARG; }
  return FGB_OK;
}

template <class R>
int ff_count(const void* bvh, const R* P, const R* N, const R* A, const long long* I,
             const long long* J, const long long* row0, const long long* nrows,
             const long long* col0, const long long* ncols, const long long* word_off,
             const long long* row_off, long long T, long long total_words, R eps, int sem,
             unsigned* bits, int* row_cnt, unsigned long long* stats, unsigned* flags,
             void* stream) {
  int st = check_tiles(bvh, T);
  if (st) return st;
  if (total_words == 0) return FGB_OK;
  TileArgs ta{row0, nrows, col0, ncols, word_off, row_off, T};
  long long threads = total_words * 32;
  ff_count_kernel<R><<<grid_for(threads, 128, 152LL * 64), 128, 0, as_stream(stream)>>>(
      view_of(bvh), P, N, A, I, J, ta, eps, sem, bits, row_cnt, stats, flags);
  FGB_LAUNCH_CHECK("ff_count_kernel");
  return FGB_OK;
}

template <class R, class IDX, class RO>
int ff_fill(const R* P, const R* N, const R* A, const long long* I, const long long* J,
            const long long* row0, const long long* nrows, const long long* col0,
            const long long* ncols, const long long* word_off, const long long* row_off,
            long long T, long long total_rows, const unsigned* bits, const long long* indptr,
            IDX* indices, RO* data, void* stream) {
  if (T < 1) { set_error("need at least one tile"); return FGB_BAD_ARG; }
  if (total_rows == 0) return FGB_OK;
  TileArgs ta{row0, nrows, col0, ncols, word_off, row_off, T};
  ff_fill_kernel<R, IDX, RO><<<grid_for(total_rows * 32, 128, 152LL * 64), 128, 0, as_stream(stream)>>>(
      P, A, N, I, J, ta, bits, indptr, indices, data);
  FGB_LAUNCH_CHECK("ff_fill_kernel");
  return FGB_OK;
}

}  // namespace
}  // namespace fgb

extern "C" {

int fgb_ff_count_f64(const void* bvh, const double* P, const double* N, const double* A,
                     const long long* I, const long long* J, const long long* row0,
                     const long long* nrows, const long long* col0, const long long* ncols,
                     const long long* word_off, const long long* row_off, long long num_tiles,
                     long long total_words, double eps, int semantics, unsigned* bits,
                     int* row_counts, unsigned long long* stats, unsigned* flags, void* stream) {
  return fgb::ff_count<double>(bvh, P, N, A, I, J, row0, nrows, col0, ncols, word_off, row_off,
                               num_tiles, total_words, eps, semantics, bits, row_counts, stats,
                               flags, stream);
}

int fgb_ff_count_f32(const void* bvh, const float* P, const float* N, const float* A,
                     const long long* I, const long long* J, const long long* row0,
                     const long long* nrows, const long long* col0, const long long* ncols,
                     const long long* word_off, const long long* row_off, long long num_tiles,
                     long long total_words, float eps, int semantics, unsigned* bits,
                     int* row_counts, unsigned long long* stats, unsigned* flags, void* stream) {
  return fgb::ff_count<float>(bvh, P, N, A, I, J, row0, nrows, col0, ncols, word_off, row_off,
                              num_tiles, total_words, eps, semantics, bits, row_counts, stats,
                              flags, stream);
}

int fgb_ff_fill_f64(const double* P, const double* N, const double* A, const long long* I,
                    const long long* J, const long long* row0, const long long* nrows,
                    const long long* col0, const long long* ncols, const long long* word_off,
                    const long long* row_off, long long num_tiles, long long total_rows,
                    const unsigned* bits, const long long* indptr, int* indices, double* data,
                    void* stream) {
  return fgb::ff_fill<double, int, double>(P, N, A, I, J, row0, nrows, col0, ncols, word_off,
                                           row_off, num_tiles, total_rows, bits, indptr, indices,
                                           data, stream);
}

int fgb_ff_fill_f64_to_f32(const double* P, const double* N, const double* A, const long long* I,
                           const long long* J, const long long* row0, const long long* nrows,
                           const long long* col0, const long long* ncols,
                           const long long* word_off, const long long* row_off,
                           long long num_tiles, long long total_rows, const unsigned* bits,
                           const long long* indptr, int* indices, float* data, void* stream) {
  return fgb::ff_fill<double, int, float>(P, N, A, I, J, row0, nrows, col0, ncols, word_off,
                                          row_off, num_tiles, total_rows, bits, indptr, indices,
                                          data, stream);
}

int fgb_ff_fill_f32(const float* P, const float* N, const float* A, const long long* I,
                    const long long* J, const long long* row0, const long long* nrows,
                    const long long* col0, const long long* ncols, const long long* word_off,
                    const long long* row_off, long long num_tiles, long long total_rows,
                    const unsigned* bits, const long long* indptr, int* indices, float* data,
                    void* stream) {
  return fgb::ff_fill<float, int, float>(P, N, A, I, J, row0, nrows, col0, ncols, word_off,
                                         row_off, num_tiles, total_rows, bits, indptr, indices,
                                         data, stream);
}

}  // extern "C"
