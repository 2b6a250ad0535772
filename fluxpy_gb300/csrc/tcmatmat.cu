// Phase B of the K-right-hand-side block product on the 5th-generation
// tensor cores (tcgen05.mma, accumulators in tensor memory).
//
// Same operator layout as matvec.cu (phase B): tile t owns 64 operator rows
// and the panel rows [p0, p1) (a multiple of 64 here); panel row l holds 64
// BF16 weights W[l, i] for the tile's rows i and a source index src[l] into
// the stacked source S = [Zb; X] (num_zrows + N rows, K BF16 columns each).
//   Y[t*64 + i, c] = add[., c] + alpha * sum_l W[l, i] S[src[l], c].
// For the tensor core the product is taken transposed, so that the long
// right-hand-side dimension is the MMA's M:
//   D (M = 128 columns of S, N = 64 tile rows) += A (S^T chunk) . B (W chunk)
// with the reduction over panel rows, 16 per MMA.  Both operands are stored
// "MN-major" (their contiguous dimension is M resp. N), in the canonical
// 128-byte-swizzled layout: for each 64-element block along M (or N) the
// K rows are 128-byte lines, eight lines to a 1 KiB swizzle atom, the
// 16-byte chunks of line k permuted by XOR with (k mod 8).
//
// CTA = (tile, slice of NC = 256 right-hand-side columns); 8 warps.  All
// warps gather the next chunks (64 panel rows: W 8 KiB, S 32 KiB) with
// cp.async into a 4-stage ring; thread 0 issues the MMAs of the current
// chunk (4 k-steps x 2 M-halves) and commits them to the stage's mbarrier,
// which the producers wait on before they refill that stage.  The FP32
// accumulators (2 x 64 TMEM columns, 128 lanes) are read back with
// tcgen05.ld by all warps (warp w reads lanes 32 (w mod 4) ..) for the
// epilogue, whose stores are coalesced along the right-hand-side columns.
//
// Every mbarrier wait is bounded (about 2 s of global time); a wait that
// runs out sets FGB_FLAG_DEVICE_TIMEOUT in the caller's flag word and the
// CTA skips the rest of its work, drains its copies and frees its TMEM.
#include "common.cuh"

#include <cuda_bf16.h>

namespace fgb {
namespace {

constexpr int kTcTileRows = 64;   // operator rows per tile (MMA N)
constexpr int kTcChunk = 64;      // panel rows per pipeline stage
constexpr int kTcNC = 256;        // right-hand-side columns per CTA (2 x MMA M)
constexpr int kTcStages = 4;
constexpr int kTcThreads = 256;
constexpr int kTcWBytes = kTcChunk * kTcTileRows * 2;          // 8 KiB
constexpr int kTcSBytes = kTcChunk * kTcNC * 2;                // 32 KiB
constexpr int kTcStageBytes = kTcWBytes + kTcSBytes;           // 40 KiB
constexpr int kTcSmemBytes = kTcStages * kTcStageBytes + 1024; // + alignment slack
constexpr int kTcTmemCols = 128;                               // 2 accumulators x 64
constexpr unsigned long long kWaitNs = 2000000000ull;          // 2 s

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void cp_async16_zfill(uint32_t s, const void* g, bool pred) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(g),
               "r"(pred ? 16 : 0));
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }
__device__ __forceinline__ void cp_wait_all() { asm volatile("cp.async.wait_all;\n" ::); }

__device__ __forceinline__ void mbar_init(uint32_t bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok) : "r"(bar), "r"(parity) : "memory");
  return ok != 0;
}
// Bounded wait for the completion of the phase with the given parity.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  if (mbar_try(bar, parity)) return true;
  const unsigned long long t0 = global_ns();
  while (true) {
    if (mbar_try(bar, parity)) return true;
    if (global_ns() - t0 > kWaitNs) return false;
  }
}

// tcgen05 shared-memory matrix descriptor: start address, leading and stride
// byte offsets (16-byte units), the fixed version bits 46-48 = 0b001 and the
// layout type in bits 61-63 (2 = 128-byte swizzle).
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46) | (2ull << 61);
}
// Instruction descriptor, kind::f16: D FP32 (bits 4-5 = 1), A and B BF16
// (bits 7-9, 10-12 = 1), A and B MN-major (bits 15, 16), N >> 3 in bits
// 17-22, M >> 4 in bits 24-28.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | (1u << 15) | (1u << 16) |
                            ((uint32_t)(kTcTileRows >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);

__device__ __forceinline__ void mma_bf16_tc(uint32_t dtmem, uint64_t adesc, uint64_t bdesc,
                                            uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
      ::"r"(dtmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate) : "memory");
}
__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
               ::"r"(bar) : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// 32 consecutive TMEM columns of this warp's 32 lanes -> 32 registers.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
      "%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
        "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

struct TcPhaseB {
  const long long* t_p0;
  const int* src;
  long long num_tiles;
  long long N;
  long long num_zrows;
};

__global__ void __launch_bounds__(kTcThreads, 1)
phaseB_tc_bf16(TcPhaseB op, const __nv_bfloat16* __restrict__ panel,
               const __nv_bfloat16* __restrict__ X, const __nv_bfloat16* __restrict__ Zb,
               long long lds, float* __restrict__ Y, long long ldy, int K,
               const float* __restrict__ add_mat, long long ld_add, float alpha,
               unsigned* __restrict__ flags) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ __align__(8) unsigned long long bars[kTcStages + 1];
  __shared__ uint32_t tmem_slot;
  __shared__ int abort_flag;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nks = (K + kTcNC - 1) / kTcNC;
  const long long t = blockIdx.x / nks;
  const int c_base = (int)(blockIdx.x % nks) * kTcNC;
  const long long p0 = op.t_p0[t], p1 = op.t_p0[t + 1];
  const int nch = (int)((p1 - p0) / kTcChunk);
  if (tid == 0 && ((p1 - p0) % kTcChunk) != 0) atomicOr(flags, FGB_FLAG_INDEX_RANGE);

  uint8_t* smem = reinterpret_cast<uint8_t*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const uint32_t sbase = smem_addr(smem);
  if (tid == 0) {
    for (int s = 0; s <= kTcStages; s++) mbar_init(smem_addr(&bars[s]), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    abort_flag = 0;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 ::"r"(smem_addr(&tmem_slot)), "r"(kTcTmemCols) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;

  // producer: chunk c -> stage s (W: rows k = tid / 8 .. , 16-byte piece
  // tid % 8; S: rows k = warp + 8 j, pieces lane (8 bf16 columns each))
  auto load = [&](int c, int s) {
    const uint32_t wst = sbase + s * kTcStageBytes;
    const uint32_t sst = wst + kTcWBytes;
    const long long l0 = p0 + (long long)c * kTcChunk;
#pragma unroll
    for (int j = 0; j < (kTcChunk * 8) / kTcThreads; j++) {
      const int p = tid + j * kTcThreads;
      const int k = p >> 3, q = p & 7;
      const __nv_bfloat16* g = panel + (l0 + k) * kTcTileRows + q * 8;
      cp_async16_zfill(wst + k * 128 + ((q ^ (k & 7)) << 4), g, true);
    }
#pragma unroll
    for (int j = 0; j < kTcChunk / 8; j++) {
      const int k = warp + 8 * j;
      const int sidx = op.src[l0 + k];
      const __nv_bfloat16* row = sidx < op.num_zrows ? Zb + (long long)sidx * lds
                                                     : X + (long long)(sidx - op.num_zrows) * lds;
      const int col = c_base + lane * 8;          // 32 pieces x 8 = 256 columns
      const int b = lane >> 3, q = lane & 7;       // 64-column block, piece in block
      const bool ok = col < K;
      cp_async16_zfill(sst + b * (kTcChunk * 128) + k * 128 + ((q ^ (k & 7)) << 4),
                       ok ? row + col : row, ok);
    }
  };

  for (int c = 0; c < kTcStages - 1; c++) {
    if (c < nch) load(c, c);
    cp_commit();
  }
  bool ok = true;
  for (int c = 0; c < nch; c++) {
    const int s = c % kTcStages;
    cp_wait<kTcStages - 2>();
    fence_proxy_async();
    __syncthreads();
    if (abort_flag) { ok = false; break; }
    if (tid == 0) {
      tc_fence_after();
      const uint32_t wst = sbase + s * kTcStageBytes;
      const uint32_t sst = wst + kTcWBytes;
#pragma unroll
      for (int q = 0; q < kTcChunk / 16; q++) {
        // 16 panel rows = two 8-line groups (SBO 1 KiB); k-step offset 2 KiB
        const uint64_t bdesc = sw128_desc(wst + q * 2048, 8192, 1024);
#pragma unroll
        for (int a = 0; a < kTcNC / 128; a++) {
          // M = 128 columns = two 64-column blocks, LBO = block stride
          const uint64_t adesc = sw128_desc(sst + a * 2 * (kTcChunk * 128) + q * 2048,
                                            kTcChunk * 128, 1024);
          mma_bf16_tc(tmem + a * kTcTileRows, adesc, bdesc, kIdesc, (c | q) != 0);
        }
      }
      mma_commit(smem_addr(&bars[s]));
    }
    const int cn = c + kTcStages - 1;
    if (cn < nch) {
      if (c >= 1) {
        const int sp = (c - 1) % kTcStages;
        if (!mbar_wait(smem_addr(&bars[sp]), ((c - 1) / kTcStages) & 1)) {
          atomicOr(flags, FGB_FLAG_DEVICE_TIMEOUT);
          abort_flag = 1;
        }
      }
      if (!abort_flag) load(cn, cn % kTcStages);
    }
    cp_commit();
  }
  cp_wait_all();
  // all MMAs of this CTA complete (they finish in order): last chunk's barrier
  if (nch > 0 && ok) {
    const int cl = nch - 1;
    if (!mbar_wait(smem_addr(&bars[cl % kTcStages]), (cl / kTcStages) & 1)) {
      atomicOr(flags, FGB_FLAG_DEVICE_TIMEOUT);
      ok = false;
    }
  }
  tc_fence_after();
  __syncthreads();
  if (abort_flag) ok = false;

  // epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31 = columns
  // c_base + 128 a + 32 (w % 4) + lane, for a = w / 4
  if (ok) {
    const int quarter = warp & 3, a = warp >> 2;
    const int col = c_base + a * 128 + quarter * 32 + lane;
#pragma unroll
    for (int h = 0; h < kTcTileRows / 32; h++) {
      float v[32];
      if (nch > 0) {
        tmem_ld32(tmem + ((uint32_t)(quarter * 32) << 16) + a * kTcTileRows + h * 32, v);
      } else {
#pragma unroll
        for (int i = 0; i < 32; i++) v[i] = 0.f;
      }
      if (col < K) {
#pragma unroll
        for (int i = 0; i < 32; i++) {
          const long long row = t * kTcTileRows + h * 32 + i;
          if (row < op.N) {
            float y = v[i];
            if (add_mat) y = add_mat[row * ld_add + col] + alpha * y;
            Y[row * ldy + col] = y;
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;"
                 ::"r"(tmem), "r"(kTcTmemCols) : "memory");
  }
}

}  // namespace
}  // namespace fgb

extern "C" {

int fgb_matmat_bf16_tc_phase_b(const struct fgb_op_desc* d, const void* panel, const void* X,
                               const void* Zb, float* Y, int K, const float* add, float alpha,
                               unsigned* flags, void* stream) {
  if (!d || !flags) { fgb::set_error("null operator or flags"); return FGB_BAD_ARG; }
  if (K < 8 || (K % 8) != 0) { fgb::set_error("K must be a positive multiple of 8"); return FGB_BAD_ARG; }
  if ((reinterpret_cast<uintptr_t>(X) & 15) || (reinterpret_cast<uintptr_t>(Zb) & 15) ||
      (reinterpret_cast<uintptr_t>(panel) & 15)) {
    fgb::set_error("X, Zb and the panel must be 16-byte aligned");
    return FGB_BAD_ARG;
  }
  if (d->num_tiles <= 0) return FGB_OK;
  static bool attr_set = false;
  if (!attr_set) {
    FGB_CUDA_TRY(cudaFuncSetAttribute(fgb::phaseB_tc_bf16,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      fgb::kTcSmemBytes));
    attr_set = true;
  }
  fgb::TcPhaseB op{d->t_p0, d->src, d->num_tiles, d->N, d->num_zrows};
  const long long nks = (K + fgb::kTcNC - 1) / fgb::kTcNC;
  const long long grid = d->num_tiles * nks;
  if (grid > 0x7fffffffLL) { fgb::set_error("grid too large"); return FGB_BAD_ARG; }
  fgb::phaseB_tc_bf16<<<(unsigned)grid, fgb::kTcThreads, fgb::kTcSmemBytes,
                        fgb::as_stream(stream)>>>(
      op, static_cast<const __nv_bfloat16*>(panel), static_cast<const __nv_bfloat16*>(X),
      static_cast<const __nv_bfloat16*>(Zb), K, Y, K, K, add, K, alpha, flags);
  FGB_LAUNCH_CHECK("phaseB_tc_bf16");
  return FGB_OK;
}

}  // extern "C"
