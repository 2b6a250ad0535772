// The K-right-hand-side block product of the compressed operator on the
// 5th-generation tensor cores (tcgen05.mma, FP32 accumulators in tensor
// memory), for both phases of the panel layout of matvec.cu:
//
//   phase B (row tiles): tile t owns R operator rows (R = 64, or 128 for the
//     re-tiled BF16 panel) and the panel rows [p0, p1) (a multiple of 64);
//     panel row l holds R BF16 weights W[l, i] for the tile's rows i and a
//     source index src[l] into S = [Z; X]:
//       Y[t*R + i, c] = add[., c] + alpha * sum_l W[l, i] S[src[l], c];
//   phase A (low-rank groups): group g (kz stacked V^T rows, columns
//     [c0, c0 + n)) is stored transposed, Vt[j, r], and work slice s of an
//     item (columns [j0, j1) of the group) computes
//       Z[z0 + 128 s + r, c] (+)= sum_j Vt[j, 128 s + r] X[c0 + j, c].
//
// Both are one "gather GEMM" with the reduction over rows l (panel rows, or
// group columns j): the product is taken transposed so that the long
// right-hand-side dimension is the MMA's M,
//   D (M = 128 columns of S, N = NR output rows) += A (S^T chunk) . B (W chunk),
// 16 reduction rows per MMA.  Both operands are stored "MN-major" (their
// contiguous dimension is M resp. N) in the canonical 128-byte-swizzled
// layout: per 64-element block along M (or N) the reduction rows are
// 128-byte lines, eight lines to a 1 KiB swizzle atom, the 16-byte chunks of
// line k permuted by XOR with (k mod 8).
//
// Split mode: each FP32 operand v is given as hi = bf16(v), lo = bf16(v -
// hi); the chunk loads W_hi, W_lo, S_hi, S_lo and issues three MMAs per
// k-step into the same accumulator, hi.hi + lo.hi + hi.lo (the lo.lo term is
// below 2^-16 relative and dropped).
//
// CTA = (tile or work slice, slice of NC right-hand-side columns), 8 warps,
// shapes per mode in TcCfg.  All warps gather the next chunks (CH reduction
// rows) with cp.async into a ring of stages (up to 200 KiB); thread 0 issues
// the MMAs of the current chunk and commits them to the stage's mbarrier,
// which the producers wait on before they refill that stage.  The
// accumulators (NC / 128 halves of NR TMEM columns, 128 lanes; two sets in
// split mode) are read back with tcgen05.ld (warp w reads lanes 32 (w mod 4)
// ..) for an epilogue whose stores are coalesced along the right-hand-side
// columns.
//
// Every mbarrier wait is bounded (about 2 s of global time); a wait that
// runs out sets FGB_FLAG_DEVICE_TIMEOUT in the caller's flag word and the
// CTA skips the rest of its work, drains its copies and frees its TMEM.
#include "common.cuh"

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

namespace fgb {
namespace {

constexpr int kTcRows = 64;        // rows of a phase-B tile
constexpr int kTcThreads = 256;
// split mode: the tensor core's FP32 accumulation loses up to ~2^-23 of the
// running sum per MMA, which over thousands of reduction steps exceeds the
// split operands' 2^-16 accuracy; every kTcWin chunks (256 reduction rows,
// 48 MMAs) the window's accumulators are drained into registers and summed
// there with Kahan compensation.  At 522k facets and 1,024 columns windows
// of 2, 4 and 8 chunks gave the same product error (6e-6 of max |F x|
// against FP64) and took 135, 130 and 127 ms for the split product.
constexpr int kTcWin = 8;
constexpr unsigned long long kWaitNs = 2000000000ull;           // 2 s

enum { kModeA = 0, kModeB = 1 };

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
// layout type in bits 61-63 (2 = 128-byte swizzle).  For these MN-major
// operands the leading offset is the stride between 64-element blocks along
// M / N and the stride offset the stride between 8-line groups along the
// reduction.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46) | (2ull << 61);
}
// Instruction descriptor, kind::f16: D FP32 (bits 4-5 = 1), A and B BF16
// (bits 7-9, 10-12 = 1), A and B MN-major (bits 15, 16), N >> 3 in bits
// 17-22, M >> 4 in bits 24-28 (here N = 64, M = 128; the per-mode shapes of
// tc_gather_gemm build their own).
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | (1u << 15) | (1u << 16) |
                            ((uint32_t)(kTcRows >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);

__device__ __forceinline__ void mma_bf16_tc(uint32_t dtmem, uint64_t adesc, uint64_t bdesc,
                                            uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
      ::"r"(dtmem), "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate) : "memory");
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

struct TcArgs {
  // phase B
  const long long* t_p0;
  const int* src;
  long long N;
  long long num_zrows;
  // phase A
  const int* a_grp;
  const int* a_j0;
  const int* a_j1;
  const unsigned char* a_excl;
  const long long* a_woff;
  const int* a_witem;      // work slice -> item (optional)
  long long num_items;
  const int* g_c0;
  const int* g_kz;
  const int* g_kzp;
  const long long* g_vtoff;
  const long long* g_z0;
  // operands (lo: split mode only)
  const __nv_bfloat16* w_hi;
  const __nv_bfloat16* w_lo;
  const __nv_bfloat16* x_hi;
  const __nv_bfloat16* x_lo;
  const __nv_bfloat16* z_hi;
  const __nv_bfloat16* z_lo;
  long long lds;           // row stride of X and Z (= K)
  int K;
  float* out;              // Y (phase B) or Z (phase A), row stride K
  // phase A with BF16 output: Z written as hi (and lo) BF16 parts instead of
  // FP32 (every work item must cover its whole group)
  __nv_bfloat16* zout_hi;
  __nv_bfloat16* zout_lo;
  const float* add;
  float alpha;
  unsigned* flags;
  // phase B: the sources as one row-major tensor S = [Z; X] (hi, and lo),
  // when X follows Z in memory (one base pointer for every gathered row);
  // null otherwise
  const __nv_bfloat16* s_hi;
  const __nv_bfloat16* s_lo;
  // phase B: the tile of work unit u is tile_order[u] (null: u)
  const int* tile_order;
};

__device__ __forceinline__ void kahan_add(float& s, float& c, float x) {
  const float y = __fsub_rn(x, c);
  const float t = __fadd_rn(s, y);
  c = __fsub_rn(__fsub_rn(t, s), y);
  s = t;
}

// Per-mode shapes.  NR = output rows per CTA (MMA N), NC = right-hand-side
// columns per CTA (a multiple of the MMA M = 128), CH = reduction rows per
// stage.  Phase A computes 128 rows of Z per CTA, so that each gathered X
// row feeds twice the flops; phase B runs 128-row tiles for the plain BF16
// product (the re-tiled panel) and the 64-row tiles for the split one;
// 256-row tiles (MMA N = 256, two CTAs per SM: 256 TMEM columns each) are
// the plain product's widest layout.
// Split mode keeps SEGS x 32 sums per thread (32 for 64-row tiles or
// slices, compensated; 64 for 128-row ones, plain FP32).
// CTAS = CTAs per SM the shape is built for.  The plain products run four
// (NC = 128, CH = 32, a 3-stage ring of 16 KiB stages): each CTA's loop
// waits, per chunk, for its copies and for the previous chunk's MMAs, and
// per work item for its TMEM allocation and epilogue; the other CTAs fill
// those waits.  At 522k facets and 1,024 columns this measured 44 ms for
// phase B and 31 ms for phase A, against 53 and 51 ms for one CTA per SM
// with NC = 256, CH = 64 and a 4-stage ring (the median phase-A group has
// 62 columns: one or two chunks per work item).  The split products run two
// CTAs per SM: on 64-row tiles / slices with 32 compensated sums per thread
// (~120 registers), on 128-row ones with 64 plain FP32 sums (128).
// right-hand-side columns per CTA of the plain phase A (128 or 256): 256
// (two accumulators of 128 columns, two CTAs per SM) halves the CTA count
// of this short-item kernel; 7.04 against 7.21 ms at 522k facets and 1,024
// columns, identical results
constexpr int kPhaseANC = 256;

template <int MODE, bool SPLIT, int NR_ = (MODE == kModeA ? 128 : 64)>
struct TcCfg {
  static constexpr int NR = NR_;
  static constexpr int NC = (MODE == kModeA && !SPLIT) ? kPhaseANC : 128;
  static constexpr int CH = 32;
  // the split products on 128-row tiles / slices sum their drained windows
  // (256 reduction rows each) in plain FP32: 64 sums per thread leave no
  // room for compensation at two CTAs of 8 warps per SM.  (With Kahan sums
  // they needed 16 warps and one CTA per SM: split phase B 146 ms against
  // 71 ms now at 522k facets and 1,024 columns, with the same product
  // error.)  The 64-row shapes keep Kahan-compensated sums.
  static constexpr bool KAHAN = !(SPLIT && NR == 128);
  static constexpr int CTAS = SPLIT ? 2 : ((NR >= 256 || NC >= 256) ? 2 : 4);
  static constexpr int THREADS = 256;
  static constexpr int NQ = THREADS / 128;           // warps per TMEM lane quarter
  // phase B: chunks ahead at which a thread loads the source indices of its
  // gathered rows (the index load would otherwise stall the copies of the
  // next chunk; measured 7 % on the plain product, nothing on the split one)
  static constexpr int SRC_PF = SPLIT ? 1 : 4;
  static constexpr int PARTS = SPLIT ? 2 : 1;
  static constexpr int WB = CH * NR * 2;             // W bytes per stage and part
  static constexpr int SB = CH * NC * 2;             // S bytes per stage and part
  static constexpr int BLK = CH * 128;               // one 64-element block (W or S)
  static constexpr int STAGE = PARTS * (WB + SB);
  static constexpr int RING = (200 * 1024) / CTAS;   // ring bytes per CTA
  static constexpr int STAGES = RING / STAGE < 6 ? RING / STAGE : 6;
  // dynamic shared memory: the ring, 1 KiB for alignment, and at least a
  // third of the SM's 228 KiB when TMEM allows only two CTAs per SM (more
  // would wait in tcgen05.alloc)
  static constexpr int SMEM_RING = STAGES * STAGE + 1024;
  static constexpr int MAX_RES = 512 / ((SPLIT ? 2 : 1) * (NC / 128) * NR);
  static constexpr int SMEM_MIN = 233472 / (MAX_RES + 1) + 16;
  static constexpr int SMEM = SMEM_RING > SMEM_MIN ? SMEM_RING : SMEM_MIN;
  static constexpr int HALVES = NC / 128;            // accumulators per set
  static constexpr int SETS = SPLIT ? 2 : 1;
  static constexpr int TMEM_COLS = SETS * HALVES * NR;
  static constexpr int SEGS = HALVES * NR / 64;      // 64-column TMEM segments per set
  static constexpr int PPR = NC / 8;                 // 16-byte pieces per S row
  static constexpr int RPP = THREADS / PPR;         // S rows per pass of the CTA
  static constexpr int SROWS = CH / RPP;             // S rows per thread and chunk
  // instruction descriptor, kind::f16: D FP32, A and B BF16, both MN-major,
  // N = NR, M = 128
  static constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | (1u << 15) |
                                    (1u << 16) | ((uint32_t)(NR >> 3) << 17) |
                                    ((uint32_t)(128 >> 4) << 24);
  static_assert(TMEM_COLS == 64 || TMEM_COLS == 128 || TMEM_COLS == 256, "TMEM allocation");
  static_assert(STAGES >= 2, "ring of at least two stages");
  static_assert(CTAS * TMEM_COLS <= 512, "TMEM of the CTAs of one SM");
  static_assert(SEGS >= 1, "at least one 64-column TMEM segment per set");
  // 32-column pieces of a set, shared out over the NQ warps of a lane quarter
  static constexpr int PIECES = 2 * SEGS;
  static constexpr int PPW = PIECES / NQ;            // pieces per warp
  static_assert(PIECES % NQ == 0 && PPW >= 1, "pieces per warp");
  static_assert((CH * NR / 8) % THREADS == 0 && CH % RPP == 0, "copy plan");
};

__device__ __forceinline__ void mma_bf16_tc_n(uint32_t dtmem, uint64_t adesc, uint64_t bdesc,
                                              uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
      ::"r"(dtmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate) : "memory");
}

template <int MODE, bool SPLIT, int NRT>
__global__ void __launch_bounds__((TcCfg<MODE, SPLIT, NRT>::THREADS), (TcCfg<MODE, SPLIT, NRT>::CTAS))
tc_gather_gemm(TcArgs a) {
  using Cfg = TcCfg<MODE, SPLIT, NRT>;
  constexpr int NR = Cfg::NR, NC = Cfg::NC, CH = Cfg::CH, WB = Cfg::WB, SB = Cfg::SB;
  constexpr int BLK = Cfg::BLK, S = Cfg::STAGES, STAGE = Cfg::STAGE;
  extern __shared__ uint8_t smem_raw[];
  __shared__ __align__(8) unsigned long long bars[S];
  __shared__ uint32_t tmem_slot;
  __shared__ int abort_flag;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nks = (a.K + NC - 1) / NC;
  const long long unit = blockIdx.x / nks;
  const int c_base = (int)(blockIdx.x % nks) * NC;

  // ---- the CTA's reduction range and output rows
  long long r_first = 0, r_end = 0;   // reduction rows (panel rows / group columns)
  long long out_row0 = 0;             // first output row
  int out_rows = NR;                  // valid output rows
  const __nv_bfloat16* wbase_hi = a.w_hi;
  const __nv_bfloat16* wbase_lo = a.w_lo;
  long long wstride = NR;             // elements between consecutive W rows
  long long xrow0 = 0;                // phase A: X row of reduction row 0
  bool excl = true;
  if (MODE == kModeB) {
    const long long tile = a.tile_order ? (long long)a.tile_order[unit] : unit;
    r_first = a.t_p0[tile];
    r_end = a.t_p0[tile + 1];
    out_row0 = tile * NR;
    out_rows = (int)min((long long)NR, a.N - out_row0);
    if (((r_end - r_first) % 64) != 0) {
      // not a whole number of chunks: flagged, and the tile is left empty
      // (the copies below assume whole chunks)
      if (tid == 0) atomicOr(a.flags, FGB_FLAG_INDEX_RANGE);
      r_end = r_first;
    }
  } else {
    long long lo = 0, hi = a.num_items - 1;
    if (a.a_witem) {
      lo = a.a_witem[unit];
    } else {
      while (lo < hi) {
        const long long mid = (lo + hi + 1) >> 1;
        if (a.a_woff[mid] <= unit) lo = mid; else hi = mid - 1;
      }
    }
    const long long it = lo;
    const int sl = (int)(unit - a.a_woff[it]);
    const int g = a.a_grp[it];
    r_first = a.a_j0[it];
    r_end = a.a_j1[it];
    out_row0 = a.g_z0[g] + (long long)sl * NR;
    out_rows = min(NR, a.g_kz[g] - sl * NR);
    wstride = a.g_kzp[g];
    wbase_hi = a.w_hi + a.g_vtoff[g] + (long long)sl * NR;
    if (SPLIT) wbase_lo = a.w_lo + a.g_vtoff[g] + (long long)sl * NR;
    xrow0 = a.g_c0[g];
    excl = a.a_excl[it] != 0;
    if (a.zout_hi && !excl && tid == 0) atomicOr(a.flags, FGB_FLAG_INDEX_RANGE);
    if (tid == 0 && (a.g_kzp[g] % NR) != 0) atomicOr(a.flags, FGB_FLAG_INDEX_RANGE);
  }
  const int nch = (int)((r_end - r_first + CH - 1) / CH);

  uint8_t* smem = reinterpret_cast<uint8_t*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const uint32_t sbase = smem_addr(smem);
  if (tid == 0) {
    for (int st = 0; st < S; st++) mbar_init(smem_addr(&bars[st]), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    abort_flag = 0;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 ::"r"(smem_addr(&tmem_slot)), "r"(Cfg::TMEM_COLS) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;

  // stage layout: [W_hi | S_hi] or [W_hi | W_lo | S_hi | S_lo]; W and S are
  // stored as 64-element blocks of CH 128-byte lines (1 KiB swizzle atoms)
  auto w_at = [&](int st, int part) { return sbase + st * STAGE + part * WB; };
  auto s_at = [&](int st, int part) {
    return sbase + st * STAGE + Cfg::PARTS * WB + part * SB;
  };
  // S rows handled by this thread: k = tid / PPR + RPP j, 16-byte piece
  // tid % PPR of each (consecutive threads on consecutive pieces of a row)
  const int srow0 = tid / Cfg::PPR;
  const int spiece = tid % Cfg::PPR;
  // phase B: source rows of this thread's S rows of chunk c (through src[]),
  // fetched SRC_PF chunks ahead into a register ring (src_ring[p]: chunk
  // cn + p of the loop below) so that the dependent index load does not
  // stall the copies
  constexpr int RPW = Cfg::SROWS, PF = Cfg::SRC_PF;
  int src_ring[PF][RPW];
  // phase B tiles are whole chunks (their row counts are multiples of 64):
  // a chunk below nch holds CH rows of the tile
  const int* srcp = a.src + r_first + srow0;
  auto fetch_src = [&](int c, int (&dst)[RPW]) {
#pragma unroll
    for (int j = 0; j < RPW; j++)
      dst[j] = (MODE == kModeB && c < nch) ? __ldg(srcp + (long long)c * CH + Cfg::RPP * j) : 0;
  };
  // this thread's copies, constant over the chunks: W pieces (row k, 16-byte
  // piece (b, q)) and S rows (k = srow0 + RPP j, piece spiece), as shared
  // offsets in a stage and global element offsets for chunk 0
  constexpr int WPT = CH * NR / 8 / Cfg::THREADS;
  uint32_t w_so[WPT];
  int w_k[WPT];
  long long w_off[WPT];
#pragma unroll
  for (int j = 0; j < WPT; j++) {
    const int p = tid + j * Cfg::THREADS;
    const int k = p / (NR / 8), rem = p % (NR / 8);
    const int b = rem >> 3, q = rem & 7;
    w_so[j] = b * BLK + k * 128 + ((q ^ (k & 7)) << 4);
    w_k[j] = k;
    w_off[j] = (r_first + k) * wstride + b * 64 + q * 8;
  }
  const long long w_step = (long long)CH * wstride;
  uint32_t s_so[RPW];
#pragma unroll
  for (int j = 0; j < RPW; j++) {
    const int k = srow0 + Cfg::RPP * j;
    s_so[j] = (spiece >> 3) * BLK + k * 128 + (((spiece & 7) ^ (k & 7)) << 4);
  }
  const int col = c_base + spiece * 8;
  const bool colok = col < a.K;
  auto load = [&](int c, int st, const int (&srcs)[RPW]) {
    const long long l0 = r_first + (long long)c * CH;
    const long long wc = (long long)c * w_step;
    const uint32_t sw = w_at(st, 0), sw_lo = w_at(st, 1);
    const uint32_t ss = s_at(st, 0), ss_lo = s_at(st, 1);
    // W: CH rows x NR weights
#pragma unroll
    for (int j = 0; j < WPT; j++) {
      const bool ok = MODE == kModeB || l0 + w_k[j] < r_end;
      const long long off = ok ? w_off[j] + wc : 0;
      cp_async16_zfill(sw + w_so[j], wbase_hi + off, ok);
      if (SPLIT) cp_async16_zfill(sw_lo + w_so[j], wbase_lo + off, ok);
    }
    // S: CH gathered rows x NC columns
#pragma unroll
    for (int j = 0; j < RPW; j++) {
      const __nv_bfloat16* rh;
      const __nv_bfloat16* rl = nullptr;
      bool ok = colok;
      if (MODE == kModeB) {
        const long long sidx = srcs[j];
        if (a.s_hi) {
          rh = a.s_hi + sidx * a.lds;
          if (SPLIT) rl = a.s_lo + sidx * a.lds;
        } else if (sidx < a.num_zrows) {
          rh = a.z_hi + sidx * a.lds;
          if (SPLIT) rl = a.z_lo + sidx * a.lds;
        } else {
          rh = a.x_hi + (sidx - a.num_zrows) * a.lds;
          if (SPLIT) rl = a.x_lo + (sidx - a.num_zrows) * a.lds;
        }
      } else {
        const long long l = l0 + srow0 + Cfg::RPP * j;
        const bool okr = l < r_end;
        ok = ok && okr;
        const long long xr = okr ? xrow0 + l : 0;
        rh = a.x_hi + xr * a.lds;
        if (SPLIT) rl = a.x_lo + xr * a.lds;
      }
      cp_async16_zfill(ss + s_so[j], ok ? rh + col : rh, ok);
      if (SPLIT) cp_async16_zfill(ss_lo + s_so[j], ok ? rl + col : rl, ok);
    }
  };

  for (int c = 0; c < S - 1; c++) {
    int src_pro[RPW];
    fetch_src(c, src_pro);
    if (c < nch) load(c, c, src_pro);
    cp_commit();
  }
#pragma unroll
  for (int p = 0; p < PF; p++) fetch_src(S - 1 + p, src_ring[p]);
  // epilogue / drain mapping: warp w reads TMEM lanes 32 (w % 4) .. + 31
  // (right-hand-side columns) of the 32-column pieces pc = w / 4 + NQ k,
  // k < PPW; piece pc = (accumulator half pc / (NR / 32), output rows
  // 32 (pc % (NR / 32)) .. + 31)
  const int quarter = warp & 3, pc0 = warp >> 2;
  constexpr int NV = SPLIT ? Cfg::PPW * 32 : 1;       // compensated sums per thread
  constexpr int NVC = Cfg::KAHAN ? NV : 1;
  float racc[NV], rcmp[NVC];
#pragma unroll
  for (int i = 0; i < NV; i++) racc[i] = 0.f;
#pragma unroll
  for (int i = 0; i < NVC; i++) rcmp[i] = 0.f;
  auto piece_col = [&](int pc) {         // TMEM column of piece pc (in a set)
    return (pc / (NR / 32)) * NR + (pc % (NR / 32)) * 32;
  };
  auto drain = [&](int set) {
    if (SPLIT) {
#pragma unroll
      for (int k = 0; k < Cfg::PPW; k++) {
        float v[32];
        tmem_ld32(tmem + ((uint32_t)(quarter * 32) << 16) + set * (Cfg::HALVES * NR) +
                      piece_col(pc0 + Cfg::NQ * k), v);
#pragma unroll
        for (int i = 0; i < 32; i++) {
          if constexpr (Cfg::KAHAN) kahan_add(racc[k * 32 + i], rcmp[k * 32 + i], v[i]);
          else racc[k * 32 + i] = __fadd_rn(racc[k * 32 + i], v[i]);
        }
      }
      tc_fence_before();
    }
  };
  // Per chunk c: every thread waits for its own copies of chunk c; thread 0
  // alone waits for the MMAs of chunk c - 1 (the others sleep in the
  // CTA barrier instead of polling, which would take issue slots from the
  // copies); after the barrier chunk c is in shared memory and stage
  // (c - 1) % S is free, so thread 0 issues chunk c's MMAs and everyone
  // refills that stage with chunk c + S - 1.
  bool ok = true;
  for (int c = 0; c < nch; c++) {
    const int st = c % S;
    cp_wait<S - 2>();
    fence_proxy_async();
    if (tid == 0 && c >= 1) {
      const int sp = (c - 1) % S;
      if (!mbar_wait(smem_addr(&bars[sp]), ((c - 1) / S) & 1)) {
        atomicOr(a.flags, FGB_FLAG_DEVICE_TIMEOUT);
        abort_flag = 1;
      }
    }
    __syncthreads();
    if (abort_flag) { ok = false; break; }
    tc_fence_after();
    if (tid == 0) {
      // split mode: window c / kTcWin accumulates into set (c / kTcWin) & 1
      const uint32_t dset = SPLIT ? (uint32_t)(((c / kTcWin) & 1) * (Cfg::HALVES * NR)) : 0u;
      const bool first = SPLIT ? (c % kTcWin) == 0 : c == 0;
#pragma unroll
      for (int q = 0; q < CH / 16; q++) {
        // 16 reduction rows = two 8-line groups (SBO 1 KiB); k-step offset
        // 2 KiB; NR output rows = NR / 64 blocks (LBO = block stride)
        const uint64_t bh = sw128_desc(w_at(st, 0) + q * 2048, BLK, 1024);
#pragma unroll
        for (int h = 0; h < Cfg::HALVES; h++) {
          // M = 128 columns = two 64-column blocks, LBO = block stride
          const uint64_t ah = sw128_desc(s_at(st, 0) + h * 2 * BLK + q * 2048, BLK, 1024);
          const uint32_t d = tmem + dset + h * NR;
          mma_bf16_tc_n(d, ah, bh, Cfg::IDESC, !(first && q == 0));
          if (SPLIT) {
            const uint64_t bl = sw128_desc(w_at(st, 1) + q * 2048, BLK, 1024);
            const uint64_t al = sw128_desc(s_at(st, 1) + h * 2 * BLK + q * 2048, BLK, 1024);
            mma_bf16_tc_n(d, al, bh, Cfg::IDESC, 1u);
            mma_bf16_tc_n(d, ah, bl, Cfg::IDESC, 1u);
          }
        }
      }
      mma_commit(smem_addr(&bars[st]));
    }
    const int cn = c + S - 1;
    int src_new[RPW];
    fetch_src(cn + PF, src_new);
    // chunk c - 1 ended a window (its MMAs are complete): its set is drained
    // while chunk c's MMAs run on the other set
    if (SPLIT && c >= 1 && (c % kTcWin) == 0) drain(((c - 1) / kTcWin) & 1);
    if (cn < nch) load(cn, cn % S, src_ring[0]);
    cp_commit();
#pragma unroll
    for (int p = 0; p < PF - 1; p++)
#pragma unroll
      for (int j = 0; j < RPW; j++) src_ring[p][j] = src_ring[p + 1][j];
#pragma unroll
    for (int j = 0; j < RPW; j++) src_ring[PF - 1][j] = src_new[j];
  }
  cp_wait_all();
  // all MMAs of this CTA complete (they finish in order): thread 0 waits for
  // the last chunk's barrier
  if (tid == 0 && nch > 0 && ok) {
    const int cl = nch - 1;
    if (!mbar_wait(smem_addr(&bars[cl % S]), (cl / S) & 1)) {
      atomicOr(a.flags, FGB_FLAG_DEVICE_TIMEOUT);
      ok = false;
    }
  }
  ok = __syncthreads_and(ok) != 0;     // one decision for the whole CTA
  tc_fence_after();

  // the last (possibly partial) window
  if (SPLIT && ok && nch > 0) drain(((nch - 1) / kTcWin) & 1);

  // epilogue (mapping as for the drain)
  const bool bf16_out = MODE == kModeA && a.zout_hi != nullptr;
  if (ok && bf16_out) {
    // phase A with BF16 Z: the NR x NC tile (hi, and lo) is staged in the
    // idle ring, row-major, then written as whole 16-byte pieces of Z rows
    // (a thread's accumulators are one column of 32-row pieces: stored
    // directly, each would be a separate 2-byte store)
    static_assert(MODE != kModeA || NR * NC * 2 * Cfg::PARTS <= S * STAGE,
                  "BF16 tile staging in the ring");
    __nv_bfloat16* t_hi = reinterpret_cast<__nv_bfloat16*>(smem);
    __nv_bfloat16* t_lo = t_hi + NR * NC;
    fence_proxy_async();
#pragma unroll
    for (int k = 0; k < Cfg::PPW; k++) {
      const int pc = pc0 + Cfg::NQ * k;
      const int h = pc / (NR / 32), rr = pc % (NR / 32);
      const int cc = h * 128 + quarter * 32 + lane;
      float v[32];
      if (SPLIT) {
#pragma unroll
        for (int i = 0; i < 32; i++) v[i] = racc[k * 32 + i];
      } else if (nch > 0) {
        tmem_ld32(tmem + ((uint32_t)(quarter * 32) << 16) + piece_col(pc), v);
      } else {
#pragma unroll
        for (int i = 0; i < 32; i++) v[i] = 0.f;
      }
#pragma unroll
      for (int i = 0; i < 32; i++) {
        const __nv_bfloat16 hv = __float2bfloat16(v[i]);
        t_hi[(rr * 32 + i) * NC + cc] = hv;
        if (SPLIT) t_lo[(rr * 32 + i) * NC + cc] = __float2bfloat16(v[i] - __bfloat162float(hv));
      }
    }
    __syncthreads();
    if (excl) {
      for (int p = tid; p < NR * NC / 8; p += Cfg::THREADS) {
        const int r = p / (NC / 8), q = p % (NC / 8);
        const int col = c_base + q * 8;
        if (r < out_rows && col < a.K) {
          const long long o = (out_row0 + r) * (long long)a.K + col;
          *reinterpret_cast<uint4*>(a.zout_hi + o) = *reinterpret_cast<const uint4*>(t_hi + r * NC + q * 8);
          if (SPLIT)
            *reinterpret_cast<uint4*>(a.zout_lo + o) = *reinterpret_cast<const uint4*>(t_lo + r * NC + q * 8);
        }
      }
    }
  } else if (ok) {
#pragma unroll
    for (int k = 0; k < Cfg::PPW; k++) {
      const int pc = pc0 + Cfg::NQ * k;
      const int h = pc / (NR / 32), rr = pc % (NR / 32);
      const int col = c_base + h * 128 + quarter * 32 + lane;
      {
        float v[32];
        if (SPLIT) {
#pragma unroll
          for (int i = 0; i < 32; i++) v[i] = racc[k * 32 + i];
        } else if (nch > 0) {
          tmem_ld32(tmem + ((uint32_t)(quarter * 32) << 16) + piece_col(pc), v);
        } else {
#pragma unroll
          for (int i = 0; i < 32; i++) v[i] = 0.f;
        }
        if (col < a.K) {
#pragma unroll
          for (int i = 0; i < 32; i++) {
            const int r = rr * 32 + i;
            if (r < out_rows) {
              const long long row = out_row0 + r;
              const long long o = row * (long long)a.K + col;
              if (MODE == kModeB) {
                float y = v[i];
                if (a.add) y = a.add[o] + a.alpha * y;
                a.out[o] = y;
              } else if (excl) {
                a.out[o] = v[i];
              } else {
                atomicAdd(a.out + o, v[i]);
              }
            }
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    __syncwarp();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;"
                 ::"r"(tmem), "r"(Cfg::TMEM_COLS) : "memory");
  }
}

// Wider panel from the 64-row FP32 one: old panel row r (64-row tile t)
// with new_row[r] >= 0 lands in part part[r] (t mod width / 64) of new row
// new_row[r], as BF16; the new panel (width weights per row) is zeroed by
// the caller (a new row gets at most one old row per part: a source appears
// once per 64-row tile).  One warp per old row.  lo (optional): the split
// operand's low part, bf16(w - bf16(w)).
__global__ void retile_panel_kernel(const float* __restrict__ panel64, long long num_rows,
                                    const long long* __restrict__ new_row,
                                    const unsigned char* __restrict__ part, int width,
                                    __nv_bfloat16* __restrict__ panel128,
                                    __nv_bfloat16* __restrict__ lo128) {
  const int lane = threadIdx.x & 31;
  const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long r = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5; r < num_rows;
       r += warps) {
    const long long nr = new_row[r];
    if (nr < 0) continue;
    const float2 w = reinterpret_cast<const float2*>(panel64 + r * 64)[lane];
    const long long o = nr * width + part[r] * 64 + 2 * lane;
    const __nv_bfloat16 hx = __float2bfloat16(w.x), hy = __float2bfloat16(w.y);
    panel128[o] = hx;
    panel128[o + 1] = hy;
    if (lo128) {
      lo128[o] = __float2bfloat16(w.x - __bfloat162float(hx));
      lo128[o + 1] = __float2bfloat16(w.y - __bfloat162float(hy));
    }
  }
}

__global__ void split_bf16_kernel(const float* __restrict__ in, __nv_bfloat16* __restrict__ hi,
                                  __nv_bfloat16* __restrict__ lo, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const float v = in[i];
    const __nv_bfloat16 h = __float2bfloat16(v);
    hi[i] = h;
    if (lo) lo[i] = __float2bfloat16(v - __bfloat162float(h));
  }
}

// Transposed phase-A panel: tile (g, s, jb) moves V^T rows 64 s .. of group g,
// columns 64 jb .., through shared memory; rows r >= kz are zero.
__global__ void vpanel_transpose_kernel(const int* __restrict__ g_n, const int* __restrict__ g_kz,
                                        const int* __restrict__ g_ldv,
                                        const long long* __restrict__ g_voff,
                                        const int* __restrict__ g_kzp,
                                        const long long* __restrict__ g_vtoff,
                                        const float* __restrict__ vpanel,
                                        const int* __restrict__ tile_g,
                                        const int* __restrict__ tile_s,
                                        const int* __restrict__ tile_j, long long num_tiles,
                                        __nv_bfloat16* __restrict__ vt_hi,
                                        __nv_bfloat16* __restrict__ vt_lo) {
  __shared__ float tile[64][65];
  for (long long t = blockIdx.x; t < num_tiles; t += gridDim.x) {
    const int g = tile_g[t], s = tile_s[t], jb = tile_j[t];
    const int n = g_n[g], kz = g_kz[g], ldv = g_ldv[g], kzp = g_kzp[g];
    const float* v = vpanel + g_voff[g];
    __syncthreads();
    for (int e = threadIdx.x; e < 64 * 64; e += blockDim.x) {
      const int rr = e >> 6, jj = e & 63;
      const int r = s * 64 + rr, j = jb * 64 + jj;
      tile[rr][jj] = (r < kz && j < n) ? v[(long long)r * ldv + j] : 0.f;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < 64 * 64; e += blockDim.x) {
      const int jj = e >> 6, rr = e & 63;
      const int r = s * 64 + rr, j = jb * 64 + jj;
      if (j < n && r < kzp) {
        const float x = tile[rr][jj];
        const __nv_bfloat16 h = __float2bfloat16(x);
        const long long o = g_vtoff[g] + (long long)j * kzp + r;
        vt_hi[o] = h;
        if (vt_lo) vt_lo[o] = __float2bfloat16(x - __bfloat162float(h));
      }
    }
  }
}

template <int MODE, bool SPLIT, int NRT = (MODE == kModeA ? 128 : 64)>
int launch_tc(const TcArgs& a, long long units, cudaStream_t st) {
  using Cfg = TcCfg<MODE, SPLIT, NRT>;
  static bool attr_set = false;
  if (!attr_set) {
    FGB_CUDA_TRY(cudaFuncSetAttribute(tc_gather_gemm<MODE, SPLIT, NRT>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg::SMEM));
    attr_set = true;
  }
  const long long nks = (a.K + Cfg::NC - 1) / Cfg::NC;
  const long long grid = units * nks;
  if (grid <= 0) return FGB_OK;
  if (grid > 0x7fffffffLL) { set_error("grid too large"); return FGB_BAD_ARG; }
  tc_gather_gemm<MODE, SPLIT, NRT><<<(unsigned)grid, Cfg::THREADS, Cfg::SMEM, st>>>(a);
  FGB_LAUNCH_CHECK("tc_gather_gemm");
  return FGB_OK;
}

bool misaligned(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) != 0; }

// ---------------------------------------------------------------------------
// Phase B with TMA (warp-specialised).  The sources must be one row-major
// tensor S = [Z; X] ((num_zrows + N) x K, BF16); its rows are gathered four
// at a time by cp.async.bulk.tensor ... tile::gather4 (a tensor map with a
// 64-column x 1-row box and the 128-byte swizzle, so rows land directly in
// the MMA's MN-major swizzled layout, four 128-byte lines per request), the
// panel chunk comes with one tiled TMA load (64 x 64 box).  Copies complete
// on the stage's "full" mbarrier (transaction bytes); no thread issues
// per-16-byte copies and no CTA-wide barrier runs per chunk.
//   warp 0      producer: lanes 0..15 gather rows 4 lane .. 4 lane + 3
//   warp 1      MMA issuer (lane 0): waits "full", issues, commits "empty"
//   warps 4..7  epilogue (TMEM lanes 32 (w - 4) ..); in split mode they also
//               drain each chunk's accumulator set into compensated sums
//               (a 64-row window; the cp.async kernel drains every kTcWin
//               32-row chunks)
// Split mode: NC = 128 columns (one accumulator half, two TMEM sets that
// alternate by chunk), hi and lo maps for both operands.
template <bool SPLIT>
struct TmaCfg {
  static constexpr int CH = 64;                       // panel rows per stage
  static constexpr int NC = SPLIT ? 128 : 256;        // right-hand-side columns per CTA
  static constexpr int PARTS = SPLIT ? 2 : 1;
  static constexpr int WB = CH * kTcRows * 2;         // 8 KiB per part
  static constexpr int SB = CH * NC * 2;              // 16 / 32 KiB per part
  static constexpr int STAGE = PARTS * (WB + SB);     // 48 / 40 KiB
  static constexpr int STAGES = SPLIT ? 4 : 5;
  static constexpr int SMEM = STAGES * STAGE + 1024;
  static constexpr int HALVES = NC / 128;
  static constexpr int TMEM_COLS = 128;
};

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y,
                                            uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];"
      ::"r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar) : "memory");
}
__device__ __forceinline__ void tma_gather4(uint32_t dst, const CUtensorMap* map, int x, int r0,
                                            int r1, int r2, int r3, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cta.global.tile::gather4.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];"
      ::"r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(r0), "r"(r1), "r"(r2),
        "r"(r3), "r"(bar) : "memory");
}

template <bool SPLIT>
__global__ void __launch_bounds__(kTcThreads, 1)
tc_phase_b_tma(const __grid_constant__ CUtensorMap tm_w_hi,
               const __grid_constant__ CUtensorMap tm_w_lo,
               const __grid_constant__ CUtensorMap tm_s_hi,
               const __grid_constant__ CUtensorMap tm_s_lo, TcArgs a) {
  using Cfg = TmaCfg<SPLIT>;
  constexpr int S = Cfg::STAGES;
  extern __shared__ uint8_t smem_raw[];
  __shared__ __align__(8) unsigned long long full_bar[S], empty_bar[S], win_full[2], win_empty[2],
      done_bar;
  __shared__ uint32_t tmem_slot;
  __shared__ volatile int abort_flag;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nks = (a.K + Cfg::NC - 1) / Cfg::NC;
  const long long t = blockIdx.x / nks;
  const int c_base = (int)(blockIdx.x % nks) * Cfg::NC;
  const long long p0 = a.t_p0[t], p1 = a.t_p0[t + 1];
  const int nch = (int)((p1 - p0) / Cfg::CH);
  const long long out_row0 = t * kTcRows;
  const int out_rows = (int)min((long long)kTcRows, a.N - out_row0);

  uint8_t* smem = reinterpret_cast<uint8_t*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const uint32_t sbase = smem_addr(smem);
  auto w_at = [&](int s, int part) { return sbase + s * Cfg::STAGE + part * Cfg::WB; };
  auto s_at = [&](int s, int part) {
    return sbase + s * Cfg::STAGE + Cfg::PARTS * Cfg::WB + part * Cfg::SB;
  };
  if (tid == 0) {
    if (((p1 - p0) % Cfg::CH) != 0) atomicOr(a.flags, FGB_FLAG_INDEX_RANGE);
    for (int i = 0; i < S; i++) {
      mbar_init(smem_addr(&full_bar[i]), 1);
      mbar_init(smem_addr(&empty_bar[i]), 1);
    }
    for (int i = 0; i < 2; i++) {
      mbar_init(smem_addr(&win_full[i]), 1);
      mbar_init(smem_addr(&win_empty[i]), 4);
    }
    mbar_init(smem_addr(&done_bar), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    abort_flag = 0;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 ::"r"(smem_addr(&tmem_slot)), "r"(Cfg::TMEM_COLS) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;
  auto fail = [&]() {
    atomicOr(a.flags, FGB_FLAG_DEVICE_TIMEOUT);
    abort_flag = 1;
  };
  // warp-uniform bounded wait (lane 0 polls) and abort test, so that the
  // warp stays converged for the .sync.aligned tcgen05 instructions
  auto warp_wait = [&](uint32_t bar, uint32_t parity) {
    int got = 1;
    if (lane == 0) got = mbar_wait(bar, parity) ? 1 : 0;
    return __shfl_sync(0xffffffffu, got, 0) != 0;
  };
  auto warp_abort = [&]() { return __shfl_sync(0xffffffffu, (int)abort_flag, 0) != 0; };

  if (warp == 0) {
    // ---------------- producer
    constexpr uint32_t kBytes = Cfg::STAGE;
    auto fetch = [&](int c) {
      int4 v = make_int4(0, 0, 0, 0);
      if (c < nch && lane < Cfg::CH / 4)
        v = __ldg(reinterpret_cast<const int4*>(a.src + p0 + (long long)c * Cfg::CH) + lane);
      return v;
    };
    int4 sv = fetch(0);
    int issued = 0;
    for (int c = 0; c < nch; c++) {
      const int s = c % S;
      const int4 sv_next = fetch(c + 1);
      if (c >= S && !warp_wait(smem_addr(&empty_bar[s]), ((c / S) - 1) & 1)) {
        if (lane == 0) fail();
      }
      if (warp_abort()) break;
      const uint32_t fb = smem_addr(&full_bar[s]);
      if (lane == 0) {
        mbar_expect_tx(fb, kBytes);
        const int y = (int)(p0 + (long long)c * Cfg::CH);
        tma_load_2d(w_at(s, 0), &tm_w_hi, 0, y, fb);
        if (SPLIT) tma_load_2d(w_at(s, 1), &tm_w_lo, 0, y, fb);
      }
      __syncwarp();
      if (lane < Cfg::CH / 4) {
#pragma unroll
        for (int b = 0; b < Cfg::NC / 64; b++) {
          const uint32_t off = b * (Cfg::CH * 128) + lane * 512;
          tma_gather4(s_at(s, 0) + off, &tm_s_hi, c_base + 64 * b, sv.x, sv.y, sv.z, sv.w, fb);
          if (SPLIT)
            tma_gather4(s_at(s, 1) + off, &tm_s_lo, c_base + 64 * b, sv.x, sv.y, sv.z, sv.w, fb);
        }
      }
      sv = sv_next;
      issued = c + 1;
    }
    // copies still in flight (an aborted run): wait for the last stages to land
    if (lane == 0 && abort_flag) {
      for (int c = max(0, issued - S); c < issued; c++)
        mbar_wait(smem_addr(&full_bar[c % S]), (c / S) & 1);
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer
    if (lane == 0) {
      for (int c = 0; c < nch; c++) {
        const int s = c % S;
        if (!mbar_wait(smem_addr(&full_bar[s]), (c / S) & 1)) { fail(); break; }
        if (abort_flag) break;
        const int set = SPLIT ? (c & 1) : 0;
        if (SPLIT && c >= 2 && !mbar_wait(smem_addr(&win_empty[set]), ((c >> 1) - 1) & 1)) {
          fail();
          break;
        }
        tc_fence_after();
#pragma unroll
        for (int q = 0; q < Cfg::CH / 16; q++) {
          const uint64_t bh = sw128_desc(w_at(s, 0) + q * 2048, 8192, 1024);
#pragma unroll
          for (int h = 0; h < Cfg::HALVES; h++) {
            const uint32_t blk = Cfg::CH * 128;
            const uint64_t ah = sw128_desc(s_at(s, 0) + h * 2 * blk + q * 2048, blk, 1024);
            const uint32_t d = tmem + (SPLIT ? set * kTcRows : h * kTcRows);
            if (SPLIT) {
              const uint64_t bl = sw128_desc(w_at(s, 1) + q * 2048, 8192, 1024);
              const uint64_t al = sw128_desc(s_at(s, 1) + h * 2 * blk + q * 2048, blk, 1024);
              mma_bf16_tc(d, ah, bh, q != 0);
              mma_bf16_tc(d, al, bh, 1u);
              mma_bf16_tc(d, ah, bl, 1u);
            } else {
              mma_bf16_tc(d, ah, bh, (c | q) != 0);
            }
          }
        }
        mma_commit(smem_addr(&empty_bar[s]));
        if (SPLIT) mma_commit(smem_addr(&win_full[set]));
      }
      mma_commit(smem_addr(&done_bar));
    }
  } else if (warp >= 4) {
    // ---------------- epilogue
    const int quarter = warp - 4;
    float racc[SPLIT ? kTcRows : 1], rcmp[SPLIT ? kTcRows : 1];
#pragma unroll
    for (int i = 0; i < (SPLIT ? kTcRows : 1); i++) { racc[i] = 0.f; rcmp[i] = 0.f; }
    bool ok = true;
    if (SPLIT) {
      for (int c = 0; c < nch; c++) {
        const int set = c & 1;
        if (!warp_wait(smem_addr(&win_full[set]), (c >> 1) & 1)) {
          if (lane == 0) fail();
          ok = false;
          break;
        }
        if (warp_abort()) { ok = false; break; }
        tc_fence_after();
#pragma unroll
        for (int half = 0; half < kTcRows / 32; half++) {
          float v[32];
          tmem_ld32(tmem + ((uint32_t)(quarter * 32) << 16) + set * kTcRows + half * 32, v);
#pragma unroll
          for (int i = 0; i < 32; i++) kahan_add(racc[half * 32 + i], rcmp[half * 32 + i], v[i]);
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(smem_addr(&win_empty[set]));
      }
    }
    if (ok && !warp_wait(smem_addr(&done_bar), 0)) {
      if (lane == 0) fail();
      ok = false;
    }
    if (warp_abort()) ok = false;
    tc_fence_after();
    if (ok) {
#pragma unroll
      for (int h = 0; h < Cfg::HALVES; h++) {
        const int col = c_base + h * 128 + quarter * 32 + lane;
#pragma unroll
        for (int half = 0; half < kTcRows / 32; half++) {
          float v[32];
          if (SPLIT) {
#pragma unroll
            for (int i = 0; i < 32; i++) v[i] = racc[half * 32 + i];
          } else if (nch > 0) {
            tmem_ld32(tmem + ((uint32_t)(quarter * 32) << 16) + h * kTcRows + half * 32, v);
          } else {
#pragma unroll
            for (int i = 0; i < 32; i++) v[i] = 0.f;
          }
          if (col < a.K) {
#pragma unroll
            for (int i = 0; i < 32; i++) {
              const int r = half * 32 + i;
              if (r < out_rows) {
                const long long row = out_row0 + r;
                float y = v[i];
                if (a.add) y = a.add[row * (long long)a.K + col] + a.alpha * y;
                a.out[row * (long long)a.K + col] = y;
              }
            }
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    __syncwarp();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;"
                 ::"r"(tmem), "r"(Cfg::TMEM_COLS) : "memory");
  }
}

// cuTensorMapEncodeTiled, resolved through the runtime at first use so that
// the library carries no link-time dependency on the driver library
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

int encode_map(CUtensorMap* m, const void* base, unsigned long long inner, unsigned long long rows,
               unsigned box_inner, unsigned box_rows) {
  cuuint64_t dims[2] = {inner, rows};
  cuuint64_t strides[1] = {inner * 2};
  cuuint32_t box[2] = {box_inner, box_rows};
  cuuint32_t es[2] = {1, 1};
  PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
  if (!fn) { set_error("cuTensorMapEncodeTiled is not available"); return FGB_CUDA_ERR; }
  CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides,
                  box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed (%d)", (int)r);
    return FGB_CUDA_ERR;
  }
  return FGB_OK;
}

template <bool SPLIT>
int launch_tma_b(const fgb_op_desc* d, const void* w_hi, const void* w_lo, const void* s_hi,
                 const void* s_lo, const TcArgs& a, cudaStream_t st) {
  using Cfg = TmaCfg<SPLIT>;
  static bool attr_set = false;
  if (!attr_set) {
    FGB_CUDA_TRY(cudaFuncSetAttribute(tc_phase_b_tma<SPLIT>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg::SMEM));
    attr_set = true;
  }
  alignas(64) CUtensorMap mw_hi, mw_lo, ms_hi, ms_lo;
  const unsigned long long srows = (unsigned long long)(d->num_zrows + d->N);
  int rc;
  if ((rc = encode_map(&mw_hi, w_hi, kTcRows, d->panel_rows, kTcRows, Cfg::CH))) return rc;
  if ((rc = encode_map(&ms_hi, s_hi, a.K, srows, 64, 1))) return rc;
  if (SPLIT) {
    if ((rc = encode_map(&mw_lo, w_lo, kTcRows, d->panel_rows, kTcRows, Cfg::CH))) return rc;
    if ((rc = encode_map(&ms_lo, s_lo, a.K, srows, 64, 1))) return rc;
  } else {
    mw_lo = mw_hi;
    ms_lo = ms_hi;
  }
  const long long nks = (a.K + Cfg::NC - 1) / Cfg::NC;
  const long long grid = d->num_tiles * nks;
  if (grid > 0x7fffffffLL) { set_error("grid too large"); return FGB_BAD_ARG; }
  tc_phase_b_tma<SPLIT><<<(unsigned)grid, kTcThreads, Cfg::SMEM, st>>>(mw_hi, mw_lo, ms_hi, ms_lo, a);
  FGB_LAUNCH_CHECK("tc_phase_b_tma");
  return FGB_OK;
}

}  // namespace
}  // namespace fgb

extern "C" {

int fgb_tc_phase_a(const struct fgb_op_desc* d, const void* vt_hi, const void* vt_lo,
                   const void* X_hi, const void* X_lo, float* Z, int K, int zero_z,
                   unsigned* flags, void* stream) {
  if (!d || !flags) { fgb::set_error("null operator or flags"); return FGB_BAD_ARG; }
  if (K < 8 || (K % 8) != 0) { fgb::set_error("K must be a positive multiple of 8"); return FGB_BAD_ARG; }
  const bool split = vt_lo != nullptr;
  if (split != (X_lo != nullptr)) { fgb::set_error("split operands must come in pairs"); return FGB_BAD_ARG; }
  if (fgb::misaligned(vt_hi) || fgb::misaligned(X_hi) || fgb::misaligned(vt_lo) ||
      fgb::misaligned(X_lo)) {
    fgb::set_error("tensor-core operands must be 16-byte aligned");
    return FGB_BAD_ARG;
  }
  if (d->slice_rows != 0 && d->slice_rows != 128) {
    fgb::set_error("fgb_tc_phase_a takes 128-row work slices");
    return FGB_BAD_ARG;
  }
  if (d->num_items <= 0 || d->num_zrows <= 0) return FGB_OK;
  cudaStream_t st = fgb::as_stream(stream);
  if (zero_z) FGB_CUDA_TRY(cudaMemsetAsync(Z, 0, sizeof(float) * d->num_zrows * (size_t)K, st));
  fgb::TcArgs a{};
  a.a_grp = d->a_grp; a.a_j0 = d->a_j0; a.a_j1 = d->a_j1; a.a_excl = d->a_excl;
  a.a_woff = d->a_woff; a.a_witem = d->a_witem; a.num_items = d->num_items;
  a.g_c0 = d->g_c0; a.g_kz = d->g_kz; a.g_kzp = d->g_kzp; a.g_vtoff = d->g_vtoff; a.g_z0 = d->g_z0;
  a.w_hi = static_cast<const __nv_bfloat16*>(vt_hi);
  a.w_lo = static_cast<const __nv_bfloat16*>(vt_lo);
  a.x_hi = static_cast<const __nv_bfloat16*>(X_hi);
  a.x_lo = static_cast<const __nv_bfloat16*>(X_lo);
  a.lds = K; a.K = K; a.out = Z; a.add = nullptr; a.alpha = 1.f; a.flags = flags;
  a.N = d->N; a.num_zrows = d->num_zrows;
  return split ? fgb::launch_tc<fgb::kModeA, true>(a, d->num_work, st)
               : fgb::launch_tc<fgb::kModeA, false>(a, d->num_work, st);
}

int fgb_tc_phase_a_bf16(const struct fgb_op_desc* d, const void* vt_hi, const void* vt_lo,
                        const void* X_hi, const void* X_lo, void* Z_hi, void* Z_lo, int K,
                        unsigned* flags, void* stream) {
  if (!d || !flags || !Z_hi) { fgb::set_error("null operator, output or flags"); return FGB_BAD_ARG; }
  if (K < 8 || (K % 8) != 0) { fgb::set_error("K must be a positive multiple of 8"); return FGB_BAD_ARG; }
  const bool split = vt_lo != nullptr;
  if (split != (X_lo != nullptr) || split != (Z_lo != nullptr)) {
    fgb::set_error("split operands must come in pairs");
    return FGB_BAD_ARG;
  }
  if (fgb::misaligned(vt_hi) || fgb::misaligned(X_hi) || fgb::misaligned(vt_lo) ||
      fgb::misaligned(X_lo) || fgb::misaligned(Z_hi) || fgb::misaligned(Z_lo)) {
    fgb::set_error("tensor-core operands and Z must be 16-byte aligned");
    return FGB_BAD_ARG;
  }
  if (d->num_items <= 0 || d->num_zrows <= 0) return FGB_OK;
  fgb::TcArgs a{};
  a.a_grp = d->a_grp; a.a_j0 = d->a_j0; a.a_j1 = d->a_j1; a.a_excl = d->a_excl;
  a.a_woff = d->a_woff; a.a_witem = d->a_witem; a.num_items = d->num_items;
  a.g_c0 = d->g_c0; a.g_kz = d->g_kz; a.g_kzp = d->g_kzp; a.g_vtoff = d->g_vtoff; a.g_z0 = d->g_z0;
  a.w_hi = static_cast<const __nv_bfloat16*>(vt_hi);
  a.w_lo = static_cast<const __nv_bfloat16*>(vt_lo);
  a.x_hi = static_cast<const __nv_bfloat16*>(X_hi);
  a.x_lo = static_cast<const __nv_bfloat16*>(X_lo);
  a.zout_hi = static_cast<__nv_bfloat16*>(Z_hi);
  a.zout_lo = static_cast<__nv_bfloat16*>(Z_lo);
  a.lds = K; a.K = K; a.out = nullptr; a.add = nullptr; a.alpha = 1.f; a.flags = flags;
  a.N = d->N; a.num_zrows = d->num_zrows;
  cudaStream_t st = fgb::as_stream(stream);
  const int sr = d->slice_rows ? d->slice_rows : 128;
  if (sr == 64) {
    if (!split) { fgb::set_error("plain phase A takes 128-row work slices"); return FGB_BAD_ARG; }
    return fgb::launch_tc<fgb::kModeA, true, 64>(a, d->num_work, st);
  }
  if (sr != 128) { fgb::set_error("work slices of phase A must be 64 or 128 rows"); return FGB_BAD_ARG; }
  return split ? fgb::launch_tc<fgb::kModeA, true>(a, d->num_work, st)
               : fgb::launch_tc<fgb::kModeA, false>(a, d->num_work, st);
}

int fgb_tc_phase_b(const struct fgb_op_desc* d, const void* w_hi, const void* w_lo,
                   const void* X_hi, const void* X_lo, const void* Z_hi, const void* Z_lo,
                   float* Y, int K, const float* add, float alpha, unsigned* flags,
                   void* stream) {
  if (!d || !flags) { fgb::set_error("null operator or flags"); return FGB_BAD_ARG; }
  if (K < 8 || (K % 8) != 0) { fgb::set_error("K must be a positive multiple of 8"); return FGB_BAD_ARG; }
  const bool split = w_lo != nullptr;
  // (an operator without low-rank blocks has no Z: its pointers may be null)
  if (split != (X_lo != nullptr) || (d->num_zrows > 0 && split != (Z_lo != nullptr))) {
    fgb::set_error("split operands must come in pairs");
    return FGB_BAD_ARG;
  }
  if (fgb::misaligned(w_hi) || fgb::misaligned(w_lo) || fgb::misaligned(X_hi) ||
      fgb::misaligned(X_lo) || fgb::misaligned(Z_hi) || fgb::misaligned(Z_lo)) {
    fgb::set_error("tensor-core operands must be 16-byte aligned");
    return FGB_BAD_ARG;
  }
  if (d->num_tiles <= 0) return FGB_OK;
  fgb::TcArgs a{};
  a.t_p0 = d->t_p0; a.src = d->src; a.N = d->N; a.num_zrows = d->num_zrows;
  a.tile_order = d->tile_order;

  a.w_hi = static_cast<const __nv_bfloat16*>(w_hi);
  a.w_lo = static_cast<const __nv_bfloat16*>(w_lo);
  a.x_hi = static_cast<const __nv_bfloat16*>(X_hi);
  a.x_lo = static_cast<const __nv_bfloat16*>(X_lo);
  a.z_hi = static_cast<const __nv_bfloat16*>(Z_hi);
  a.z_lo = static_cast<const __nv_bfloat16*>(Z_lo);
  a.lds = K; a.K = K; a.out = Y; a.add = add; a.alpha = alpha; a.flags = flags;
  // one base pointer for the gathered rows when X follows Z in memory
  const long long zspan = d->num_zrows * (long long)K;
  const bool stacked_hi = d->num_zrows == 0 || a.z_hi + zspan == a.x_hi;
  const bool stacked_lo = !split || d->num_zrows == 0 || a.z_lo + zspan == a.x_lo;
  if (stacked_hi && stacked_lo) {
    a.s_hi = d->num_zrows ? a.z_hi : a.x_hi;
    a.s_lo = split ? (d->num_zrows ? a.z_lo : a.x_lo) : nullptr;
  }
  cudaStream_t st = fgb::as_stream(stream);
  const int tr = d->tile_rows ? d->tile_rows : 64;
  if (tr == 128)
    return split ? fgb::launch_tc<fgb::kModeB, true, 128>(a, d->num_tiles, st)
                 : fgb::launch_tc<fgb::kModeB, false, 128>(a, d->num_tiles, st);
  if (tr == 256) {
    if (split) { fgb::set_error("split products take 64- or 128-row tiles"); return FGB_BAD_ARG; }
    return fgb::launch_tc<fgb::kModeB, false, 256>(a, d->num_tiles, st);
  }
  if (tr != 64) { fgb::set_error("tile_rows must be 64, 128 or 256"); return FGB_BAD_ARG; }
  return split ? fgb::launch_tc<fgb::kModeB, true, 64>(a, d->num_tiles, st)
               : fgb::launch_tc<fgb::kModeB, false, 64>(a, d->num_tiles, st);
}

int fgb_tc_phase_b_tma(const struct fgb_op_desc* d, const void* w_hi, const void* w_lo,
                       const void* S_hi, const void* S_lo, float* Y, int K, const float* add,
                       float alpha, unsigned* flags, void* stream) {
  if (!d || !flags) { fgb::set_error("null operator or flags"); return FGB_BAD_ARG; }
  if (K < 8 || (K % 8) != 0) { fgb::set_error("K must be a positive multiple of 8"); return FGB_BAD_ARG; }
  const bool split = w_lo != nullptr;
  if (split != (S_lo != nullptr)) { fgb::set_error("split operands must come in pairs"); return FGB_BAD_ARG; }
  if (fgb::misaligned(w_hi) || fgb::misaligned(w_lo) || fgb::misaligned(S_hi) ||
      fgb::misaligned(S_lo) || (reinterpret_cast<uintptr_t>(d->src) & 15)) {
    fgb::set_error("TMA operands and src must be 16-byte aligned");
    return FGB_BAD_ARG;
  }
  if (d->num_tiles <= 0) return FGB_OK;
  if (d->panel_rows <= 0) { fgb::set_error("panel_rows not set"); return FGB_BAD_ARG; }
  if (d->tile_rows != 0 && d->tile_rows != 64) { fgb::set_error("the TMA variant takes 64-row tiles"); return FGB_BAD_ARG; }
  fgb::TcArgs a{};
  a.t_p0 = d->t_p0; a.src = d->src; a.N = d->N; a.num_zrows = d->num_zrows;
  a.K = K; a.lds = K; a.out = Y; a.add = add; a.alpha = alpha; a.flags = flags;
  cudaStream_t st = fgb::as_stream(stream);
  return split ? fgb::launch_tma_b<true>(d, w_hi, w_lo, S_hi, S_lo, a, st)
               : fgb::launch_tma_b<false>(d, w_hi, nullptr, S_hi, nullptr, a, st);
}

int fgb_retile_panel_bf16(const float* panel64, long long num_rows, const long long* new_row,
                          const unsigned char* half, void* panel128, void* stream) {
  if (num_rows < 0 || !panel64 || !panel128) { fgb::set_error("bad arguments"); return FGB_BAD_ARG; }
  if (num_rows == 0) return FGB_OK;
  fgb::retile_panel_kernel<<<fgb::grid_for(num_rows * 32, 256, 152LL * 64), 256, 0,
                             fgb::as_stream(stream)>>>(
      panel64, num_rows, new_row, half, 128, static_cast<__nv_bfloat16*>(panel128), nullptr);
  FGB_LAUNCH_CHECK("retile_panel_kernel");
  return FGB_OK;
}

int fgb_retile_panel_bf16_n(const float* panel64, long long num_rows, const long long* new_row,
                            const unsigned char* part, int width, void* out, void* stream) {
  if (num_rows < 0 || !panel64 || !out || (width != 128 && width != 256)) {
    fgb::set_error("bad arguments (width must be 128 or 256)");
    return FGB_BAD_ARG;
  }
  if (num_rows == 0) return FGB_OK;
  fgb::retile_panel_kernel<<<fgb::grid_for(num_rows * 32, 256, 152LL * 64), 256, 0,
                             fgb::as_stream(stream)>>>(
      panel64, num_rows, new_row, part, width, static_cast<__nv_bfloat16*>(out), nullptr);
  FGB_LAUNCH_CHECK("retile_panel_kernel");
  return FGB_OK;
}

int fgb_retile_panel_split_bf16(const float* panel64, long long num_rows,
                                const long long* new_row, const unsigned char* half,
                                void* hi128, void* lo128, void* stream) {
  if (num_rows < 0 || !panel64 || !hi128 || !lo128) { fgb::set_error("bad arguments"); return FGB_BAD_ARG; }
  if (num_rows == 0) return FGB_OK;
  fgb::retile_panel_kernel<<<fgb::grid_for(num_rows * 32, 256, 152LL * 64), 256, 0,
                             fgb::as_stream(stream)>>>(
      panel64, num_rows, new_row, half, 128, static_cast<__nv_bfloat16*>(hi128),
      static_cast<__nv_bfloat16*>(lo128));
  FGB_LAUNCH_CHECK("retile_panel_kernel");
  return FGB_OK;
}

int fgb_split_bf16(const float* in, void* hi, void* lo, long long n, void* stream) {
  if (n < 0 || !hi) { fgb::set_error("bad arguments"); return FGB_BAD_ARG; }
  if (n == 0) return FGB_OK;
  fgb::split_bf16_kernel<<<fgb::grid_for(n, 256, 152LL * 16), 256, 0, fgb::as_stream(stream)>>>(
      in, static_cast<__nv_bfloat16*>(hi), static_cast<__nv_bfloat16*>(lo), n);
  FGB_LAUNCH_CHECK("split_bf16_kernel");
  return FGB_OK;
}

int fgb_vpanel_transpose_bf16(const struct fgb_op_desc* d, const float* vpanel,
                              const int* tile_g, const int* tile_s, const int* tile_j,
                              long long num_tiles, void* vt_hi, void* vt_lo, void* stream) {
  if (!d || num_tiles < 0 || !vt_hi) { fgb::set_error("bad arguments"); return FGB_BAD_ARG; }
  if (num_tiles == 0) return FGB_OK;
  fgb::vpanel_transpose_kernel<<<fgb::grid_for(num_tiles, 1, 152LL * 32), 256, 0,
                                  fgb::as_stream(stream)>>>(
      d->g_n, d->g_kz, d->g_ldv, d->g_voff, d->g_kzp, d->g_vtoff, vpanel, tile_g, tile_s, tile_j,
      num_tiles, static_cast<__nv_bfloat16*>(vt_hi), static_cast<__nv_bfloat16*>(vt_lo));
  FGB_LAUNCH_CHECK("vpanel_transpose_kernel");
  return FGB_OK;
}

}  // extern "C"
