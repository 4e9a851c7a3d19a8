// Mixed-precision multi-right-hand-side product on the 5th-generation tensor
// cores (tcgen05, sm_103a): Y = H X for up to 64 right-hand sides per pass.
//
// Storage. Every panel of the product (a row tile of the near/U pass, or a
// column piece of at most 64 V rows of a source group) is stored once more as
// FP16 pairs a = hi + lo (hi = fp16(a), lo = fp16(a - hi): 22 significant
// bits, relative residual about 2^-23), already in the UMMA canonical K-major
// layout, 64 columns per chunk, so a chunk is two contiguous byte ranges
// copied as they are. FP16 has FP32's precision to within two bits but a
// narrow exponent range, so every operand carries power-of-two scales that
// put its largest magnitude in [2^14, 2^15) (exact, and undone exactly):
//   panel rows   one scale per row (rho_i), undone in the epilogue; its
//                inverse trails the item's chunks (64 floats);
//   V rows       nu_k per rank row, and a second per-rank-row scale gamma_k =
//                2^-ceil(log2 ||V_k||_1) that bounds the t entries it makes:
//                the V pass writes t~_k = t_k sigma gamma_k (below 2^15 for
//                any x), and the U columns that read t~_k are stored times
//                1/gamma_k;
//   x            sigma_r per right-hand side, from max |x_r| at run time,
//                undone on y.
// The right-hand sides live in XTS, one row per entry of XT = [x permuted |
// t]: R FP16 hi values, then R lo values (4R bytes).
//
// Pipelines (one persistent CTA per SM; items from a ticket counter, in list
// order, so concurrent CTAs work on neighbouring panels and share XTS rows in
// L2; warp 0 takes the tickets and queues them for the other roles). A 32-wide
// pass runs two pipelines, item n in pipeline n & 1; they share the tensor
// cores but have their own stages, producers, MMA warp and epilogue set,
// because one MMA warp's own instructions per chunk bound a pipeline. A
// 64-wide pass runs one (every item in pipeline 0), whose epilogue sets still
// take every other item:
//   warp 0      item tickets (lane 0), queued in shared memory for the others;
//   producers   warps 1, 3 and 8.. (one per stage; producer b serves pipeline
//               b mod kPipes, and the pipeline's chunk g goes to its producer
//               g mod kPipeStages) of each pipeline's ring of 64-column
//               chunks: two bulk copies of the chunk that complete on the
//               stage's mbarrier (hi rows to tile rows 0..63, lo rows to tile
//               rows 64..127), and the XTS rows of its columns (whole rows) as
//               an N-major (MN-major) FP16 tile: for a V piece, whose columns
//               are consecutive rows, one TMA tile load of 64 rows on the same
//               barrier; for a row tile, one 8-row TMA tile load per K group
//               of 8 columns that are 8 consecutive rows (the runs of whole
//               source clusters and rank ranges), 16-byte cp.async gathers
//               for the other groups (padding columns read the zero row),
//               then a wait, a proxy fence and an mbarrier arrive;
//   MMA         warp 2 (pipeline 0) and, in a 32-wide pass, the last warp
//               (pipeline 1); one elected lane each: per 16 columns one UMMA,
//               [A_hi; A_lo] x [B_hi B_lo] with M = 128, N = 2R (hi and lo
//               stacked along both M and N; items have at most 64 rows), into
//               a fresh TMEM accumulator buffer (FP32) every kSegChunks
//               chunks; commits free the stage and hand each buffer to the
//               item's epilogue set. In a V piece's last chunk it first
//               zeroes the B rows of padding columns (other blocks' XTS rows,
//               which the 64-row tile load brought in: 0 * Inf must not reach
//               a sum);
//   epilogue    two sets of 4 warps (warps 4-7 and the four after the last
//               producer), set e for items n with n & 1 == e: per
//               accumulator buffer, tcgen05.ld of the warp's 32 TMEM lanes
//               added to FP32 registers; at the item's end the sum of the
//               four hi/lo quadrants (the hi-row and lo-row warps of the same
//               rows swap halves of their sums, so each finishes half of the
//               right-hand sides), the scales undone, then y rows, t rows of
//               XTS (split again) or partial rows P.
// Every wait is bounded by the global timer; one that runs out records a code
// in `status`, raises a CTA-wide abort flag and every role leaves its loop.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "hm_device.h"

namespace hm {

namespace {

constexpr int kKc = 64;                // columns per chunk
constexpr int kABytes = 128 * kKc * 2;  // A tile: 64 hi rows, then 64 lo rows: 16 KB
constexpr int kQ = 16;                  // item queue slots
#ifndef HM_TC_SEG_CHUNKS
#define HM_TC_SEG_CHUNKS 1
#endif
#ifndef HM_TC_SEG_CHUNKS_V
#define HM_TC_SEG_CHUNKS_V HM_TC_SEG_CHUNKS
#endif
// chunks per accumulator buffer, for near/U tiles and for V pieces: the
// tensor cores' own accumulation spans at most this many chunks (4 UMMAs
// each) before the epilogue takes the partial sums into FP32 registers
constexpr int kSegChunksDU = HM_TC_SEG_CHUNKS;

constexpr int kSegChunksV = HM_TC_SEG_CHUNKS_V;

// MN-major B: the hi and lo halves of the R right-hand sides are stacked along
// N, so one XTS row (4R bytes) is one K row of B. Core matrices of 8 N values
// (16 B) x 8 columns; the N groups are kBGroupN bytes apart, the K groups of 8
// columns TcShape<R>::kBGroupK bytes apart.
constexpr uint32_t kBGroupN = 128;

// The shape of a pass over R = 32 or 64 right-hand sides. A 64-wide pass reads
// every tile once for twice the columns; its B tiles are twice as large, so
// the ring has 6 stages instead of 8.
template <int R>
struct TcShape {
  static_assert(R == 32 || R == 64, "32 or 64 right-hand sides per pass");
  static constexpr int kBN = 2 * R;                   // B rows: R hi, then R lo
  static constexpr int kBBytes = kBN * kKc * 2;       // one FP16 B tile: 8 or 16 KB
  static constexpr int kStages = R == 32 ? 8 : 6;
  // Two pipelines for 32 right-hand sides. A 64-wide pass keeps one: a 17th
  // warp would cap every thread at 96 registers (warps per scheduler x
  // threads x registers), and its epilogue needs more for 64 sums a row.
  static constexpr int kPipes = R == 32 ? 2 : 1;
  static constexpr int kPipeStages = kStages / kPipes;  // stages of each pipeline
  static constexpr int kBProducers = kStages;           // warps 1, 3, 8 .. 5 + kStages
  static constexpr int kEpi1 = 6 + kBProducers;         // first warp of the second epilogue set
  static constexpr int kMma1 = kEpi1 + 4;               // MMA warp of the second pipeline, if any
  static constexpr int kWarps = kMma1 + kPipes - 1;     // roles: see the header comment
  static constexpr int kThreads = kWarps * 32;
  // TMEM: every column of the SM's 512, cut into accumulator buffers of kBN
  // columns, half of them for each epilogue set
  static constexpr uint32_t kTmemCols = 512;
  static constexpr int kBufs = static_cast<int>(kTmemCols) / kBN;  // 8 or 4
  static constexpr int kSetBufs = kBufs / 2;
  static constexpr int kConsumers = kBProducers + kPipes + 8;  // warps that read each queued item
  static constexpr uint32_t kBGroupK = (kBN / 8) * kBGroupN;
  static constexpr int kPieces = R / 4;               // 16-byte pieces of an XTS row
  static constexpr int kRowsPerCopy = 32 / kPieces;   // XTS rows per warp-wide copy
  // kind::f16 instruction descriptor: FP32 D, FP16 A (K-major) and B
  // (MN-major), N = kBN, M = 128.
  static constexpr uint32_t kIdesc = (1u << 4) | (1u << 16) | ((static_cast<uint32_t>(kBN) >> 3) << 17) |
                                     ((128u >> 4) << 24);
  // One producer per stage: a producer then never waits for a stage more than
  // one release ahead, which a parity wait on the stage's barrier could not
  // tell apart from the release before.
  static_assert(kBProducers == kStages, "one producer warp per stage");
  // the MMA warp waits for a whole segment's chunks before it releases any
  static_assert(kSegChunksDU <= kPipeStages && kSegChunksV <= kPipeStages, "a segment fits a pipeline's stages");
};
constexpr unsigned long long kWaitNs = 2000000000ull;  // 2 s per wait
constexpr unsigned long long kWaitIters = 1ull << 26;   // backstop if the timer stood still
constexpr int kSelfTestCode = 90;                        // status of the self-test's wait


__device__ __forceinline__ uint32_t su32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= static_cast<uint64_t>((saddr >> 4) & 0x3FFF);
  d |= static_cast<uint64_t>((lbo >> 4) & 0x3FFF) << 16;
  d |= static_cast<uint64_t>((sbo >> 4) & 0x3FFF) << 32;
  d |= static_cast<uint64_t>(1) << 46;  // descriptor version for tcgen05; no swizzle
  return d;
}

__device__ __forceinline__ void mma(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(bar))
               : "memory");
}

__device__ __forceinline__ void arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(su32(bar)) : "memory");
}

__device__ __forceinline__ bool elect_one() {
  uint32_t pred;
  asm volatile(
      "{\n\t.reg .pred p;\n\telect.sync _|p, 0xffffffff;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(pred));
  return pred != 0;
}

// 16 consecutive accumulator columns of this warp's 32 TMEM lanes.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}

// w[c] = D[.., t1 + c] + D[.., t2 + c] for c < 16: the products with B_hi
// and with B_lo of the same right-hand sides.
__device__ __forceinline__ void tmem_sum16(uint32_t t1, uint32_t t2, float (&w)[16]) {
  uint32_t r[16], r2[16];
  tmem_ld16(t1, r);
  tmem_ld16(t2, r2);
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int c = 0; c < 16; c++) w[c] = __uint_as_float(r[c]) + __uint_as_float(r2[c]);
}

__device__ __forceinline__ unsigned long long now_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

template <int R>
struct TcSmem {
  using Sh = TcShape<R>;
  unsigned char a[Sh::kStages][kABytes];
  unsigned char b[Sh::kStages][Sh::kBBytes];
  // per epilogue set: halves of the row sums handed from the lo-row warps to
  // the hi-row warps (xa) and back (xb)
  float xa[2][64][R / 2 + 1], xb[2][64][R / 2 + 1];
  uint64_t full[Sh::kStages], empty[Sh::kStages];
  uint64_t seg_full[Sh::kBufs], seg_empty[Sh::kBufs];  // per accumulator buffer
  uint64_t xa_ready[2], xa_free[2], xb_ready[2], xb_free[2];
  uint64_t qfull[kQ], qempty[kQ];
  TcItem qdata[kQ];  // item queue: ticket order; kind -1 ends it
  uint32_t tmem;
  volatile int32_t abort;
};
// 128 bytes of alignment slack on top (the tile loads and the no-swizzle
// operand layouts need 128-byte alignment at most); 232448 bytes is the
// per-block limit
constexpr size_t kSmemAlign = 128;
static_assert(sizeof(TcSmem<32>) + kSmemAlign <= 232448 && sizeof(TcSmem<64>) + kSmemAlign <= 232448,
              "tensor-core pass shared memory");

// Waits for the phase of `bar` with parity `parity`; false when the abort flag
// is up or the time limit ran out (then the flag goes up and `code` is recorded).
__device__ __forceinline__ bool try_bar(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(su32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// The bounded wait itself: an iteration cap backs up the timer.
__device__ __forceinline__ bool wait_bar_bounded(uint64_t *bar, uint32_t parity, volatile int32_t *abort,
                                                 int32_t *status, int code, unsigned long long limit_ns) {
  if (try_bar(bar, parity)) return true;  // the common case reads no timer
  const unsigned long long t0 = now_ns();
  for (unsigned long long it = 0;; it++) {
    if (try_bar(bar, parity)) return true;
    if (*abort) return false;
    if (now_ns() - t0 > limit_ns || it > kWaitIters) {
      atomicCAS(status, 0, code);
      *abort = 1;
      return false;
    }
  }
}

template <class SM>
__device__ __forceinline__ bool wait_bar(SM &S, uint64_t *bar, uint32_t parity, int32_t *status,
                                         int code) {
  return wait_bar_bounded(bar, parity, &S.abort, status, code, kWaitNs);
}

// wait_bar by every lane of a warp, with one answer for the whole warp
template <class SM>
__device__ __forceinline__ bool wait_bar_warp(SM &S, uint64_t *bar, uint32_t parity, int32_t *status,
                                              int code) {
  return __all_sync(0xffffffffu, wait_bar(S, bar, parity, status, code));
}

// Item n of this CTA from the queue (false: no more items, or an abort); every
// consumer warp calls it once per n and releases the slot. The item itself
// travels in the queue, so no consumer waits on a global load per item.
template <class SM>
__device__ __forceinline__ bool next_item(SM &S, int n, int32_t *status, TcItem &I) {
  const int q = n % kQ;
  if (!wait_bar_warp(S, &S.qfull[q], static_cast<uint32_t>((n / kQ) & 1), status, 30)) return false;
  I = S.qdata[q];
  __syncwarp();
  if ((threadIdx.x & 31) == 0) arrive(&S.qempty[q]);
  return I.kind >= 0;
}

__device__ __forceinline__ int64_t chunk_bytes(int G, int kc) { return static_cast<int64_t>(G) * kc * 16; }

__device__ __forceinline__ uint32_t pack2(float a, float b) {
  __half2 v = __floats2half2_rn(a, b);
  return *reinterpret_cast<uint32_t *>(&v);
}

// hi/lo split of 8 values (|v| < 2^16) into two 16-byte words of FP16:
// hi = fp16(v), lo = fp16(v - hi), v - hi exact in FP32
__device__ __forceinline__ void split8(const float *v, uint4 &hi, uint4 &lo) {
  float h[8];
#pragma unroll
  for (int i = 0; i < 8; i++) h[i] = __half2float(__float2half_rn(v[i]));
  hi = make_uint4(pack2(h[0], h[1]), pack2(h[2], h[3]), pack2(h[4], h[5]), pack2(h[6], h[7]));
  lo = make_uint4(pack2(v[0] - h[0], v[1] - h[1]), pack2(v[2] - h[2], v[3] - h[3]),
                  pack2(v[4] - h[4], v[5] - h[5]), pack2(v[6] - h[6], v[7] - h[7]));
}

// 2^e for the scale that puts a largest magnitude `mx` in [2^14, 2^15); 1 for
// a zero, infinite or NaN `mx` (the values then pass unscaled and a non-finite
// input stays non-finite). Exponents are clamped so that the scale and its
// inverse are normal FP32 numbers.
__device__ __forceinline__ float pow2_scale(float mx) {
  if (!(mx > 0.0f) || !isfinite(mx)) return 1.0f;
  int e = 14 - ilogbf(mx);
  e = max(-120, min(120, e));
  return __int_as_float((e + 127) << 23);
}

// Offset of the row factors (64 floats, then the item's batch member as an
// int32 and padding: kTrailer bytes) that trail an item's chunks.
__device__ __host__ __forceinline__ int64_t trailer_off(int m, int ncols) {
  const int64_t npad = ncols > 0 ? (ncols + 15) & ~15 : 16;
  return int64_t(32) * ((m + 7) / 8) * npad;
}

// Self-test of the bounded wait: a barrier nobody arrives at, waited on with
// a short limit; the wait must give up, record kSelfTestCode and return.
__global__ void wait_selftest_kernel(unsigned long long limit_ns, int32_t *status, unsigned long long *waited) {
  __shared__ uint64_t bar;
  __shared__ int32_t abort_flag;
  if (threadIdx.x != 0) return;
  abort_flag = 0;
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&bar)));
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  const unsigned long long t0 = now_ns();
  const bool done = wait_bar_bounded(&bar, 0, &abort_flag, status, kSelfTestCode, limit_ns);
  *waited = now_ns() - t0;
  if (done) atomicCAS(status, 0, -1);  // the phase cannot complete
}

struct TcArgs {
  CUtensorMap xmap;            // XTS as 8 FP16 x rows x N groups, 64-row boxes: the B tiles of V pieces
  CUtensorMap xmap8;           // the same view, 8-row boxes: K groups of near/U B tiles
  const unsigned char *adata;  // tensor-core panels
  const TcItem *items;
  int32_t nitems;
  int32_t grab;                // items per ticket while many remain (1 or 8)
  int32_t *ticket;             // next item (zeroed by the permutation kernel)
  const int32_t *colmap;
  const uint16_t *xts;         // XTS rows (2R FP16 each)
  const float *xs_inv;         // 1 / sigma per batch member and right-hand side (64 per member)
  uint16_t *xts_out;           // t rows (kind 1)
  float *prow;                 // P rows (kind 2)
  const TileDesc *tiles;
  const int32_t *tmap0;
  float *y;
  int64_t ldy;
  int32_t nr;
  int32_t zero_row;
  int32_t *status;
};

template <int R>
__global__ void __launch_bounds__(TcShape<R>::kThreads, 1) tc_kernel(const __grid_constant__ TcArgs a) {
  using Sh = TcShape<R>;
  constexpr int kStages = Sh::kStages;
  extern __shared__ unsigned char smem_raw[];
  TcSmem<R> &S = *reinterpret_cast<TcSmem<R> *>(
      (reinterpret_cast<uintptr_t>(smem_raw) + kSmemAlign - 1) & ~static_cast<uintptr_t>(kSmemAlign - 1));
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    S.abort = 0;
    for (int s = 0; s < kStages; s++) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&S.full[s])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&S.empty[s])));
    }
    for (int b = 0; b < Sh::kBufs; b++) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&S.seg_full[b])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 4;" ::"r"(su32(&S.seg_empty[b])));
    }
    for (int q = 0; q < kQ; q++) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&S.qfull[q])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(&S.qempty[q])), "r"(Sh::kConsumers));
    }
    for (int e = 0; e < 2; e++) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 2;" ::"r"(su32(&S.xa_ready[e])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 2;" ::"r"(su32(&S.xa_free[e])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 2;" ::"r"(su32(&S.xb_ready[e])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 2;" ::"r"(su32(&S.xb_free[e])));
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(&S.tmem)),
                 "r"(Sh::kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

  if (warp == 0) {
    // ---- item tickets, queued with the items for the other roles -------------
    // One atomic takes a.grab consecutive items while more than 16 per CTA
    // remain (one ticket round trip per a.grab short items), single items
    // after that so that the CTAs finish together. Lanes load the grabbed
    // items in parallel; lane 0 writes each into its queue slot.
    int n = 0, last = 0;
    for (bool more = true; more;) {
      const int want = last + 16 * static_cast<int>(gridDim.x) < a.nitems ? a.grab : 1;
      int b = 0;
      if (lane == 0) b = atomicAdd(a.ticket, want);
      b = __shfl_sync(0xffffffffu, b, 0);
      last = b;
      TcItem mine{};
      mine.kind = -1;
      if (lane < want && b + lane < a.nitems) mine = a.items[b + lane];
      for (int j = 0; j < want; j++, n++) {
        TcItem t;
        t.a_off = __shfl_sync(0xffffffffu, mine.a_off, j);
        t.m = __shfl_sync(0xffffffffu, mine.m, j);
        t.ncols = __shfl_sync(0xffffffffu, mine.ncols, j);
        t.map = __shfl_sync(0xffffffffu, mine.map, j);
        t.out = __shfl_sync(0xffffffffu, mine.out, j);
        t.kind = __shfl_sync(0xffffffffu, mine.kind, j);
        t.row0 = __shfl_sync(0xffffffffu, mine.row0, j);
        const int q = n % kQ;
        if (!wait_bar_warp(S, &S.qempty[q], static_cast<uint32_t>((n / kQ) & 1) ^ 1u, a.status, 29)) {
          more = false;
          break;
        }
        if (lane == 0) {
          S.qdata[q] = t;
          arrive(&S.qfull[q]);
        }
        if (t.kind < 0) {
          more = false;
          break;
        }
      }
    }
  } else if (warp == 1 || warp == 3 || (warp >= 8 && warp < Sh::kEpi1)) {
    // ---- producers: pipeline p = bw & 1 (items n with n & 1 == p); its chunk
    // g (stage p kPipeStages + g % kPipeStages) goes to its producer
    // q = g % kPipeStages. Column rows are looked up before the stage is
    // free; then each warp-wide copy moves kRowsPerCopy whole XTS rows
    // (kPieces lanes x 16 bytes per row), the warp waits for its copies,
    // fences them for the tensor cores' proxy and publishes the stage.
    const int bw = warp == 1 ? 0 : warp == 3 ? 1 : warp - 6;  // 0..kStages-1
    const int pipe = bw % Sh::kPipes, q = bw / Sh::kPipes;
    int64_t g = 0, last_g = -1;  // last_g: the chunk whose bulk copies this warp issued last
    bool stop = false;
    const int piece = lane % Sh::kPieces, sub = lane / Sh::kPieces;
    for (int n = 0; !stop; n++) {
      TcItem I;
      if (!next_item(S, n, a.status, I)) break;
      if ((n & 1) % Sh::kPipes != pipe) continue;
      const int npad = I.ncols > 0 ? (I.ncols + 15) & ~15 : 16;
      for (int c0 = 0; c0 < npad; c0 += kKc, g++) {
        if (g % Sh::kPipeStages != q) continue;
        const int kc = min(kKc, npad - c0), s = pipe * Sh::kPipeStages + static_cast<int>(g % Sh::kPipeStages);
        // B of a V piece by one tile load of 64 XTS rows (in a last chunk the
        // MMA warp zeroes the rows of padding columns before it multiplies)
        const bool tma_b = I.kind != 0;
        int rows[kKc / 32];  // XTS rows of columns c0 + lane + 32 h
#pragma unroll
        for (int h = 0; h < kKc / 32; h++) {
          const int c = c0 + lane + 32 * h;
          rows[h] = a.zero_row;
          if (c < I.ncols) rows[h] = I.kind == 0 ? __ldg(a.colmap + I.map + c) : I.map + c;
        }
        // near/U tiles: a K group of 8 columns that are 8 consecutive XTS rows
        // (most are: a tile's columns come in runs of whole source clusters
        // and rank ranges) arrives by one 8-row tile load straight into its
        // place in the B tile; the other groups are gathered row by row
        uint32_t gmask = 0;  // bit q: K group q by tile load
        int grow[kKc / 8];   // first XTS row of each K group
        if (!tma_b) {
#pragma unroll
          for (int h = 0; h < kKc / 32; h++) {
            const int prev = __shfl_up_sync(0xffffffffu, rows[h], 1);
            const bool ok = c0 + lane + 32 * h < I.ncols && ((lane & 7) == 0 || rows[h] == prev + 1);
            const uint32_t b = __ballot_sync(0xffffffffu, ok);
#pragma unroll
            for (int j = 0; j < 4; j++) {
              if (((b >> (8 * j)) & 0xffu) == 0xffu) gmask |= 1u << (4 * h + j);
              grow[4 * h + j] = __shfl_sync(0xffffffffu, rows[h], 8 * j);
            }
          }
          gmask &= (1u << (kc / 8)) - 1u;
        }
        if (!wait_bar_warp(S, &S.empty[s], static_cast<uint32_t>((g / Sh::kPipeStages) & 1) ^ 1u, a.status, 22)) {
          stop = true;
          break;
        }
        if (lane == 0) {
          // A: the chunk's hi rows to tile rows 0.., its lo rows to tile rows
          // 64..: two bulk copies that complete on the stage's barrier (read
          // once: evict-first in L2, so the gathered XTS rows stay resident)
          uint64_t pol;
          asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
          const int G = (I.m + 7) >> 3;
          const uint32_t half = static_cast<uint32_t>(G * kc * 16);
          const unsigned char *src = a.adata + I.a_off + static_cast<int64_t>(c0 / kKc) * 2 * chunk_bytes(G, kKc);
          const uint32_t hi = su32(S.a[s]), lo = hi + 128u * kc;
          const uint32_t bar = su32(&S.full[s]);
          const uint32_t btx = tma_b ? static_cast<uint32_t>(Sh::kBBytes)
                                     : static_cast<uint32_t>(__popc(gmask)) * Sh::kBGroupK;
          asm volatile("mbarrier.expect_tx.relaxed.cta.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(2 * half + btx)
                       : "memory");
          asm volatile(
              "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(hi),
              "l"(src), "r"(half), "r"(bar), "l"(pol)
              : "memory");
          asm volatile(
              "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(lo),
              "l"(src + half), "r"(half), "r"(bar), "l"(pol)
              : "memory");
          if (tma_b) {
            // B of a V piece: its columns are the consecutive XTS rows map + c0
            // .., so one tile load of 64 rows lands them in the canonical
            // MN-major layout (K groups 128 B apart, N groups 1024 B apart)
            asm volatile(
                "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, "
                "%4}], [%5];" ::"r"(su32(S.b[s])),
                "l"(reinterpret_cast<uint64_t>(&a.xmap)), "r"(0), "r"(I.map + c0), "r"(0), "r"(bar)
                : "memory");
            arrive(&S.full[s]);
          }
        }
        last_g = g;
        if (tma_b) {  // the copies complete on the stage's barrier
          __syncwarp();
          continue;
        }
        __syncwarp();  // the stage's expected bytes are set before any tile load lands
#pragma unroll
        for (int q = 0; q < kKc / 8; q++)
          if (lane == q && ((gmask >> q) & 1u))
            asm volatile(
                "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, "
                "%4}], [%5];" ::"r"(su32(S.b[s]) + static_cast<uint32_t>(q) * Sh::kBGroupK),
                "l"(reinterpret_cast<uint64_t>(&a.xmap8)), "r"(0), "r"(grow[q]), "r"(0), "r"(su32(&S.full[s]))
                : "memory");
        const uint32_t dst0 = su32(S.b[s]) + piece * kBGroupN;
#pragma unroll
        for (int i = 0; i < kKc / Sh::kRowsPerCopy; i++) {
          const int k = Sh::kRowsPerCopy * i + sub;
          const int r = __shfl_sync(0xffffffffu, rows[(i * Sh::kRowsPerCopy) >> 5], k & 31);
          if (k < kc && !((gmask >> (k >> 3)) & 1u)) {
            const uint16_t *src = a.xts + static_cast<int64_t>(r) * (2 * R) + piece * 8;
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst0 + (k >> 3) * Sh::kBGroupK + (k & 7) * 16),
                         "l"(src)
                         : "memory");
          }
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
        asm volatile("cp.async.wait_group 0;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncwarp();
        if (lane == 0) arrive(&S.full[s]);
      }
    }
    // The bulk copies of this warp's last chunk land before the CTA can exit,
    // aborted or not (one stage per producer: earlier chunks have landed).
    if (last_g >= 0 && lane == 0) {
      volatile int32_t none = 0;
      wait_bar_bounded(&S.full[pipe * Sh::kPipeStages + last_g % Sh::kPipeStages],
                       static_cast<uint32_t>((last_g / Sh::kPipeStages) & 1), &none, a.status, 31, kWaitNs);
    }
    __syncwarp();
  } else if (warp == 2 || (Sh::kPipes == 2 && warp == Sh::kMma1)) {
    // ---- MMA issuers: one warp per pipeline, one elected lane issues. The
    // issuing warp's own instructions per chunk (waits, fence, election,
    // UMMAs, commits) bound a single pipeline, so with two pipelines, each
    // with its own stages, they share the tensor cores.
    // Per 16 columns one UMMA: [A_hi; A_lo] (M = 128) x [B_hi B_lo] (N = 2R)
    // into the item's accumulator; the epilogue adds its four quadrants.
    const int pipe = warp == 2 ? 0 : 1;
    const int s0 = pipe * Sh::kPipeStages;  // the pipeline's first stage
    int64_t g = 0;                          // the pipeline's chunks so far
    int n = 0;
    bool stop = false;
    // Every kSegChunks chunks of an item go to a fresh accumulator buffer of
    // the item's epilogue set (set n & 1, buffers used in turn), whose warps
    // add the buffers' sums in FP32 registers: the tensor cores' own
    // accumulation then spans at most 4 kSegChunks UMMAs, whatever the item's
    // length.
    uint32_t kseg[2] = {0u, 0u};  // buffers handed to each epilogue set so far
    for (; !stop; n++) {
      TcItem I;
      if (!next_item(S, n, a.status, I)) break;
      if ((n & 1) % Sh::kPipes != pipe) continue;
      const int e = n & 1;
      const int npad = I.ncols > 0 ? (I.ncols + 15) & ~15 : 16;
      // V pieces' B tiles come from the tile load (K groups 128 B apart, N
      // groups 1024 B), near/U tiles' from the gather (kBGroupK, 128 B)
      const bool tma_b = I.kind != 0;
      const int kSegChunks = tma_b ? kSegChunksV : kSegChunksDU;
      // One pass of this loop per accumulator buffer: the segment's chunks
      // c0 / kKc .. + nseg - 1 (stages g .. g + nseg - 1) are waited for
      // first, then all their UMMAs go out under one fence and one election.
      // The warp's own per-chunk instructions are what bound the pass, so
      // they are paid once per segment. nseg <= kPipeStages: the producers of
      // the segment's chunks never wait for the segment itself.
      for (int c0 = 0; c0 < npad;) {
        const int nseg = min(kSegChunks, (npad - c0 + kKc - 1) / kKc);
        const int buf = e * Sh::kSetBufs + static_cast<int>(kseg[e] % Sh::kSetBufs);
        bool ok = wait_bar_warp(S, &S.seg_empty[buf], ((kseg[e] / Sh::kSetBufs) & 1u) ^ 1u, a.status, 23);
        for (int j = 0; ok && j < nseg; j++)
          ok = wait_bar_warp(S, &S.full[s0 + static_cast<int>((g + j) % Sh::kPipeStages)],
                             static_cast<uint32_t>(((g + j) / Sh::kPipeStages) & 1), a.status, 24);
        if (!ok) {
          stop = true;
          break;
        }
        const int cl = c0 + (nseg - 1) * kKc, kcl = min(kKc, npad - cl);  // the segment's last chunk
        if (tma_b && I.ncols - cl < kcl) {
          // the last chunk of a V piece: the tile load brought 64 consecutive
          // XTS rows, and those of the padding columns [ncols, kc) belong to
          // other blocks (or are t rows being rewritten). The A tile is zero
          // there, but 0 * Inf and 0 * NaN are not, so the rows are zeroed
          // (16 bytes per row and N group) before the UMMAs read them.
          const uint32_t bl = su32(S.b[s0 + static_cast<int>((g + nseg - 1) % Sh::kPipeStages)]);
          const int valid = I.ncols - cl, nz = kcl - valid;
          for (int z = lane; z < nz * (Sh::kBN / 8); z += 32) {
            const int k = valid + z % nz, gq = z / nz;
            asm volatile("st.shared.v4.b32 [%0], {%1, %1, %1, %1};" ::"r"(bl + gq * 1024u + k * 16u), "r"(0u)
                         : "memory");
          }
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
          __syncwarp();
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (elect_one()) {
          const uint32_t acc = S.tmem + static_cast<uint32_t>(buf * Sh::kBN);
          for (int j = 0; j < nseg; j++) {
            const int st = s0 + static_cast<int>((g + j) % Sh::kPipeStages), kc = min(kKc, npad - c0 - j * kKc);
            // leading byte offset: K direction; stride byte offset: N direction
            const uint64_t da = sdesc(su32(S.a[st]), 128, static_cast<uint32_t>(kc) * 16);
            const uint64_t db =
                tma_b ? sdesc(su32(S.b[st]), 128, 1024) : sdesc(su32(S.b[st]), Sh::kBGroupK, kBGroupN);
#pragma unroll
            for (int ks = 0; ks < kKc / 16; ks++) {
              if (ks < kc / 16) {
                // the start address field counts 16-byte units
                const uint64_t oa = static_cast<uint64_t>(ks * 256) >> 4,
                               ob = static_cast<uint64_t>(tma_b ? ks * 256 : ks * 2 * Sh::kBGroupK) >> 4;
                mma(acc, da + oa, db + ob, Sh::kIdesc, (j == 0 && ks == 0) ? 0u : 1u);
              }
            }
            commit(&S.empty[st]);
          }
          commit(&S.seg_full[buf]);
        }
        __syncwarp();
        kseg[e]++;
        g += nseg;
        c0 += nseg * kKc;
      }
    }
    // the last stage release must land before the CTA's shared memory goes away
    if (!stop && g > 0)
      wait_bar_warp(S, &S.empty[s0 + static_cast<int>((g - 1) % Sh::kPipeStages)],
                    static_cast<uint32_t>(((g - 1) / Sh::kPipeStages) & 1), a.status, 26);
  } else if ((warp >= 4 && warp < 8) || (warp >= Sh::kEpi1 && warp < Sh::kEpi1 + 4)) {
    // ---- epilogue -----------------------------------------------------------
    // Set e (warps 4-7 or the last four) takes accumulator e, that is items
    // n = e, e + 2, ... Warp w reads TMEM lanes 32(w mod 4)..: quarters 0, 1
    // hold the A_hi rows, quarters 2, 3 the A_lo rows of the same panel rows.
    // The hi-row warp hands the sums of right-hand sides [H, R) to its lo-row
    // partner and takes those of [0, H) from it (H = R / 2), so that each
    // finishes and writes half of the row; sum = hi-row part + lo-row part
    // either way.
    constexpr int H = R / 2;
    const int e = warp >= Sh::kEpi1 ? 1 : 0;
    const int quarter = warp & 3, row = (quarter & 1) * 32 + lane;
    const bool lo_part = quarter >= 2;
    const int keep = lo_part ? H : 0;
    float(*xo)[H + 1] = lo_part ? S.xa[e] : S.xb[e];  // written by this warp
    float(*xi)[H + 1] = lo_part ? S.xb[e] : S.xa[e];  // read by this warp
    uint64_t *o_ready = lo_part ? &S.xa_ready[e] : &S.xb_ready[e];
    uint64_t *o_free = lo_part ? &S.xa_free[e] : &S.xb_free[e];
    uint64_t *i_ready = lo_part ? &S.xb_ready[e] : &S.xa_ready[e];
    uint64_t *i_free = lo_part ? &S.xb_free[e] : &S.xa_free[e];
    uint32_t kseg = 0;  // accumulator buffers of this set consumed so far
    for (int n = 0;; n++) {
      TcItem I;
      if (!next_item(S, n, a.status, I)) break;
      if ((n & 1) != e) continue;
      const uint32_t k = static_cast<uint32_t>(n >> 1);  // this set's item count
      const int nch = ((I.ncols > 0 ? (I.ncols + 15) & ~15 : 16) + kKc - 1) / kKc;
      const int span = I.kind != 0 ? kSegChunksV : kSegChunksDU;
      const int nbuf = (nch + span - 1) / span;  // accumulator buffers of the item
      // the row's factor (1 / rho_i, or gamma_k / nu_k for V rows) and, for y
      // rows, the output row and the member, loaded now: they do not depend on
      // the MMA, so their latency hides behind its wait
      const bool has_row = row < I.m;
      const float *trailer = reinterpret_cast<const float *>(a.adata + I.a_off + trailer_off(I.m, I.ncols));
      const float f = has_row ? __ldg(trailer + row) : 0.0f;
      int64_t yrow = 0;
      int mem = 0;
      if (I.kind == 0 && has_row) {
        yrow = a.tmap0[a.tiles[I.out].row0 + I.row0 + row];
        mem = __float_as_int(__ldg(trailer + 64));
      }
      // w[c]: A_part B_hi + A_part B_lo of right-hand side c, chunk by chunk
      float w[R];
#pragma unroll
      for (int c = 0; c < R; c++) w[c] = 0.0f;
      bool ok = true;
      for (int ch = 0; ch < nbuf; ch++, kseg++) {
        const int buf = e * Sh::kSetBufs + static_cast<int>(kseg % Sh::kSetBufs);
        if (!wait_bar_warp(S, &S.seg_full[buf], (kseg / Sh::kSetBufs) & 1u, a.status, 25)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t taddr = S.tmem + static_cast<uint32_t>(buf * Sh::kBN) + (static_cast<uint32_t>(quarter * 32) << 16);
#pragma unroll
        for (int c0 = 0; c0 < R; c0 += 16) {
          float d[16];
          tmem_sum16(taddr + c0, taddr + R + c0, d);
#pragma unroll
          for (int c = 0; c < 16; c++) w[c0 + c] += d[c];
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncwarp();
        if (lane == 0) arrive(&S.seg_empty[buf]);
      }
      if (!ok) break;
      // the hi-row warp keeps right-hand sides [0, H), the lo-row warp [H, R)
      // (selects, not a runtime index: w stays in registers)
      if (!wait_bar_warp(S, o_free, (k & 1u) ^ 1u, a.status, 27)) break;
#pragma unroll
      for (int c = 0; c < H; c++) xo[row][c] = lo_part ? w[c] : w[H + c];
      __syncwarp();
      if (lane == 0) arrive(o_ready);
      if (!wait_bar_warp(S, i_ready, k & 1u, a.status, 28)) break;
      float v[H];
#pragma unroll
      for (int c = 0; c < H; c++) v[c] = (lo_part ? w[H + c] : w[c]) + xi[row][c];
      __syncwarp();
      if (lane == 0) arrive(i_free);
      if (!has_row) continue;
#pragma unroll
      for (int c = 0; c < H; c++) v[c] *= f;
      if (I.kind == 0) {
        float *yr = a.y + yrow;
        const float *xs = a.xs_inv + mem * kTcMaxRhs + keep;  // its member's
#pragma unroll
        for (int c = 0; c < H; c++)
          if (keep + c < a.nr) yr[(keep + c) * a.ldy] = v[c] * __ldg(xs + c);
      } else if (I.kind == 1) {
        uint4 *dst = reinterpret_cast<uint4 *>(a.xts_out + static_cast<int64_t>(I.out + row) * (2 * R)) + keep / 8;
#pragma unroll
        for (int q = 0; q < H / 8; q++) {
          uint4 hi, lo;
          split8(v + 8 * q, hi, lo);
          dst[q] = hi;
          dst[R / 8 + q] = lo;
        }
      } else {
        float4 *dst = reinterpret_cast<float4 *>(a.prow + static_cast<int64_t>(I.out + row) * R + keep);
#pragma unroll
        for (int q = 0; q < H / 4; q++) dst[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(S.tmem), "r"(Sh::kTmemCols));
}

// Batch member of source index j: the largest k with col0[k] <= j.
__device__ __forceinline__ int member_of(const int64_t *col0, int nmem, int64_t j) {
  int lo = 0, hi = nmem - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (col0[mid] <= j)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// max |X[., r]| per batch member and right-hand side r < nr, as FP32 bits
// (non-negative floats order as unsigned integers) into xmax[member * 64 + r],
// which starts at zero. Members own the contiguous source ranges [col0[k],
// col0[k + 1]). Block x takes source indices [x kXmaxSpan, (x + 1)
// kXmaxSpan), its warp w right-hand side 8 y + w: coalesced loads along the
// indices, eight in flight per lane, one atomic per member met.
constexpr int kXmaxSpan = 2048;
__global__ void xmax_kernel(const float *__restrict__ X, int64_t ldx, int nr, int64_t n_src,
                            const int64_t *__restrict__ col0, int nmem, unsigned *__restrict__ xmax) {
  const int lane = threadIdx.x & 31;
  const int r = blockIdx.y * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (r >= nr) return;
  const int64_t j0 = blockIdx.x * static_cast<int64_t>(kXmaxSpan), j1 = min(n_src, j0 + kXmaxSpan);
  const float *xr = X + r * ldx;
  for (int k = member_of(col0, nmem, j0); k < nmem && col0[k] < j1; k++) {
    const int64_t a0 = max(j0, col0[k]), a1 = min(j1, col0[k + 1]);
    unsigned m = 0u;
    int64_t j = a0 + lane;
    for (; j + 224 < a1; j += 256) {
      float v[8];
#pragma unroll
      for (int i = 0; i < 8; i++) v[i] = xr[j + 32 * i];
#pragma unroll
      for (int i = 0; i < 8; i++) m = max(m, __float_as_uint(fabsf(v[i])));
    }
    for (; j < a1; j += 32) m = max(m, __float_as_uint(fabsf(xr[j])));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0 && a1 > a0) atomicMax(&xmax[k * kTcMaxRhs + r], m);
  }
}

// sigma per member and right-hand side (sig) and its inverse (xs_inv), from
// the maxima; right-hand sides past nr get 1.
__global__ void sigma_kernel(const unsigned *__restrict__ xmax, int nmem, int nr, float *__restrict__ sig,
                             float *__restrict__ xs_inv) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nmem * kTcMaxRhs; e += gridDim.x * blockDim.x) {
    const int r = e % kTcMaxRhs;
    const float s = r < nr ? pow2_scale(__uint_as_float(xmax[e])) : 1.0f;
    sig[e] = s;
    xs_inv[e] = 1.0f / s;
  }
}

// XTS x rows from X in its own order: the R right-hand sides X[j + r ldx]
// (0 for r >= nr) of source index j, times sigma of (j's batch member, r),
// split into FP16 hi (first 2R bytes) and lo (last 2R bytes), go to row
// sinv[j]. Reads of X are coalesced along j and every row is written whole;
// x-region rows that no source index maps to stay zero from the allocation.
// Also re-arms the two item tickets.
template <int R>
__global__ void permute_split_kernel(const float *__restrict__ X, int64_t ldx, int nr,
                                     const int32_t *__restrict__ sinv0, int64_t n_src,
                                     uint16_t *__restrict__ xts, int32_t *__restrict__ tickets,
                                     const int64_t *__restrict__ col0, int nmem, const float *__restrict__ sig) {
  __shared__ float tile[64][R + 1];
  __shared__ int mem[64];
  if (blockIdx.x == 0 && threadIdx.x < 2) tickets[threadIdx.x] = 0;  // V and near/U item tickets
  for (int64_t j0 = blockIdx.x * 64ll; j0 < n_src; j0 += gridDim.x * 64ll) {
    if (threadIdx.x < 64) mem[threadIdx.x] = member_of(col0, nmem, min(j0 + threadIdx.x, n_src - 1));
    __syncthreads();
    for (int e = threadIdx.x; e < 64 * R; e += blockDim.x) {
      const int r = e / 64, jj = e % 64;  // consecutive threads: consecutive j
      const int64_t j = j0 + jj;
      tile[jj][r] = (j < n_src && r < nr) ? X[j + r * ldx] * __ldg(sig + mem[jj] * kTcMaxRhs + r) : 0.0f;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < 64 * (R / 8); e += blockDim.x) {
      const int jj = e / (R / 8), q = e % (R / 8);
      if (j0 + jj < n_src) {
        float v[8];
#pragma unroll
        for (int i = 0; i < 8; i++) v[i] = tile[jj][8 * q + i];
        uint4 hi, lo;
        split8(v, hi, lo);
        uint4 *dst = reinterpret_cast<uint4 *>(xts + static_cast<int64_t>(sinv0[j0 + jj]) * (2 * R));
        dst[q] = hi;
        dst[R / 8 + q] = lo;
      }
    }
    __syncthreads();
  }
}

// t rows from partial rows (already scaled by their rows' factors), pieces
// summed in order; one warp per row, lane = right-hand side (and lane + 32 in
// a 64-wide pass).
template <int R>
__global__ void reduce_split_kernel(const MVReduce *__restrict__ red, int32_t nred, const float *__restrict__ P,
                                    uint16_t *__restrict__ xts) {
  const int lane = threadIdx.x & 31;
  for (int32_t e = static_cast<int32_t>(blockIdx.x); e < nred; e += gridDim.x) {
    const MVReduce D = red[e];
    for (int row = threadIdx.x >> 5; row < D.nrows; row += blockDim.x >> 5) {
      uint16_t *dst = xts + static_cast<int64_t>(D.t_row + row) * (2 * R);
#pragma unroll
      for (int c = lane; c < R; c += 32) {
        float s = 0.0f;
        for (int j = 0; j < D.npieces; j++)
          s += P[(static_cast<int64_t>(D.p_row) + static_cast<int64_t>(j) * D.nrows + row) * R + c];
        const __half hb = __float2half_rn(s);
        const __half lb = __float2half_rn(s - __half2float(hb));
        dst[c] = *reinterpret_cast<const uint16_t *>(&hb);
        dst[R + c] = *reinterpret_cast<const uint16_t *>(&lb);
      }
    }
  }
}

// Scales of the rank rows, from the FP32 V rows of each source group (one
// block per group, a warp per row): nu[t] = pow2_scale(max |V_t|) and
// gam[t] = 2^-ceil(log2 ||V_t||_1) (1 for a zero row), at the row's XT row t;
// colsc[t] = 1 / gam[t] (colsc is 1 on the x rows).
__global__ void tscale_kernel(const VGroup *__restrict__ groups, const float *__restrict__ vdata,
                              float *__restrict__ nu, float *__restrict__ gam, float *__restrict__ colsc) {
  const VGroup g = groups[blockIdx.x];
  const int lane = threadIdx.x & 31;
  for (int r = threadIdx.x >> 5; r < g.rows; r += blockDim.x >> 5) {
    const float *v = vdata + g.v_off + static_cast<int64_t>(r) * g.stride;
    float mx = 0.0f, l1 = 0.0f;
    for (int j = lane; j < g.stride; j += 32) {
      const float a = fabsf(v[j]);
      mx = fmaxf(mx, a);
      l1 += a;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
      l1 += __shfl_xor_sync(0xffffffffu, l1, o);
    }
    if (lane == 0) {
      float gm = 1.0f;
      if (l1 > 0.0f && isfinite(l1)) {
        // the smallest power of two >= l1, with a margin for the rounding of l1
        int e = ilogbf(l1 * 1.0001f) + 1;
        e = max(-120, min(120, e));
        gm = __int_as_float((127 - e) << 23);
      }
      const int64_t t = static_cast<int64_t>(g.t_off) + r;
      nu[t] = pow2_scale(mx);
      gam[t] = gm;
      colsc[t] = 1.0f / gm;
    }
  }
}

__global__ void fill_kernel(float *__restrict__ p, int64_t n, float v) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    p[i] = v;
}

// Canonical FP16 (hi, lo) chunks of one item from its FP32 row-major source,
// with the item's row factors after them. Near/U rows (kind 0): every column
// times colsc of its XT row, the row scaled by rho_i = pow2_scale(its largest
// magnitude), factor 1 / rho_i. V rows (kind 1): scaled by nu of their rank
// row, factor gam / nu.
__global__ void pack_tc_kernel(const TcPack *__restrict__ jobs, const float *__restrict__ src,
                               unsigned char *__restrict__ adata, const int32_t *__restrict__ colmap,
                               const float *__restrict__ colsc, const float *__restrict__ nu,
                               const float *__restrict__ gam) {
  const TcPack J = jobs[blockIdx.x];
  __shared__ float rs[64], fac[64];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  auto csc = [&](int c) { return J.kind == 0 ? colsc[colmap[J.map + c]] : 1.0f; };
  for (int r = warp; r < 64; r += blockDim.x >> 5) {
    float sc = 1.0f, f = 0.0f;
    if (r < J.m) {
      if (J.kind == 0) {
        float mx = 0.0f;
        for (int c = lane; c < J.ncols; c += 32)
          mx = fmaxf(mx, fabsf(src[J.src_off + static_cast<int64_t>(r) * J.ld + c] * csc(c)));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        sc = pow2_scale(mx);
        f = 1.0f / sc;
      } else {
        sc = nu[J.trow + r];
        f = gam[J.trow + r] / sc;
      }
    }
    if (lane == 0) {
      rs[r] = sc;
      fac[r] = f;
    }
  }
  __syncthreads();
  const int G = (J.m + 7) >> 3;
  const int npad = J.ncols > 0 ? (J.ncols + 15) & ~15 : 16;
  unsigned char *base = adata + J.a_off;
  for (int c0 = 0; c0 < npad; c0 += kKc) {
    const int kc = min(kKc, npad - c0);
    const int64_t half = static_cast<int64_t>(G) * kc * 16;
    const int units = G * 8 * (kc / 8);  // (row, 8 columns)
    for (int u = threadIdx.x; u < units; u += blockDim.x) {
      const int r = u / (kc / 8), k8 = (u % (kc / 8)) * 8;
      float v[8];
#pragma unroll
      for (int i = 0; i < 8; i++) {
        const int c = c0 + k8 + i;
        v[i] = (r < J.m && c < J.ncols) ? src[J.src_off + static_cast<int64_t>(r) * J.ld + c] * csc(c) * rs[r]
                                        : 0.0f;
      }
      uint4 hi, lo;
      split8(v, hi, lo);
      const int64_t off = static_cast<int64_t>(r >> 3) * kc * 16 + (k8 >> 3) * 128 + (r & 7) * 16;
      *reinterpret_cast<uint4 *>(base + off) = hi;
      *reinterpret_cast<uint4 *>(base + half + off) = lo;
    }
    base += 2 * half;
  }
  float *tr = reinterpret_cast<float *>(adata + J.a_off + trailer_off(J.m, J.ncols));
  for (int r = threadIdx.x; r < 68; r += blockDim.x) tr[r] = r < 64 ? fac[r] : __int_as_float(r == 64 ? J.member : 0);
}

}  // namespace

template <int R>
static size_t smem_bytes() {
  return sizeof(TcSmem<R>) + kSmemAlign;
}
size_t tc_smem_bytes(int nr) { return nr > 32 ? smem_bytes<64>() : smem_bytes<32>(); }

static void tc_attrs() {
  static bool done = false;
  if (done) return;
  cudaFuncSetAttribute(tc_kernel<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem_bytes<32>()));
  cudaFuncSetAttribute(tc_kernel<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem_bytes<64>()));
  done = true;
}

cudaError_t encode_xts_map(DevTc &t, int R) {
  // cuTensorMapEncodeTiled through the runtime's driver entry point (no
  // link-time dependence on the driver library)
  static PFN_cuTensorMapEncodeTiled_v12000 enc = [] {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
  }();
  uint16_t *xts = R == 64 ? t.xts64 : t.xts;
  if (!enc || !xts || t.xt_rows < 8 || (R != 32 && R != 64)) return cudaErrorInvalidValue;
  // element (e, row, g) = XTS[row][8 g + e]: a box of 8 x 64 x 2R/8 lands as
  // 2R/8 N groups of 64 rows x 16 bytes
  cuuint64_t dims[3] = {8, static_cast<cuuint64_t>(t.xt_rows), static_cast<cuuint64_t>(2 * R / 8)};
  cuuint64_t strides[2] = {static_cast<cuuint64_t>(4 * R), 16};
  for (int b = 0; b < 2; b++) {  // boxes of 64 rows (V pieces) and of 8 rows (K groups of near/U tiles)
    cuuint32_t box[3] = {8, b == 0 ? 64u : 8u, static_cast<cuuint32_t>(2 * R / 8)};
    cuuint32_t es[3] = {1, 1, 1};
    const CUresult r = enc(&t.xmap[2 * b + R / 64], CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 3, xts, dims, strides, box, es,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return cudaErrorInvalidValue;
  }
  return cudaSuccess;
}

template <int R>
static int run_tc(const DevPlan &p, const DevTc &t, const float *X, int64_t ldx, int nr, float *Y, int64_t ldy,
                  cudaStream_t s, cudaEvent_t *ev) {
  using Sh = TcShape<R>;
  uint16_t *xts = R == 64 ? t.xts64 : t.xts;
  int nl = 0;
  int gp = static_cast<int>((p.n_src + 63) / 64);
  if (gp > 8192) gp = 8192;
  if (ev) cudaEventRecord(ev[0], s);
  // per member and right-hand side: max |x| bits, sigma, 1 / sigma
  const int64_t nm64 = static_cast<int64_t>(t.nmem) * kTcMaxRhs;
  unsigned *xmax = reinterpret_cast<unsigned *>(t.xscale);
  float *sig = t.xscale + nm64, *xs_inv = t.xscale + 2 * nm64;
  cudaMemsetAsync(xmax, 0, nm64 * sizeof(unsigned), s);
  const dim3 gx(static_cast<unsigned>((p.n_src + kXmaxSpan - 1) / kXmaxSpan), static_cast<unsigned>((nr + 7) / 8));
  xmax_kernel<<<gx, 256, 0, s>>>(X, ldx, nr, p.n_src, t.mcol0, t.nmem, xmax);
  sigma_kernel<<<static_cast<unsigned>((nm64 + 255) / 256), 256, 0, s>>>(xmax, t.nmem, nr, sig, xs_inv);
  permute_split_kernel<R><<<gp, 256, 0, s>>>(X, ldx, nr, p.sinv0, p.n_src, xts, p.counter + 2, t.mcol0, t.nmem,
                                              sig);
  nl += 3;
  if (ev) cudaEventRecord(ev[1], s);
  TcArgs a{};
  a.xmap = t.xmap[R / 64];
  a.xmap8 = t.xmap[2 + R / 64];
  a.adata = static_cast<const unsigned char *>(t.adata);
  a.colmap = t.colmap;
  a.xts = xts;
  a.xs_inv = xs_inv;
  a.xts_out = xts;
  a.prow = t.prow;
  a.tiles = p.tiles;
  a.tmap0 = p.tmap0;
  a.y = Y;
  a.ldy = ldy;
  a.nr = nr;
  a.zero_row = static_cast<int32_t>(p.zero_row);
  a.status = p.status;
  const size_t smem = smem_bytes<R>();
  if (t.n_v > 0) {
    a.items = t.v_items;
    a.nitems = t.n_v;
    a.grab = 8;  // V pieces are short: a few chunks each
    a.ticket = p.counter + 2;
    tc_kernel<R><<<t.ctas, Sh::kThreads, smem, s>>>(a);
    nl++;
    if (t.n_reduce > 0) {
      reduce_split_kernel<R><<<t.n_reduce < 4096 ? t.n_reduce : 4096, 256, 0, s>>>(t.reduce, t.n_reduce, t.prow, xts);
      nl++;
    }
  }
  if (ev) cudaEventRecord(ev[2], s);
  a.items = t.du_items;
  a.nitems = t.n_du;
  a.grab = 1;  // row tiles are long; single tickets keep neighbouring tiles together
  a.ticket = p.counter + 3;
  tc_kernel<R><<<t.ctas, Sh::kThreads, smem, s>>>(a);
  nl++;
  if (ev) cudaEventRecord(ev[3], s);
  return nl;
}

cudaError_t launch_tc_scales(const VGroup *groups, int64_t ngroups, const float *vdata, int64_t xt_rows,
                             float *nu, float *gam, float *colsc, cudaStream_t s) {
  fill_kernel<<<1024, 256, 0, s>>>(colsc, xt_rows, 1.0f);
  for (int64_t g0 = 0; g0 < ngroups; g0 += 65535) {
    const int nb = static_cast<int>(ngroups - g0 < 65535 ? ngroups - g0 : 65535);
    tscale_kernel<<<nb, 256, 0, s>>>(groups + g0, vdata, nu, gam, colsc);
  }
  return cudaGetLastError();
}

cudaError_t launch_pack_tc(const TcPack *jobs, int64_t njobs, const float *src, void *adata, const int32_t *colmap,
                           const float *colsc, const float *nu, const float *gam, cudaStream_t s) {
  for (int64_t j0 = 0; j0 < njobs; j0 += 65535) {
    const int nb = static_cast<int>(njobs - j0 < 65535 ? njobs - j0 : 65535);
    pack_tc_kernel<<<nb, 256, 0, s>>>(jobs + j0, src, static_cast<unsigned char *>(adata), colmap, colsc, nu, gam);
  }
  return cudaGetLastError();
}

cudaError_t launch_matvec_tc(const DevPlan &p, const DevTc &t, const float *X, int64_t ldx, int nr,
                             float *Y, int64_t ldy, cudaStream_t s, cudaEvent_t *ev, int *launches) {
  if (nr < 1 || nr > 64 || (nr > 32 && !t.xts64) || !t.xts || !t.xscale || !t.mcol0 || t.nmem < 1)
    return cudaErrorInvalidValue;
  tc_attrs();
  const int nl = nr > 32 ? run_tc<64>(p, t, X, ldx, nr, Y, ldy, s, ev) : run_tc<32>(p, t, X, ldx, nr, Y, ldy, s, ev);
  if (launches) *launches = nl;
  return cudaGetLastError();
}

}  // namespace hm

extern "C" int hmgpu_selftest_bounded_wait(int64_t limit_ns, int32_t *code, double *waited_ms) {
  if (!code || !waited_ms) return hm::fail(HMGPU_ERR_INVALID, "NULL argument");
  if (limit_ns < 1000000 || limit_ns > 2000000000)
    return hm::fail(HMGPU_ERR_INVALID, "limit must lie in [1 ms, 2 s]");
  int32_t *dst = nullptr;
  unsigned long long *dw = nullptr;
  cudaError_t e = cudaMalloc(&dst, sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMalloc(&dw, sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMemset(dst, 0, sizeof(int32_t));
  if (e == cudaSuccess) {
    hm::wait_selftest_kernel<<<1, 32>>>(static_cast<unsigned long long>(limit_ns), dst, dw);
    e = cudaGetLastError();
  }
  int32_t st = 0;
  unsigned long long w = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&st, dst, sizeof st, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(&w, dw, sizeof w, cudaMemcpyDeviceToHost);
  if (dst) cudaFree(dst);
  if (dw) cudaFree(dw);
  if (e != cudaSuccess)
    return hm::fail(HMGPU_ERR_CUDA, std::string("bounded-wait self-test: ") + cudaGetErrorString(e));
  *code = st;
  *waited_ms = static_cast<double>(w) * 1e-6;
  return HMGPU_OK;
}
