// Mixed-precision multi-right-hand-side product on the 5th-generation tensor
// cores (tcgen05, sm_103a): Y = H X for up to 32 right-hand sides per pass.
//
// Storage. Every panel of the product (a row tile of the near/U pass, or a
// column piece of at most 128 V rows of a source group) is stored once more as
// BF16 pairs a = hi + lo (hi = bf16(a), lo = bf16(a - hi); relative residual
// about 2^-17; all four products of the hi/lo pairs are formed), already in
// the UMMA canonical K-major layout, 64 columns per
// chunk, so a chunk is two contiguous byte ranges copied as they are. The right-hand sides live in XTS, one 128-byte
// row per entry of XT = [x permuted | t]: 32 BF16 hi values, then 32 lo values.
//
// Pipeline (one persistent CTA per SM; items from a ticket counter, in list
// order, so concurrent CTAs work on neighbouring panels and share XTS rows in
// L2; warp 0 takes the tickets and queues them for the other roles):
//   warp 0      item tickets (lane 0), queued in shared memory for the others;
//   warps 1, 3, 8-13  producers (chunk g to producer g mod 8) of an 8-stage
//               ring of 64-column chunks: 16-byte cp.async copies of the chunk (hi rows to tile
//               rows 0..63, lo rows to tile rows 64..127) and gathers of the
//               XTS rows of its columns (whole 128-byte rows) into an N-major
//               (MN-major) BF16 tile, then a wait, a proxy fence and an
//               mbarrier arrive;
//   warp 2      MMA issuer (one elected lane): per 16 columns one UMMA,
//               [A_hi; A_lo] x [B_hi B_lo] with M = 128, N = 64 (hi and lo
//               stacked along both M and N; items have at most 64 rows), into
//               one of two 64-column TMEM accumulators (FP32); commits free the
//               stage and, at the end of an item, hand the accumulator on;
//   warps 4-7   epilogue: tcgen05.ld of TMEM lanes 32(w-4).., the sum of the
//               four hi/lo quadrants, then y rows, t rows of XTS (split again)
//               or partial rows P.
// Every wait is bounded by the global timer; one that runs out records a code
// in `status`, raises a CTA-wide abort flag and every role leaves its loop.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "hm_device.h"

namespace hm {

namespace {

constexpr int kTcWarps = 14;   // roles: see the header comment
constexpr int kBProducers = 8;  // warps 1, 3, 8..13
constexpr int kTcThreads = kTcWarps * 32;
constexpr int kTcRhs = 32;
constexpr int kKc = 64;             // columns per chunk
constexpr int kStages = 8;
constexpr int kABytes = 128 * kKc * 2;    // A tile: 64 hi rows, then 64 lo rows: 16 KB
constexpr int kBN = 2 * kTcRhs;           // B rows: 32 hi right-hand sides, then 32 lo
constexpr int kBBytes = kBN * kKc * 2;    // one BF16 B tile: 8 KB
constexpr uint32_t kTmemCols = 128;       // two 64-column accumulators
constexpr int kQ = 16;                    // item queue slots
constexpr int kConsumers = kBProducers + 1 + 4;  // warps that read each queued item
// One producer per stage: a producer then never waits for a stage more than one
// release ahead, which a parity wait on the stage's barrier could not tell
// apart from the release before.
static_assert(kBProducers == kStages, "one producer warp per stage");
constexpr unsigned long long kWaitNs = 2000000000ull;  // 2 s per wait
constexpr unsigned long long kWaitIters = 1ull << 26;   // backstop if the timer stood still
constexpr int kSelfTestCode = 90;                        // status of the self-test's wait

// MN-major B with N = 64: the hi and lo halves of the 32 right-hand sides are
// stacked along N, so one XTS row (128 bytes) is one K row of B. Core
// matrices of 8 N values (16 B) x 8 columns; the 8 N groups are kBGroupN
// bytes apart, the K groups of 8 columns kBGroupK bytes apart.
constexpr uint32_t kBGroupN = 128;
constexpr uint32_t kBGroupK = 8 * kBGroupN;
constexpr uint32_t kBLbo = kBGroupK;  // leading byte offset: K direction
constexpr uint32_t kBSbo = kBGroupN;  // stride byte offset: N direction

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

// kind::f16 instruction descriptor: FP32 D, BF16 A (K-major) and B (MN-major),
// N = 64, M = 128.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | (1u << 16) |
                            ((static_cast<uint32_t>(kBN) >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ void mma(uint32_t tmem, uint64_t a, uint64_t b, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
      "l"(a), "l"(b), "r"(kIdesc), "r"(acc));
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

// 32 consecutive accumulator columns of this warp's 32 TMEM lanes.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]),
        "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]),
        "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
}

__device__ __forceinline__ unsigned long long now_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

struct TcSmem {
  unsigned char a[kStages][kABytes];
  unsigned char b[kStages][kBBytes];
  float epi[64][kTcRhs + 1];  // lo-row sums handed from epilogue warps 6, 7 to 4, 5
  uint64_t full[kStages], empty[kStages], acc_full[2], acc_empty[2], epi_ready, epi_free;
  uint64_t qfull[kQ], qempty[kQ];
  int32_t qitem[kQ];  // item queue: ticket order, -1 ends it
  uint32_t tmem;
  volatile int32_t abort;
};

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

__device__ __forceinline__ bool wait_bar(TcSmem &S, uint64_t *bar, uint32_t parity, int32_t *status,
                                         int code) {
  return wait_bar_bounded(bar, parity, &S.abort, status, code, kWaitNs);
}

// wait_bar by every lane of a warp, with one answer for the whole warp
__device__ __forceinline__ bool wait_bar_warp(TcSmem &S, uint64_t *bar, uint32_t parity, int32_t *status,
                                              int code) {
  return __all_sync(0xffffffffu, wait_bar(S, bar, parity, status, code));
}

// Item n of this CTA from the queue (-1: no more items, or an abort); every
// consumer warp calls it once per n and releases the slot.
__device__ __forceinline__ int next_item(TcSmem &S, int n, int32_t *status) {
  const int q = n % kQ;
  if (!wait_bar_warp(S, &S.qfull[q], static_cast<uint32_t>((n / kQ) & 1), status, 30)) return -1;
  const int it = S.qitem[q];
  __syncwarp();
  if ((threadIdx.x & 31) == 0) arrive(&S.qempty[q]);
  return it;
}

__device__ __forceinline__ int64_t chunk_bytes(int G, int kc) { return static_cast<int64_t>(G) * kc * 16; }

__device__ __forceinline__ uint32_t pack2(float a, float b) {
  __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t *>(&v);
}

// hi/lo split of 8 values into two 16-byte words
__device__ __forceinline__ void split8(const float *v, uint4 &hi, uint4 &lo) {
  float h[8];
#pragma unroll
  for (int i = 0; i < 8; i++) h[i] = __bfloat162float(__float2bfloat16_rn(v[i]));
  hi = make_uint4(pack2(h[0], h[1]), pack2(h[2], h[3]), pack2(h[4], h[5]), pack2(h[6], h[7]));
  lo = make_uint4(pack2(v[0] - h[0], v[1] - h[1]), pack2(v[2] - h[2], v[3] - h[3]),
                  pack2(v[4] - h[4], v[5] - h[5]), pack2(v[6] - h[6], v[7] - h[7]));
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
  const unsigned char *adata;  // tensor-core panels
  const TcItem *items;
  int32_t nitems;
  int32_t *ticket;             // next item (zeroed by the permutation kernel)
  const int32_t *colmap;
  const uint16_t *xts;         // XTS rows (64 BF16 each)
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

__global__ void __launch_bounds__(kTcThreads, 1) tc_kernel(TcArgs a) {
  extern __shared__ unsigned char smem_raw[];
  TcSmem &S = *reinterpret_cast<TcSmem *>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    S.abort = 0;
    for (int s = 0; s < kStages; s++) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&S.full[s])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&S.empty[s])));
    }
    for (int b = 0; b < 2; b++) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&S.acc_full[b])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 4;" ::"r"(su32(&S.acc_empty[b])));
    }
    for (int q = 0; q < kQ; q++) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&S.qfull[q])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(&S.qempty[q])), "r"(kConsumers));
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 2;" ::"r"(su32(&S.epi_ready)));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 2;" ::"r"(su32(&S.epi_free)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(&S.tmem)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

  if (warp == 0) {
    // ---- A producer ---------------------------------------------------------
    // ---- item tickets: lane 0 takes them and queues them for the others ----
    if (lane == 0) {
      for (int n = 0; !S.abort; n++) {
        const int q = n % kQ;
        if (!wait_bar(S, &S.qempty[q], static_cast<uint32_t>((n / kQ) & 1) ^ 1u, a.status, 29)) break;
        int it = atomicAdd(a.ticket, 1);
        if (it >= a.nitems) it = -1;
        S.qitem[q] = it;
        arrive(&S.qfull[q]);
        if (it < 0) break;
      }
    }
  } else if (warp == 1 || warp == 3 || warp >= 8) {
    // ---- producers: chunk g (stage g % 8) goes to producer g % 8 --------------
    // Column rows are looked up before the stage is free; then each of kKc / 4
    // instructions copies 4 whole XTS rows (8 lanes x 16 bytes per row), the
    // warp waits for its copies, fences them for the tensor cores' proxy and
    // publishes the stage.
    const int bw = warp == 1 ? 0 : warp == 3 ? 1 : warp - 6;  // 0..7
    int64_t g = 0;
    bool stop = false;
    const int piece = lane & 7, sub = lane >> 3;
    for (int n = 0; !stop; n++) {
      const int it = next_item(S, n, a.status);
      if (it < 0) break;
      const TcItem I = a.items[it];
      const int npad = I.ncols > 0 ? (I.ncols + 15) & ~15 : 16;
      for (int c0 = 0; c0 < npad; c0 += kKc, g++) {
        if ((g & (kBProducers - 1)) != bw) continue;
        const int kc = min(kKc, npad - c0), s = static_cast<int>(g % kStages);
        int rows[kKc / 32];  // XTS rows of columns c0 + lane + 32 h
#pragma unroll
        for (int h = 0; h < kKc / 32; h++) {
          const int c = c0 + lane + 32 * h;
          rows[h] = a.zero_row;
          if (c < I.ncols) rows[h] = I.kind == 0 ? __ldg(a.colmap + I.map + c) : I.map + c;
        }
        if (!wait_bar_warp(S, &S.empty[s], static_cast<uint32_t>((g / kStages) & 1) ^ 1u, a.status, 22)) {
          stop = true;
          break;
        }
        {  // A: the chunk's hi rows to tile rows 0.., its lo rows to tile rows 64..
          // (read once: evict-first in L2, so the gathered XTS rows stay resident)
          uint64_t pol;
          asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
          const int G = (I.m + 7) >> 3;
          const int units = G * kc;  // 16-byte units of each half
          const unsigned char *src = a.adata + I.a_off + static_cast<int64_t>(c0 / kKc) * 2 * chunk_bytes(G, kKc);
          const uint32_t hi = su32(S.a[s]), lo = hi + 128u * kc;
          for (int u = lane; u < units; u += 32) {
            asm volatile("cp.async.cg.shared.global.L2::cache_hint [%0], [%1], 16, %2;" ::"r"(hi + 16u * u),
                         "l"(src + 16 * u), "l"(pol)
                         : "memory");
            asm volatile("cp.async.cg.shared.global.L2::cache_hint [%0], [%1], 16, %2;" ::"r"(lo + 16u * u),
                         "l"(src + 16 * (units + u)), "l"(pol)
                         : "memory");
          }
        }
        const uint32_t dst0 = su32(S.b[s]) + piece * kBGroupN;
#pragma unroll
        for (int i = 0; i < kKc / 4; i++) {
          const int k = 4 * i + sub;
          const int r = __shfl_sync(0xffffffffu, rows[i >> 3], k & 31);
          if (k < kc) {
            const uint16_t *src = a.xts + static_cast<int64_t>(r) * (2 * kTcRhs) + piece * 8;
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst0 + (k >> 3) * kBGroupK + (k & 7) * 16),
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
  } else if (warp == 2) {
    // ---- MMA issuer: the warp runs the loop, one elected lane issues --------
    // Per 16 columns one UMMA: [A_hi; A_lo] (M = 128) x [B_hi B_lo] (N = 64)
    // into the item's accumulator; the epilogue adds its four quadrants.
    int64_t g = 0;
    int n = 0;
    bool stop = false;
    for (; !stop; n++) {
      const int it = next_item(S, n, a.status);
      if (it < 0) break;
      const TcItem I = a.items[it];
      const int npad = I.ncols > 0 ? (I.ncols + 15) & ~15 : 16;
      const int ab = n & 1;
      if (!wait_bar_warp(S, &S.acc_empty[ab], static_cast<uint32_t>((n >> 1) & 1) ^ 1u, a.status, 23)) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t acc = S.tmem + ab * kBN;
      // two chunks per turn where the item has them: one round of waits,
      // descriptors and hand-offs per 128 columns
      for (int c0 = 0; c0 < npad;) {
        const int two = c0 + kKc < npad ? 2 : 1;
        int s2[2], kc2[2];
        bool ok = true;
        for (int h = 0; h < two; h++) {
          kc2[h] = min(kKc, npad - c0 - h * kKc);
          s2[h] = static_cast<int>((g + h) % kStages);
          ok = ok && wait_bar_warp(S, &S.full[s2[h]], static_cast<uint32_t>(((g + h) / kStages) & 1), a.status, 24);
        }
        if (!ok) {
          stop = true;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (elect_one()) {
          for (int h = 0; h < two; h++) {
            const uint64_t da = sdesc(su32(S.a[s2[h]]), 128, static_cast<uint32_t>(kc2[h]) * 16);
            const uint64_t db = sdesc(su32(S.b[s2[h]]), kBLbo, kBSbo);
            for (int ks = 0; ks < kc2[h] / 16; ks++) {
              // the start address field counts 16-byte units
              const uint64_t oa = static_cast<uint64_t>(ks * 256) >> 4, ob = static_cast<uint64_t>(ks * 2 * kBGroupK) >> 4;
              mma(acc, da + oa, db + ob, ((c0 + h * kKc) | ks) ? 1u : 0u);
            }
            commit(&S.empty[s2[h]]);
          }
        }
        __syncwarp();
        g += two;
        c0 += two * kKc;
      }
      if (stop) break;
      if (elect_one()) commit(&S.acc_full[ab]);
      __syncwarp();
    }
    // the last stage release must land before the CTA's shared memory goes away
    if (!stop && g > 0)
      wait_bar_warp(S, &S.empty[(g - 1) % kStages], static_cast<uint32_t>(((g - 1) / kStages) & 1), a.status, 26);
  } else if (warp >= 4 && warp < 8) {
    // ---- epilogue -----------------------------------------------------------
    // Warp w reads TMEM lanes 32(w-4)..: warps 4, 5 hold the A_hi rows, warps
    // 6, 7 the A_lo rows of the same panel rows. Warps 6, 7 hand their sums
    // to 4, 5 through shared memory; 4, 5 add and write the results.
    const int quarter = warp & 3, row = (quarter & 1) * 32 + lane;
    const bool lo_part = quarter >= 2;
    int n = 0;
    for (;; n++) {
      const int it = next_item(S, n, a.status);
      if (it < 0) break;
      const TcItem I = a.items[it];
      const int ab = n & 1;
      if (!wait_bar_warp(S, &S.acc_full[ab], static_cast<uint32_t>((n >> 1) & 1), a.status, 25)) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      uint32_t r[kTcRhs], r2[kTcRhs];
      const uint32_t taddr = S.tmem + ab * kBN + (static_cast<uint32_t>(quarter * 32) << 16);
      tmem_ld32(taddr, r);
      tmem_ld32(taddr + kTcRhs, r2);
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) arrive(&S.acc_empty[ab]);
      float v[kTcRhs];  // A_part B_hi + A_part B_lo
#pragma unroll
      for (int q = 0; q < kTcRhs; q++) v[q] = __uint_as_float(r[q]) + __uint_as_float(r2[q]);
      if (lo_part) {
        if (!wait_bar_warp(S, &S.epi_free, static_cast<uint32_t>(n & 1) ^ 1u, a.status, 27)) break;
#pragma unroll
        for (int q = 0; q < kTcRhs; q++) S.epi[row][q] = v[q];
        __syncwarp();
        if (lane == 0) arrive(&S.epi_ready);
        continue;
      }
      if (!wait_bar_warp(S, &S.epi_ready, static_cast<uint32_t>(n & 1), a.status, 28)) break;
#pragma unroll
      for (int q = 0; q < kTcRhs; q++) v[q] += S.epi[row][q];
      __syncwarp();
      if (lane == 0) arrive(&S.epi_free);
      if (row >= I.m) continue;
      if (I.kind == 0) {
        float *yr = a.y + a.tmap0[a.tiles[I.out].row0 + I.row0 + row];
#pragma unroll
        for (int q = 0; q < kTcRhs; q++)
          if (q < a.nr) yr[q * a.ldy] = v[q];
      } else if (I.kind == 1) {
        uint4 *dst = reinterpret_cast<uint4 *>(a.xts_out + static_cast<int64_t>(I.out + row) * (2 * kTcRhs));
#pragma unroll
        for (int q = 0; q < 4; q++) {
          uint4 hi, lo;
          split8(v + 8 * q, hi, lo);
          dst[q] = hi;
          dst[4 + q] = lo;
        }
      } else {
        float4 *dst = reinterpret_cast<float4 *>(a.prow + static_cast<int64_t>(I.out + row) * kTcRhs);
#pragma unroll
        for (int q = 0; q < 8; q++) dst[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(S.tmem), "r"(kTmemCols));
}

// XTS x rows from X in its own order: the 32 right-hand sides X[j + r ldx]
// (0 for r >= nr) of source index j, split into BF16 hi (first 64 bytes) and lo
// (last 64 bytes), go to row sinv[j]. Reads of X are coalesced along j and
// every row is written whole; x-region rows that no source index maps to stay
// zero from the allocation. Also re-arms the two item tickets.
__global__ void permute_split_kernel(const float *__restrict__ X, int64_t ldx, int nr,
                                     const int32_t *__restrict__ sinv0, int64_t n_src,
                                     uint16_t *__restrict__ xts, int32_t *__restrict__ tickets) {
  __shared__ float tile[64][kTcRhs + 1];
  if (blockIdx.x == 0 && threadIdx.x < 2) tickets[threadIdx.x] = 0;  // V and near/U item tickets
  for (int64_t j0 = blockIdx.x * 64ll; j0 < n_src; j0 += gridDim.x * 64ll) {
    for (int e = threadIdx.x; e < 64 * kTcRhs; e += blockDim.x) {
      const int r = e / 64, jj = e % 64;  // consecutive threads: consecutive j
      const int64_t j = j0 + jj;
      tile[jj][r] = (j < n_src && r < nr) ? X[j + r * ldx] : 0.0f;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < 64 * 4; e += blockDim.x) {
      const int jj = e >> 2, q = e & 3;
      if (j0 + jj < n_src) {
        float v[8];
#pragma unroll
        for (int i = 0; i < 8; i++) v[i] = tile[jj][8 * q + i];
        uint4 hi, lo;
        split8(v, hi, lo);
        uint4 *dst = reinterpret_cast<uint4 *>(xts + static_cast<int64_t>(sinv0[j0 + jj]) * (2 * kTcRhs));
        dst[q] = hi;
        dst[4 + q] = lo;
      }
    }
    __syncthreads();
  }
}

// t rows from partial rows, pieces summed in order; one warp per row, lane =
// right-hand side.
__global__ void reduce_split_kernel(const MVReduce *__restrict__ red, int32_t nred, const float *__restrict__ P,
                                    uint16_t *__restrict__ xts) {
  const int lane = threadIdx.x & 31;
  for (int32_t e = static_cast<int32_t>(blockIdx.x); e < nred; e += gridDim.x) {
    const MVReduce R = red[e];
    for (int row = threadIdx.x >> 5; row < R.nrows; row += blockDim.x >> 5) {
      float s = 0.0f;
      for (int j = 0; j < R.npieces; j++)
        s += P[(static_cast<int64_t>(R.p_row) + static_cast<int64_t>(j) * R.nrows + row) * kTcRhs + lane];
      const __nv_bfloat16 hb = __float2bfloat16_rn(s);
      const __nv_bfloat16 lb = __float2bfloat16_rn(s - __bfloat162float(hb));
      uint16_t *dst = xts + static_cast<int64_t>(R.t_row + row) * (2 * kTcRhs);
      dst[lane] = *reinterpret_cast<const uint16_t *>(&hb);
      dst[kTcRhs + lane] = *reinterpret_cast<const uint16_t *>(&lb);
    }
  }
}

// Canonical BF16 (hi, lo) chunks of one item from its FP32 row-major source.
__global__ void pack_tc_kernel(const TcPack *__restrict__ jobs, const float *__restrict__ src,
                               unsigned char *__restrict__ adata) {
  const TcPack J = jobs[blockIdx.x];
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
        v[i] = (r < J.m && c < J.ncols) ? src[J.src_off + static_cast<int64_t>(r) * J.ld + c] : 0.0f;
      }
      uint4 hi, lo;
      split8(v, hi, lo);
      const int64_t off = static_cast<int64_t>(r >> 3) * kc * 16 + (k8 >> 3) * 128 + (r & 7) * 16;
      *reinterpret_cast<uint4 *>(base + off) = hi;
      *reinterpret_cast<uint4 *>(base + half + off) = lo;
    }
    base += 2 * half;
  }
}

}  // namespace

size_t tc_smem_bytes() { return sizeof(TcSmem) + 1024; }

static void tc_attrs() {
  static bool done = false;
  if (done) return;
  cudaFuncSetAttribute(tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(tc_smem_bytes()));
  done = true;
}

cudaError_t launch_pack_tc(const TcPack *jobs, int64_t njobs, const float *src, void *adata, cudaStream_t s) {
  for (int64_t j0 = 0; j0 < njobs; j0 += 65535) {
    const int nb = static_cast<int>(njobs - j0 < 65535 ? njobs - j0 : 65535);
    pack_tc_kernel<<<nb, 256, 0, s>>>(jobs + j0, src, static_cast<unsigned char *>(adata));
  }
  return cudaGetLastError();
}

cudaError_t launch_matvec_tc(const DevPlan &p, const DevTc &t, const float *X, int64_t ldx, int nr,
                             float *Y, int64_t ldy, cudaStream_t s, cudaEvent_t *ev, int *launches) {
  tc_attrs();
  int nl = 0;
  int gp = static_cast<int>((p.n_src + 63) / 64);
  if (gp > 2048) gp = 2048;
  if (ev) cudaEventRecord(ev[0], s);
  permute_split_kernel<<<gp, 256, 0, s>>>(X, ldx, nr, p.sinv0, p.n_src, t.xts, p.counter + 2);
  nl++;
  if (ev) cudaEventRecord(ev[1], s);
  TcArgs a{};
  a.adata = static_cast<const unsigned char *>(t.adata);
  a.colmap = t.colmap;
  a.xts = t.xts;
  a.xts_out = t.xts;
  a.prow = t.prow;
  a.tiles = p.tiles;
  a.tmap0 = p.tmap0;
  a.y = Y;
  a.ldy = ldy;
  a.nr = nr;
  a.zero_row = static_cast<int32_t>(p.zero_row);
  a.status = p.status;
  const size_t smem = tc_smem_bytes();
  if (t.n_v > 0) {
    a.items = t.v_items;
    a.nitems = t.n_v;
    a.ticket = p.counter + 2;
    tc_kernel<<<t.ctas, kTcThreads, smem, s>>>(a);
    nl++;
    if (t.n_reduce > 0) {
      reduce_split_kernel<<<t.n_reduce < 4096 ? t.n_reduce : 4096, 256, 0, s>>>(t.reduce, t.n_reduce, t.prow, t.xts);
      nl++;
    }
  }
  if (ev) cudaEventRecord(ev[2], s);
  a.items = t.du_items;
  a.nitems = t.n_du;
  a.ticket = p.counter + 3;
  tc_kernel<<<t.ctas, kTcThreads, smem, s>>>(a);
  nl++;
  if (ev) cudaEventRecord(ev[3], s);
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
