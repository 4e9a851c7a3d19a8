// Mixed-precision multi-right-hand-side product on the 5th-generation tensor
// cores (tcgen05, sm_103a): Y = H X for 32 right-hand sides per pass.
//
// Every panel (<= 128 rows of a row tile, or of a V source group) meets the
// XT rows of its columns as a GEMM D[128 x 32] += A[128 x K] B[32 x K]^T with
// an FP32 accumulator in tensor memory. Operands are split on the fly into
// BF16 pairs, a = a_hi + a_lo with a_hi = bf16(a), a_lo = bf16(a - a_hi)
// (relative residual ~2^-17), and each 16-column step issues three UMMAs:
// A_hi B_hi + A_hi B_lo + A_lo B_hi. Per 64-column chunk the CTA converts A
// and B into canonical K-major no-swizzle layouts in shared memory (core
// matrices of 8 rows x 16 bytes; K-adjacent cores 128 B apart, 8-row groups
// 1024 B apart), double-buffered, while the previous chunk's UMMAs run; one
// thread issues the UMMAs and commits them to an mbarrier per buffer. The
// accumulator is read back with tcgen05.ld (warp w reads TMEM lanes
// 32w..32w+31). All mbarrier waits are bounded and report into `status`.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "hm_device.h"

namespace hm {

namespace {

constexpr int kTcThreads = 128;   // 4 warps: one per 32 TMEM lanes
constexpr int kTcRhs = 32;        // N of the UMMA
constexpr int kKc = 64;           // columns per chunk (4 UMMA K-steps of 16)
constexpr int kABytes = 128 * kKc * 2;   // one BF16 A tile: 16 KB
constexpr int kBBytes = kTcRhs * kKc * 2;  // one BF16 B tile: 4 KB
constexpr uint32_t kSpin = 1u << 24;

__device__ __forceinline__ uint32_t su32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
  uint64_t d = 0;
  d |= static_cast<uint64_t>((saddr >> 4) & 0x3FFF);
  d |= static_cast<uint64_t>(128 >> 4) << 16;   // K-adjacent core matrices
  d |= static_cast<uint64_t>(1024 >> 4) << 32;  // 8-row groups
  d |= static_cast<uint64_t>(1) << 46;          // descriptor version for tcgen05
  return d;                                     // no swizzle, base offset 0
}

// kind::f16 instruction descriptor: BF16 A and B (K-major), FP32 D, M = 128, N = 32.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((kTcRhs >> 3) << 17) | ((128u >> 4) << 24);

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

__device__ __forceinline__ bool wait_parity(uint64_t *bar, uint32_t parity) {
  for (uint32_t i = 0; i < kSpin; i++) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(su32(bar)), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

// Byte offset of element (row, k) in a canonical K-major BF16 tile of 64 columns.
__device__ __forceinline__ int canon(int row, int k) {
  return (row >> 3) * 1024 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2;
}

__device__ __forceinline__ void split(float v, __nv_bfloat16 &hi, __nv_bfloat16 &lo) {
  hi = __float2bfloat16_rn(v);
  lo = __float2bfloat16_rn(v - __bfloat162float(hi));
}

struct TcSmem {
  unsigned char a_hi[2][kABytes], a_lo[2][kABytes];
  unsigned char b_hi[2][kBBytes], b_lo[2][kBBytes];
  float xrow[kKc][kTcRhs];  // the chunk's XT rows (FP32) before splitting
  uint64_t bar[2];
  uint32_t tmem;
  int32_t ticket[2];
  int32_t abort;  // a bounded wait ran out: stop taking work
  int32_t cmap[kKc];
};

}  // namespace

// One panel: rows [0, m) (m <= 128) of a row-major FP32 matrix A (stride lda,
// rows zero-padded to a multiple of 4 columns), K = ncols_pad columns, times the
// XT rows named by `col_row(c)` (-1 = zero row). Calls emit(row, q, value).
template <typename ColRow, typename Emit>
__device__ __forceinline__ void tc_panel(TcSmem &S, uint32_t (&phase)[2], uint32_t (&pending)[2],
                                         const float *A, int64_t lda, int m, int ncols_pad,
                                         const float *xt, ColRow col_row, Emit emit,
                                         int32_t *status) {
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  int buf = 0;
  bool first = true;
  for (int c0 = 0; c0 < ncols_pad; c0 += kKc) {
    const int cn = min(kKc, ncols_pad - c0);  // a multiple of 4
    // the UMMAs that last read this buffer must be done before it is rewritten
    if (pending[buf]) {
      if (tid == 0 && !wait_parity(&S.bar[buf], phase[buf])) {
        atomicCAS(status, 0, 11);
        S.abort = 1;
      }
      __syncthreads();
      phase[buf] ^= 1;
      pending[buf] = 0;
      if (S.abort) return;  // uniform: read after the barrier
    }
    // XT rows of the chunk's columns
    for (int j = tid; j < kKc; j += kTcThreads) S.cmap[j] = j < cn ? col_row(c0 + j) : -1;
    __syncthreads();
    for (int e = tid; e < kKc * (kTcRhs / 4); e += kTcThreads) {
      const int j = e / (kTcRhs / 4), q = (e % (kTcRhs / 4)) * 4;
      const int r = S.cmap[j];
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (r >= 0) v = *reinterpret_cast<const float4 *>(xt + static_cast<int64_t>(r) * kTcRhs + q);
      *reinterpret_cast<float4 *>(&S.xrow[j][q]) = v;
    }
    // A: rows split into hi/lo, canonical layout; two rows per warp per step,
    // 16 lanes x 4 columns per row
    // (all 16 loads of a thread are issued before the first is used)
    {
      const int half = lane >> 4, c4 = (lane & 15) * 4, row0 = warp * 2 + half;
      float4 v[16];
#pragma unroll
      for (int i = 0; i < 16; i++) {
        const int row = row0 + 8 * i;
        v[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (row < m && c4 < cn) v[i] = __ldcs(reinterpret_cast<const float4 *>(A + static_cast<int64_t>(row) * lda + c0 + c4));
      }
#pragma unroll
      for (int i = 0; i < 16; i++) {
        __nv_bfloat16 h[4], l[4];
        split(v[i].x, h[0], l[0]);
        split(v[i].y, h[1], l[1]);
        split(v[i].z, h[2], l[2]);
        split(v[i].w, h[3], l[3]);
        const int off = canon(row0 + 8 * i, c4);
        *reinterpret_cast<uint2 *>(S.a_hi[buf] + off) = *reinterpret_cast<uint2 *>(h);
        *reinterpret_cast<uint2 *>(S.a_lo[buf] + off) = *reinterpret_cast<uint2 *>(l);
      }
    }
    __syncthreads();
    // B: for right-hand side n and 8 consecutive columns k, one 16-byte store
    for (int e = tid; e < kTcRhs * (kKc / 8); e += kTcThreads) {
      const int n = e % kTcRhs, k8 = (e / kTcRhs) * 8;
      __nv_bfloat16 h[8], l[8];
#pragma unroll
      for (int q = 0; q < 8; q++) split(S.xrow[k8 + q][n], h[q], l[q]);
      const int off = canon(n, k8);
      *reinterpret_cast<uint4 *>(S.b_hi[buf] + off) = *reinterpret_cast<uint4 *>(h);
      *reinterpret_cast<uint4 *>(S.b_lo[buf] + off) = *reinterpret_cast<uint4 *>(l);
    }
    // generic-proxy writes -> visible to the tensor cores' async proxy
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (tid == 0) {
      const uint32_t ah = su32(S.a_hi[buf]), al = su32(S.a_lo[buf]);
      const uint32_t bh = su32(S.b_hi[buf]), bl = su32(S.b_lo[buf]);
      bool overwrite = first;
      for (int ks = 0; ks < cn / 16 + (cn % 16 ? 1 : 0); ks++) {
        const uint32_t step = ks * 256;  // 16 columns = two K-adjacent core matrices
        mma(S.tmem, sdesc(ah + step), sdesc(bh + step), overwrite ? 0u : 1u);
        overwrite = false;
        mma(S.tmem, sdesc(ah + step), sdesc(bl + step), 1u);
        mma(S.tmem, sdesc(al + step), sdesc(bh + step), 1u);
      }
      commit(&S.bar[buf]);
    }
    first = false;  // uniform across the CTA: the accumulator now holds this panel's sums
    pending[buf] = 1;
    buf ^= 1;
  }
  // wait for the last UMMAs, then read the accumulator
  for (int b = 0; b < 2; b++)
    if (pending[b]) {
      if (tid == 0 && !wait_parity(&S.bar[b], phase[b])) {
        atomicCAS(status, 0, 12);
        S.abort = 1;
      }
      __syncthreads();
      phase[b] ^= 1;
      pending[b] = 0;
    }
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  uint32_t r[kTcRhs];
  const uint32_t taddr = S.tmem + (static_cast<uint32_t>(warp * 32) << 16);
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]),
        "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]),
        "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
  const int row = warp * 32 + lane;
  if (first == false && row < m)
#pragma unroll
    for (int q = 0; q < kTcRhs; q++) emit(row, q, __uint_as_float(r[q]));
  if (first && row < m)  // no columns: the panel contributes zeros
#pragma unroll
    for (int q = 0; q < kTcRhs; q++) emit(row, q, 0.0f);
  // the next panel's first UMMA overwrites the accumulator
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
}

__device__ __forceinline__ void tc_setup(TcSmem &S) {
  if (threadIdx.x == 0) {
    S.abort = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&S.bar[0])));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&S.bar[1])));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if ((threadIdx.x >> 5) == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 32;" ::"r"(su32(&S.tmem)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tc_teardown(TcSmem &S) {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if ((threadIdx.x >> 5) == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 32;" ::"r"(S.tmem));
}

// V pass: t rows of every V unit (source-group rows), 128 at a time.
__global__ void __launch_bounds__(kTcThreads) v_tc_kernel(const float *__restrict__ V,
                                                          const VUnit *__restrict__ units,
                                                          int32_t nunits, float *__restrict__ xt,
                                                          int32_t *counter, int32_t *status) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  TcSmem &S = *reinterpret_cast<TcSmem *>(smem_raw);
  tc_setup(S);
  uint32_t phase[2] = {0, 0}, pending[2] = {0, 0};
  for (int it = 0;; it++) {
    if (threadIdx.x == 0) S.ticket[it & 1] = atomicAdd(counter, 1);
    __syncthreads();
    const int u = S.ticket[it & 1];
    if (u >= nunits) break;
    const VUnit U = units[u];
    for (int k0 = 0; k0 < U.nrows; k0 += 128) {
      const int rows = min(128, U.nrows - k0);
      tc_panel(
          S, phase, pending, V + U.v_off + static_cast<int64_t>(k0) * U.stride, U.stride, rows,
          U.stride, xt, [&](int c) { return U.x_off + c; },
          [&](int row, int q, float v) { xt[static_cast<int64_t>(U.t_off + k0 + row) * kTcRhs + q] = v; },
          status);
      if (S.abort) break;
    }
    if (S.abort) break;
  }
  tc_teardown(S);
}

// Near/U pass: one whole row tile per panel.
struct DuTcArgs {
  const float *panels;
  const TileDesc *tiles;
  const int32_t *order;
  int32_t ntiles;
  const Seg *segs;
  const float *xt;
  const int32_t *tmap0;
  float *y;
  int64_t ldy;
  int nr;
  int32_t *counter;
  int32_t *status;
};

__global__ void __launch_bounds__(kTcThreads) du_tc_kernel(DuTcArgs a) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  TcSmem &S = *reinterpret_cast<TcSmem *>(smem_raw);
  tc_setup(S);
  uint32_t phase[2] = {0, 0}, pending[2] = {0, 0};
  for (int it = 0;; it++) {
    if (threadIdx.x == 0) S.ticket[it & 1] = atomicAdd(a.counter, 1);
    __syncthreads();
    const int u = S.ticket[it & 1];
    if (u >= a.ntiles) break;
    const TileDesc d = a.tiles[a.order[u]];
    const Seg *sg = a.segs + d.seg0;
    tc_panel(
        S, phase, pending, a.panels + d.data_off, d.ld, d.m, d.ld, a.xt,
        [&](int c) {
          if (c >= d.ncols) return -1;
          int lo = 0, hi = d.nseg - 1;
          while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (sg[mid].col0 <= c)
              lo = mid;
            else
              hi = mid - 1;
          }
          return sg[lo].vec_off + (c - sg[lo].col0);
        },
        [&](int row, int q, float v) {
          if (q < a.nr) a.y[a.tmap0[d.row0 + row] + q * a.ldy] = v;
        },
        a.status);
    if (S.abort) break;
  }
  tc_teardown(S);
}

size_t tc_smem_bytes() { return sizeof(TcSmem) + 1024; }

static void tc_attrs() {
  static bool done = false;
  if (done) return;
  cudaFuncSetAttribute(v_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(tc_smem_bytes()));
  cudaFuncSetAttribute(du_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(tc_smem_bytes()));
  done = true;
}

int occupancy_tc() {
  tc_attrs();
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, du_tc_kernel, kTcThreads, tc_smem_bytes());
  return n > 0 ? n : 1;
}

// The V pass of this form takes its units from the ticket counter, so the
// permutation re-arms it and the near/U pass uses the second counter slot.
cudaError_t launch_matvec_tc(const DevPlan &p, const float *panels, const float *vdata, float *xt,
                             int grid, cudaStream_t s, float *Y, int64_t ldy, int nr,
                             cudaEvent_t ev_mid) {
  tc_attrs();
  const size_t smem = tc_smem_bytes();
  if (!p.warp_begin_empty)
    v_tc_kernel<<<grid, kTcThreads, smem, s>>>(vdata, p.vunits, p.nvunits, xt, p.counter, p.status);
  if (ev_mid) cudaEventRecord(ev_mid, s);
  DuTcArgs a{panels, p.tiles, p.tile_order, p.ntiles, p.segs, xt, p.tmap0, Y, ldy, nr,
             p.counter + 1, p.status};
  du_tc_kernel<<<grid, kTcThreads, smem, s>>>(a);
  return cudaGetLastError();
}

}  // namespace hm
