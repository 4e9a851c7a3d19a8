// Near/U pass with a bulk-copy pipeline (sm_103a): y = D x + U t.
//
// Same work units, thread mapping and fixed summation order as du_pass_kernel
// (hm_matvec.cu), but the panel bytes reach shared memory through
// cp.async.bulk copies completed on mbarriers instead of per-thread loads:
//   * warp 0 (one elected lane) takes units from the ticket counter and keeps
//     a ring of kStages 16 KB stages filled, each stage tagged with its unit
//     and first 16-byte vector;
//   * warps 1..8 wait for a full stage, consume it from shared memory with the
//     fixed-row accumulation and release it to the producer.
// Copies of the next unit are in flight while the consumers gather the unit's
// vector entries and reduce the previous unit, so HBM stays busy across unit
// boundaries. Every wait is bounded: on expiry the kernel records an error
// code in `status`, stops taking work, drains the copies it issued and returns.
#include <cuda_runtime.h>

#include "hm_device.h"

namespace hm {

namespace {

constexpr int kStages = 5;
constexpr int kStageBytes = 16384;
constexpr int kConsumers = 256;             // 8 consumer warps
constexpr int kTmaThreads = kConsumers + 32;
constexpr int kMaxSegs = 256;
constexpr uint32_t kSpinLimit = 1u << 24;   // bounded mbarrier polls (seconds)
constexpr int kEnd = -1, kAbort = -2;

__device__ __forceinline__ uint32_t su32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t *b, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_tx(uint64_t *b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(b)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(su32(b)) : "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t *b, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(su32(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait for the completion of the phase with the given parity.
__device__ __forceinline__ bool mbar_wait(uint64_t *b, uint32_t parity) {
  for (uint32_t i = 0; i < kSpinLimit; i++)
    if (mbar_test(b, parity)) return true;
  return false;
}
__device__ __forceinline__ void bulk_copy(void *dst, const void *src, uint32_t bytes, uint64_t *b) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          su32(dst)),
      "l"(src), "r"(bytes), "r"(su32(b))
      : "memory");
}
__device__ __forceinline__ void consumer_sync() {
  asm volatile("bar.sync 1, %0;" ::"n"(kConsumers) : "memory");
}

template <typename T>
struct V16t;
template <>
struct V16t<float> {
  using type = float4;
  static constexpr int N = 4;
};
template <>
struct V16t<double> {
  using type = double2;
  static constexpr int N = 2;
};

__device__ __forceinline__ float fmaT(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fmaT(double a, double b, double c) { return __fma_rn(a, b, c); }

template <typename T>
__device__ __forceinline__ void dot2(T &s, T &c, T a, T b) {
  T p = a * b, pe = fmaT(a, b, -p), t = s + p, z = t - s;
  c += ((s - (t - z)) + (p - z)) + pe;
  s = t;
}

struct StageMeta {
  int32_t unit;   // unit index, kEnd or kAbort
  int32_t nvec;   // 16-byte vectors in the stage
  int64_t f0;     // first vector, counted from the tile panel's start
};

}  // namespace

template <typename T>
struct DuTmaArgs {
  const T *panels;
  const TileDesc *tiles;
  const DuUnit *units;
  int32_t nunits;
  const Seg *segs;
  const T *xt;
  const int32_t *tmap0;
  T *y;
  int32_t *counter;
  T *part;
  int32_t *tile_cnt;
  int32_t *status;  // 0, or the code of the first bounded wait that expired
};

template <typename T, bool COMP>
__global__ void __launch_bounds__(kTmaThreads, 2) du_tma_kernel(DuTmaArgs<T> a) {
  using VT = typename V16t<T>::type;
  constexpr int VEC = V16t<T>::N;
  constexpr int kVecPerStage = kStageBytes / 16;
  constexpr int kCols = 16384 / sizeof(T);
  extern __shared__ __align__(128) unsigned char smem_raw[];
  T *ring = reinterpret_cast<T *>(smem_raw);  // kStages * kStageBytes
  __shared__ __align__(8) uint64_t full[kStages], empty[kStages];
  __shared__ StageMeta meta[kStages];
  __shared__ T vals[kCols];
  __shared__ Seg ssegs[kMaxSegs];
  __shared__ T part[kConsumers * VEC];
  __shared__ T partc[COMP ? kConsumers * VEC : 1];
  __shared__ int32_t s_last;
  __shared__ StageMeta s_meta[2];  // by iteration parity: written while the other is read

  const int tid = threadIdx.x;
  if (tid == 0) {
    for (int s = 0; s < kStages; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], kConsumers / 32);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();

  if (tid < 32) {
    // ------------------------------ producer ------------------------------
    if (tid != 0) return;
    int stage = 0;
    uint32_t uses[kStages] = {0, 0, 0, 0, 0};
    bool ok = true;
    auto acquire = [&](int s) -> bool {  // wait until consumers released stage s
      if (uses[s] == 0) return true;
      return mbar_wait(&empty[s], (uses[s] - 1) & 1);
    };
    for (;;) {
      const int u = atomicAdd(a.counter, 1);
      if (u >= a.nunits) break;
      const DuUnit U = a.units[u];
      const TileDesc d = a.tiles[U.tile];
      const int64_t v_lo = (static_cast<int64_t>(U.c0) * d.m) / VEC;
      const int64_t v_hi = (static_cast<int64_t>(U.c1) * d.m + VEC - 1) / VEC;
      const char *base = reinterpret_cast<const char *>(a.panels + d.data_off);
      for (int64_t v = v_lo; v < v_hi || v == v_lo; v += kVecPerStage) {
        const int nv = static_cast<int>(v_hi - v < kVecPerStage ? v_hi - v : kVecPerStage);
        if (!acquire(stage)) {
          ok = false;
          break;
        }
        meta[stage].unit = u;
        meta[stage].nvec = nv;
        meta[stage].f0 = v;
        if (nv > 0) {
          mbar_arrive_tx(&full[stage], static_cast<uint32_t>(nv) * 16u);
          bulk_copy(ring + static_cast<size_t>(stage) * (kStageBytes / sizeof(T)), base + v * 16,
                    static_cast<uint32_t>(nv) * 16u, &full[stage]);
        } else {
          mbar_arrive(&full[stage]);  // an empty unit still passes through the ring
        }
        uses[stage]++;
        stage = (stage + 1) % kStages;
        if (nv <= 0) break;
      }
      if (!ok) break;
    }
    if (ok && acquire(stage)) {
      meta[stage].unit = kEnd;
      meta[stage].nvec = 0;
      mbar_arrive(&full[stage]);
      uses[stage]++;
    } else {
      atomicCAS(a.status, 0, 1);
    }
    // drain: every copy this thread issued must land before the CTA exits
    for (int s = 0; s < kStages; s++)
      if (uses[s] > 0 && !mbar_wait(&full[s], (uses[s] - 1) & 1)) atomicCAS(a.status, 0, 2);
    return;
  }

  // ------------------------------- consumers -------------------------------
  const int ct = tid - 32, lane = tid & 31;
  int stage = 0;
  uint32_t phase[kStages] = {0, 0, 0, 0, 0};
  int cur = -1;
  DuUnit U{};
  TileDesc d{};
  int m = 1, G = 1, g = 0, t = 0;
  bool active = false;
  int base[VEC];
  T acc[VEC], cmp[VEC];

  auto finish = [&]() {  // reduce the current unit and write y or its partial rows
    if (active)
#pragma unroll
      for (int uu = 0; uu < VEC; uu++) {
        part[g * VEC * m + VEC * t + uu] = acc[uu];
        if (COMP) partc[g * VEC * m + VEC * t + uu] = cmp[uu];
      }
    consumer_sync();
    T s = T(0), c = T(0);
    if (ct < m) {
      for (int gg = 0; gg < G; gg++)
#pragma unroll
        for (int k = 0; k < VEC; k++) {
          const int idx = gg * VEC * m + ct + k * m;
          if (COMP) {
            const T p = part[idx], tt = s + p, z = tt - s;
            c += ((s - (tt - z)) + (p - z)) + partc[idx];
            s = tt;
          } else {
            s += part[idx];
          }
        }
    }
    if (U.nslots == 1) {
      if (ct < m) a.y[a.tmap0[d.row0 + ct]] = COMP ? s + c : s;
      return;
    }
    const int64_t pb = U.part_off + static_cast<int64_t>(U.slot) * m + ct;
    if (ct < m) {
      if (COMP) {
        a.part[2 * pb] = s;
        a.part[2 * pb + 1] = c;
      } else {
        a.part[pb] = s;
      }
    }
    __threadfence();
    consumer_sync();
    if (ct == 0) s_last = atomicAdd(&a.tile_cnt[U.tile], 1) == U.nslots - 1;
    consumer_sync();
    if (s_last) {
      __threadfence();
      if (ct < m) {
        T ts = T(0), tc = T(0);
        for (int sl = 0; sl < U.nslots; sl++) {
          const int64_t idx = U.part_off + static_cast<int64_t>(sl) * m + ct;
          if (COMP) {
            const T p = __ldcg(a.part + 2 * idx), tt = ts + p, z = tt - ts;
            tc += ((ts - (tt - z)) + (p - z)) + __ldcg(a.part + 2 * idx + 1);
            ts = tt;
          } else {
            ts += __ldcg(a.part + idx);
          }
        }
        a.y[a.tmap0[d.row0 + ct]] = COMP ? ts + tc : ts;
      }
      if (ct == 0) a.tile_cnt[U.tile] = 0;
    }
  };

  for (uint32_t iter = 0;; iter++) {
    // one thread waits for the stage; the decision is shared through a barrier
    if (ct == 0) {
      if (mbar_wait(&full[stage], phase[stage])) {
        s_meta[iter & 1] = meta[stage];
      } else {
        s_meta[iter & 1].unit = kAbort;
        atomicCAS(a.status, 0, 3);
      }
    }
    consumer_sync();
    const StageMeta sm = s_meta[iter & 1];
    if (sm.unit < 0) {  // end of work (or an expired wait)
      if (cur >= 0) finish();
      break;
    }
    if (sm.unit != cur) {
      if (cur >= 0) finish();
      consumer_sync();  // vals, ssegs and part are free again
      cur = sm.unit;
      U = a.units[cur];
      d = a.tiles[U.tile];
      m = d.m;
      for (int s = ct; s < U.nseg; s += kConsumers) ssegs[s] = a.segs[U.seg0 + s];
      consumer_sync();
      for (int c = U.c0 + ct; c < U.c1; c += kConsumers) {
        int lo = 0, hi = U.nseg - 1;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (ssegs[mid].col0 <= c)
            lo = mid;
          else
            hi = mid - 1;
        }
        vals[c - U.c0] = a.xt[ssegs[lo].vec_off + (c - ssegs[lo].col0)];
      }
      consumer_sync();
      G = kConsumers / m;
      if (G > 16) G = 16;
      g = ct / m;
      t = ct - g * m;
      active = g < G;
#pragma unroll
      for (int uu = 0; uu < VEC; uu++) {
        base[uu] = (VEC * t + uu) / m;
        acc[uu] = cmp[uu] = T(0);
      }
    }
    if (active && sm.nvec > 0) {
      const VT *S = reinterpret_cast<const VT *>(ring + static_cast<size_t>(stage) * (kStageBytes / sizeof(T)));
      const int64_t f_lo = sm.f0, f_hi = sm.f0 + sm.nvec;
      int64_t q = f_lo > t ? (f_lo - t + m - 1) / m : 0;
      q += ((g - static_cast<int>(q % G)) % G + G) % G;
      const int c0 = U.c0, c1 = U.c1;
      for (int64_t f = t + m * q; f < f_hi; f += static_cast<int64_t>(m) * G, q += G) {
        const VT v = S[f - f_lo];
        const T *e = reinterpret_cast<const T *>(&v);
#pragma unroll
        for (int uu = 0; uu < VEC; uu++) {
          const int c = base[uu] + static_cast<int>(VEC * q);
          if (c >= c0 && c < c1) {
            if (COMP)
              dot2(acc[uu], cmp[uu], e[uu], vals[c - c0]);
            else
              acc[uu] = fmaT(e[uu], vals[c - c0], acc[uu]);
          }
        }
      }
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[stage]);
    phase[stage] ^= 1;
    stage = (stage + 1) % kStages;
  }
}

size_t du_tma_smem_bytes() { return static_cast<size_t>(kStages) * kStageBytes; }

template <typename T, bool COMP>
static int occ_tma() {
  const size_t dyn = du_tma_smem_bytes();
  cudaFuncSetAttribute(du_tma_kernel<T, COMP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       static_cast<int>(dyn));
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, du_tma_kernel<T, COMP>, kTmaThreads, dyn);
  return n > 0 ? n : 1;
}

int occupancy_du_tma(bool f64, bool comp) {
  if (f64) return occ_tma<double, false>();
  return comp ? occ_tma<float, true>() : occ_tma<float, false>();
}

template <typename T, bool COMP>
static cudaError_t run_tma(const DevPlan &p, const T *panels, T *xt, T *y, int grid,
                           cudaStream_t s) {
  DuTmaArgs<T> a{panels, p.tiles, p.units, p.nunits, p.segs, xt, p.tmap0, y,
                 p.counter, static_cast<T *>(p.part), p.tile_cnt, p.status};
  du_tma_kernel<T, COMP><<<grid, kTmaThreads, du_tma_smem_bytes(), s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_du_tma(bool f64, bool comp, const DevPlan &p, const void *panels, void *xt,
                          void *y, int grid, cudaStream_t s) {
  if (f64)
    return run_tma<double, false>(p, static_cast<const double *>(panels), static_cast<double *>(xt),
                                  static_cast<double *>(y), grid, s);
  if (comp)
    return run_tma<float, true>(p, static_cast<const float *>(panels), static_cast<float *>(xt),
                                static_cast<float *>(y), grid, s);
  return run_tma<float, false>(p, static_cast<const float *>(panels), static_cast<float *>(xt),
                               static_cast<float *>(y), grid, s);
}

}  // namespace hm
