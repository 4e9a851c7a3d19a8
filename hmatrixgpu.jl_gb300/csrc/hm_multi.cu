// Multi-right-hand-side H-matrix product, plain form (FP32 or FP64 on the CUDA
// cores): Y = H X for up to kRhs right-hand sides per pass.
//
// XT holds, for every permuted source index and every rank row, the kRhs values
// of that row contiguously (row-major, 128 bytes per row in FP32), so one
// matrix element meets all right-hand sides in one 16-byte-vector gather. The
// matrix is read once per pass; every element feeds kRhs FMAs, which makes this
// form bound by the CUDA cores' FMA rate rather than by HBM.
//
// Threads own one output row and 8 right-hand sides each; the columns of a
// unit are split over K slices whose partial sums meet in shared memory in a
// fixed order, so results are deterministic.
#include <cuda_runtime.h>

#include "hm_device.h"

namespace hm {

constexpr int kRhs = 32;    // right-hand sides per pass (row length of XT)
constexpr int kRg = 8;      // right-hand sides per thread
template <typename T>
struct Cc {
  static constexpr int value = 512 / sizeof(T);  // columns of XT rows staged at once
};

template <typename T>
struct V8;
template <>
struct V8<float> {
  static __device__ __forceinline__ void load(const float *p, float (&v)[8]) {
    const float4 a = *reinterpret_cast<const float4 *>(p), b = *reinterpret_cast<const float4 *>(p + 4);
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
  }
};
template <>
struct V8<double> {
  static __device__ __forceinline__ void load(const double *p, double (&v)[8]) {
#pragma unroll
    for (int q = 0; q < 8; q += 2) {
      const double2 a = *reinterpret_cast<const double2 *>(p + q);
      v[q] = a.x;
      v[q + 1] = a.y;
    }
  }
};

template <typename T>
__device__ __forceinline__ T ldg_s(const T *p) {
  return __ldcs(p);  // streamed matrix data: evict-first
}

// XT rows: XT[c * kRhs + r] = X[smap[c] + r * ldx] for c < n and r < nr, else 0.
template <typename T>
__global__ void permute_multi_kernel(const T *__restrict__ X, int64_t ldx, int nr,
                                     const int32_t *__restrict__ smap0, int64_t n, int64_t x_len,
                                     T *__restrict__ xt, int32_t *__restrict__ counter) {
  __shared__ T tile[64][kRhs + 1];
  if (blockIdx.x == 0 && threadIdx.x == 0) *counter = 0;
  for (int64_t c0 = blockIdx.x * 64ll; c0 < x_len; c0 += gridDim.x * 64ll) {
    for (int e = threadIdx.x; e < 64 * kRhs; e += blockDim.x) {
      const int r = e / 64, cc = e % 64;  // consecutive threads: consecutive c
      const int64_t c = c0 + cc;
      tile[cc][r] = (c < n && r < nr) ? X[smap0[c] + r * ldx] : T(0);
    }
    __syncthreads();
    for (int e = threadIdx.x; e < 64 * kRhs; e += blockDim.x) {
      const int cc = e / kRhs, r = e % kRhs;
      if (c0 + cc < x_len) xt[(c0 + cc) * kRhs + r] = tile[cc][r];
    }
    __syncthreads();
  }
}

// Shared K-split accumulation of one unit: rows x 32 outputs; thread (row
// slot i, group rg, slice ks) keeps 8 accumulators (2 rows when rows > 64).
template <typename T>
struct MultiAcc {
  T acc[2][kRg];
};

// V pass: t[(t_off + k) * kRhs + r] = sum_j V[k, j] XT[(x_off + j) * kRhs + r].
// CTA b works through units [warp_begin[8b], warp_begin[8b + 8]), the same
// byte-balanced split as the single-right-hand-side pass.
template <typename T>
__global__ void __launch_bounds__(kThreads) v_multi_kernel(const T *__restrict__ V,
                                                           const VUnit *__restrict__ units,
                                                           const int32_t *__restrict__ warp_begin,
                                                           int nwarps, T *__restrict__ xt) {
  __shared__ T red[kThreads * kRg];
  const int tid = threadIdx.x;
  const int w0 = blockIdx.x * (kThreads / 32);
  if (w0 >= nwarps) return;
  const int u0 = warp_begin[w0], u1 = warp_begin[min(w0 + kThreads / 32, nwarps)];
  for (int u = u0; u < u1; u++) {
    const VUnit U = units[u];
    for (int k0 = 0; k0 < U.nrows; k0 += 64) {
      const int rows = min(64, U.nrows - k0);
      int S = kThreads / (rows * (kRhs / kRg));
      if (S < 1) S = 1;
      const int per_slice = rows * (kRhs / kRg);
      const int ks = tid / per_slice, rem = tid - ks * per_slice;
      const int k = rem % rows, rg = rem / rows;
      T acc[kRg];
#pragma unroll
      for (int q = 0; q < kRg; q++) acc[q] = T(0);
      if (ks < S) {
        const T *row = V + U.v_off + static_cast<int64_t>(k0 + k) * U.stride;
        const T *xb = xt + static_cast<int64_t>(U.x_off) * kRhs + rg * kRg;
        for (int j = ks; j < U.stride; j += S) {
          const T a = ldg_s(row + j);
          T b[kRg];
          V8<T>::load(xb + static_cast<int64_t>(j) * kRhs, b);
#pragma unroll
          for (int q = 0; q < kRg; q++) acc[q] = fma(a, b[q], acc[q]);
        }
      }
      __syncthreads();
      if (ks < S)
#pragma unroll
        for (int q = 0; q < kRg; q++) red[(ks * per_slice + rem) * kRg + q] = acc[q];
      __syncthreads();
      for (int o = tid; o < rows * kRhs; o += kThreads) {
        const int kk = o / kRhs, r = o % kRhs, g = r / kRg, q = r % kRg;
        T s = T(0);
        for (int sl = 0; sl < S; sl++) s += red[(sl * per_slice + g * rows + kk) * kRg + q];
        xt[static_cast<int64_t>(U.t_off + k0 + kk) * kRhs + r] = s;
      }
    }
  }
}

// Near/U pass over the same units as the single-right-hand-side pass.
template <typename T>
struct DuMultiArgs {
  const T *panels;
  const TileDesc *tiles;
  const DuUnit *units;
  int32_t nunits;
  const Seg *segs;
  const T *xt;
  const int32_t *tmap0;
  T *y;
  int64_t ldy;
  int nr;
  int32_t *counter;
  T *part;            // split tiles: nslots * m * kRhs partial values per tile
  int32_t *tile_cnt;
};

template <typename T>
__global__ void __launch_bounds__(kThreads) du_multi_kernel(DuMultiArgs<T> a) {
  constexpr int kCc = Cc<T>::value;
  __shared__ T xv[kCc * kRhs];
  __shared__ int32_t cmap[kCc];
  __shared__ Seg ssegs[512];
  __shared__ T red[kThreads * kRg];
  __shared__ int32_t s_ticket, s_last;
  const int tid = threadIdx.x;
  for (;;) {
    if (tid == 0) s_ticket = atomicAdd(a.counter, 1);
    __syncthreads();
    const int32_t ticket = s_ticket;
    if (ticket >= a.nunits) break;
    const DuUnit U = a.units[ticket];
    const TileDesc d = a.tiles[U.tile];
    const int m = d.m;
    for (int s = tid; s < U.nseg; s += kThreads) ssegs[s] = a.segs[U.seg0 + s];
    // thread roles: row slot i (rows i and i + 64 when m > 64), group rg, slice ks
    const int rslots = m > 64 ? 64 : m;
    const int per_slice = rslots * (kRhs / kRg);
    int S = kThreads / per_slice;
    if (S < 1) S = 1;
    const int ks = tid / per_slice, rem = tid - ks * per_slice;
    const int i = rem % rslots, rg = rem / rslots;
    const bool active = ks < S;
    const bool two = m > 64 && i + 64 < m;
    T acc0[kRg], acc1[kRg];
#pragma unroll
    for (int q = 0; q < kRg; q++) acc0[q] = acc1[q] = T(0);
    const T *P = a.panels + d.data_off;
    for (int cb = U.c0; cb < U.c1; cb += kCc) {
      const int ce = min(U.c1, cb + kCc);
      __syncthreads();
      for (int c = cb + tid; c < ce; c += kThreads) {
        int lo = 0, hi = U.nseg - 1;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (ssegs[mid].col0 <= c)
            lo = mid;
          else
            hi = mid - 1;
        }
        cmap[c - cb] = ssegs[lo].vec_off + (c - ssegs[lo].col0);
      }
      __syncthreads();
      for (int e = tid; e < (ce - cb) * kRhs; e += kThreads)
        xv[e] = a.xt[static_cast<int64_t>(cmap[e / kRhs]) * kRhs + (e % kRhs)];
      __syncthreads();
      if (active) {
        for (int c = cb + ks; c < ce; c += S) {
          T b[kRg];
          V8<T>::load(xv + (c - cb) * kRhs + rg * kRg, b);
          const T a0 = ldg_s(P + static_cast<int64_t>(c) * m + i);
#pragma unroll
          for (int q = 0; q < kRg; q++) acc0[q] = fma(a0, b[q], acc0[q]);
          if (two) {
            const T a1 = ldg_s(P + static_cast<int64_t>(c) * m + i + 64);
#pragma unroll
            for (int q = 0; q < kRg; q++) acc1[q] = fma(a1, b[q], acc1[q]);
          }
        }
      }
    }
    // reduce the K slices (fixed order), one row pass per row half
    for (int half = 0; half < (m > 64 ? 2 : 1); half++) {
      const int rows = half == 0 ? rslots : m - 64;
      __syncthreads();
      if (active && (half == 0 || two))
#pragma unroll
        for (int q = 0; q < kRg; q++) red[(ks * per_slice + rem) * kRg + q] = half ? acc1[q] : acc0[q];
      __syncthreads();
      for (int o = tid; o < rows * kRhs; o += kThreads) {
        const int ii = o / kRhs, r = o % kRhs, g = r / kRg, q = r % kRg;
        T s = T(0);
        for (int sl = 0; sl < S; sl++) s += red[(sl * per_slice + g * rslots + ii) * kRg + q];
        const int row = half * 64 + ii;
        if (U.nslots == 1) {
          if (r < a.nr) a.y[a.tmap0[d.row0 + row] + r * a.ldy] = s;
        } else {
          a.part[(U.part_off + static_cast<int64_t>(U.slot) * m + row) * kRhs + r] = s;
        }
      }
    }
    if (U.nslots == 1) continue;
    __threadfence();
    __syncthreads();
    if (tid == 0) s_last = atomicAdd(&a.tile_cnt[U.tile], 1) == U.nslots - 1;
    __syncthreads();
    if (s_last) {
      __threadfence();
      for (int o = tid; o < m * kRhs; o += kThreads) {
        const int row = o / kRhs, r = o % kRhs;
        T s = T(0);
        for (int sl = 0; sl < U.nslots; sl++)
          s += __ldcg(a.part + (U.part_off + static_cast<int64_t>(sl) * m + row) * kRhs + r);
        if (r < a.nr) a.y[a.tmap0[d.row0 + row] + r * a.ldy] = s;
      }
      if (tid == 0) a.tile_cnt[U.tile] = 0;
    }
  }
}

template <typename T>
static cudaError_t run_multi(const DevPlan &p, const T *panels, const T *vdata, T *xt, T *part,
                             const T *X, int64_t ldx, int nr, T *Y, int64_t ldy, int grid_v,
                             int grid_du, cudaStream_t s, cudaEvent_t *ev, int *launches) {
  int gp = static_cast<int>((p.x_len + 63) / 64);
  if (gp > 2048) gp = 2048;
  int nl = 0;
  if (ev) cudaEventRecord(ev[0], s);
  permute_multi_kernel<T><<<gp, kThreads, 0, s>>>(X, ldx, nr, p.smap0, p.n, p.x_len, xt, p.counter);
  nl++;
  if (ev) cudaEventRecord(ev[1], s);
  if (!p.warp_begin_empty) {
    v_multi_kernel<T><<<grid_v, kThreads, 0, s>>>(vdata, p.vunits, p.warp_begin, p.nwarps, xt);
    nl++;
  }
  if (ev) cudaEventRecord(ev[2], s);
  DuMultiArgs<T> a{panels, p.tiles, p.units, p.nunits, p.segs, xt, p.tmap0, Y, ldy, nr,
                   p.counter, part, p.tile_cnt};
  du_multi_kernel<T><<<grid_du, kThreads, 0, s>>>(a);
  nl++;
  if (ev) cudaEventRecord(ev[3], s);
  if (launches) *launches = nl;
  return cudaGetLastError();
}

int rhs_per_pass() { return kRhs; }

int occupancy_du_multi(bool f64) {
  int n = 0;
  if (f64)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, du_multi_kernel<double>, kThreads, 0);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, du_multi_kernel<float>, kThreads, 0);
  return n > 0 ? n : 1;
}

cudaError_t launch_matvec_multi(bool f64, const DevPlan &p, const void *panels, const void *vdata,
                                void *xt, void *part, const void *X, int64_t ldx, int nr, void *Y,
                                int64_t ldy, int grid_v, int grid_du, cudaStream_t s,
                                cudaEvent_t *ev, int *launches) {
  if (f64)
    return run_multi<double>(p, static_cast<const double *>(panels), static_cast<const double *>(vdata),
                             static_cast<double *>(xt), static_cast<double *>(part),
                             static_cast<const double *>(X), ldx, nr, static_cast<double *>(Y), ldy,
                             grid_v, grid_du, s, ev, launches);
  return run_multi<float>(p, static_cast<const float *>(panels), static_cast<const float *>(vdata),
                          static_cast<float *>(xt), static_cast<float *>(part),
                          static_cast<const float *>(X), ldx, nr, static_cast<float *>(Y), ldy,
                          grid_v, grid_du, s, ev, launches);
}

}  // namespace hm
