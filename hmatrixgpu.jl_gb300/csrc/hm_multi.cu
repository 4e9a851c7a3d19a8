// Multi-right-hand-side H-matrix product, plain form (FP32 or FP64 on the CUDA
// cores): Y = H X for up to kRhs right-hand sides per pass.
//
// XT holds, for every permuted source index and every rank row, the kRhs values
// of that row contiguously (row-major, 128 bytes per row in FP32). The matrix
// is read once per pass and every element feeds kRhs FMAs, so this form is
// bound by the CUDA cores' FMA rate, not by HBM.
//
// Both passes run the same register-tiled micro-kernel: a thread owns 4 matrix
// rows x 8 right-hand sides (32 accumulators) over one of 16 column slices;
// per step it loads 4 columns of its 4 rows (four 16-byte loads) and the 4
// matching XT rows from shared memory (eight 16-byte loads) for 128 FMAs. The
// 16 slices of an output sit in 16 lanes of one warp and meet in a fixed
// shuffle butterfly, so results are deterministic.
#include <cuda_runtime.h>

#include "hm_device.h"

namespace hm {

constexpr int kRhs = 32;   // right-hand sides per pass (row length of XT)
constexpr int kSl = 16;    // column slices (lanes of a half-warp)
constexpr int kRows = 16;  // matrix rows per step of the micro-kernel (4 quads)

template <typename T>
struct Cols {
  static constexpr int value = 16384 / (kRhs * sizeof(T));  // XT rows staged at once
};

template <typename T>
struct V4;
template <>
struct V4<float> {
  using type = float4;
};
template <>
struct V4<double> {
  struct type {
    double x, y, z, w;
  };
};

template <typename T>
__device__ __forceinline__ void ld4(const T *p, T (&v)[4]) {
  if constexpr (sizeof(T) == 4) {
    const float4 a = __ldcs(reinterpret_cast<const float4 *>(p));
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
  } else {
    const double2 a = __ldcs(reinterpret_cast<const double2 *>(p));
    const double2 b = __ldcs(reinterpret_cast<const double2 *>(p) + 1);
    v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
  }
}

template <typename T>
__device__ __forceinline__ void lds8(const T *p, T (&v)[8]) {
  if constexpr (sizeof(T) == 4) {
    const float4 a = reinterpret_cast<const float4 *>(p)[0], b = reinterpret_cast<const float4 *>(p)[1];
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
  } else {
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const double2 a = reinterpret_cast<const double2 *>(p)[q];
      v[2 * q] = a.x;
      v[2 * q + 1] = a.y;
    }
  }
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

// The micro-kernel over columns [c0, c0 + cn) of `nrows` (<= 16) rows starting
// at A (row stride lda, 16-byte aligned, columns padded with zeros to a
// multiple of 4), against XT rows staged in xs (cn rows of kRhs values).
template <typename T>
struct Tile4x8 {
  T acc[4][8];
  __device__ __forceinline__ void zero() {
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
      for (int j = 0; j < 8; j++) acc[i][j] = T(0);
  }
  __device__ __forceinline__ void run(const T *A, int64_t lda, int nrows, int rq, int rg, int ks,
                                      const T *xs, int cn) {
    const bool ok[4] = {rq * 4 + 0 < nrows, rq * 4 + 1 < nrows, rq * 4 + 2 < nrows, rq * 4 + 3 < nrows};
    for (int c = 4 * ks; c < cn; c += 4 * kSl) {
      T a[4][4];
#pragma unroll
      for (int i = 0; i < 4; i++) {
        if (ok[i])
          ld4(A + static_cast<int64_t>(rq * 4 + i) * lda + c, a[i]);
        else
          a[i][0] = a[i][1] = a[i][2] = a[i][3] = T(0);
      }
#pragma unroll
      for (int k = 0; k < 4; k++) {
        T b[8];
        lds8(xs + (c + k) * kRhs + rg * 8, b);
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
          for (int j = 0; j < 8; j++) acc[i][j] = fma(a[i][k], b[j], acc[i][j]);
      }
    }
  }
  // Sums the 16 slices (lanes ks = 0..15 of a half-warp) in a fixed butterfly.
  __device__ __forceinline__ void reduce() {
#pragma unroll
    for (int o = kSl / 2; o > 0; o >>= 1)
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 8; j++) acc[i][j] += __shfl_xor_sync(0xffffffffu, acc[i][j], o);
  }
};

// V pass: t[(t_off + k) * kRhs + r] = sum_j V[k, j] XT[(x_off + j) * kRhs + r].
// CTA b works through units [warp_begin[8b], warp_begin[8b + 8]), the same
// byte-balanced split as the single-right-hand-side pass.
template <typename T>
__global__ void __launch_bounds__(kThreads) v_multi_kernel(const T *__restrict__ V,
                                                           const VUnit *__restrict__ units,
                                                           const int32_t *__restrict__ warp_begin,
                                                           int nwarps, T *__restrict__ xt) {
  constexpr int CC = Cols<T>::value;
  __shared__ __align__(16) T xs[CC * kRhs];
  const int tid = threadIdx.x, ks = tid % kSl, rg = (tid / kSl) % 4, rq = tid / (kSl * 4);
  const int w0 = blockIdx.x * (kThreads / 32);
  if (w0 >= nwarps) return;
  const int u0 = warp_begin[w0], u1 = warp_begin[min(w0 + kThreads / 32, nwarps)];
  for (int u = u0; u < u1; u++) {
    const VUnit U = units[u];
    for (int k0 = 0; k0 < U.nrows; k0 += kRows) {
      const int rows = min(kRows, U.nrows - k0);
      Tile4x8<T> t;
      t.zero();
      for (int c0 = 0; c0 < U.stride; c0 += CC) {
        const int cn = min(CC, U.stride - c0);
        __syncthreads();
        const T *src = xt + static_cast<int64_t>(U.x_off + c0) * kRhs;
        for (int e = tid; e < cn * kRhs; e += kThreads) xs[e] = src[e];
        __syncthreads();
        t.run(V + U.v_off + static_cast<int64_t>(k0) * U.stride + c0, U.stride, rows, rq, rg, ks, xs, cn);
      }
      t.reduce();
      if (ks == 0)
#pragma unroll
        for (int i = 0; i < 4; i++)
          if (rq * 4 + i < rows)
#pragma unroll
            for (int j = 0; j < 8; j++)
              xt[static_cast<int64_t>(U.t_off + k0 + rq * 4 + i) * kRhs + rg * 8 + j] = t.acc[i][j];
    }
  }
}

// Near/U pass over the row units of the single-RHS pass.
template <typename T>
struct DuMultiArgs {
  const T *panels;
  const TileDesc *tiles;
  const RowUnit *units;
  int32_t nunits;
  const Seg *segs;
  const T *xt;
  const int32_t *tmap0;
  T *y;
  int64_t ldy;
  int nr;
  int32_t *counter;
};

template <typename T>
__global__ void __launch_bounds__(kThreads) du_multi_kernel(DuMultiArgs<T> a) {
  constexpr int CC = Cols<T>::value;
  __shared__ __align__(16) T xs[CC * kRhs];
  __shared__ int32_t s_ticket[2];
  const int tid = threadIdx.x, ks = tid % kSl, rg = (tid / kSl) % 4, rq = tid / (kSl * 4);
  for (int it = 0;; it++) {
    if (tid == 0) s_ticket[it & 1] = atomicAdd(a.counter, 1);
    __syncthreads();
    const int32_t u = s_ticket[it & 1];
    if (u >= a.nunits) break;
    const RowUnit U = a.units[u];
    const TileDesc d = a.tiles[U.tile];
    const int rows = U.i1 - U.i0;
    Tile4x8<T> t;
    t.zero();
    for (int c0 = 0; c0 < d.ld; c0 += CC) {
      const int cn = min(CC, d.ld - c0);
      __syncthreads();
      for (int e = tid; e < cn * kRhs; e += kThreads) {
        const int c = c0 + e / kRhs;
        T v = T(0);
        if (c < d.ncols) {
          int lo = 0, hi = d.nseg - 1;
          const Seg *S = a.segs + d.seg0;
          while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (S[mid].col0 <= c)
              lo = mid;
            else
              hi = mid - 1;
          }
          v = a.xt[static_cast<int64_t>(S[lo].vec_off + (c - S[lo].col0)) * kRhs + (e % kRhs)];
        }
        xs[e] = v;
      }
      __syncthreads();
      t.run(a.panels + d.data_off + static_cast<int64_t>(U.i0) * d.ld + c0, d.ld, rows, rq, rg, ks,
            xs, cn);
    }
    t.reduce();
    if (ks == 0)
#pragma unroll
      for (int i = 0; i < 4; i++)
        if (rq * 4 + i < rows) {
          const int64_t yrow = a.tmap0[d.row0 + U.i0 + rq * 4 + i];
#pragma unroll
          for (int j = 0; j < 8; j++)
            if (rg * 8 + j < a.nr) a.y[yrow + (rg * 8 + j) * a.ldy] = t.acc[i][j];
        }
  }
}

template <typename T>
static cudaError_t run_multi(const DevPlan &p, const T *panels, const T *vdata, T *xt, const T *X,
                             int64_t ldx, int nr, T *Y, int64_t ldy, int grid_v, int grid_du,
                             cudaStream_t s, cudaEvent_t *ev, int *launches) {
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
  DuMultiArgs<T> a{panels, p.tiles, p.units, p.nunits, p.segs, xt, p.tmap0, Y, ldy, nr, p.counter};
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
                                void *xt, const void *X, int64_t ldx, int nr, void *Y, int64_t ldy,
                                int grid_v, int grid_du, cudaStream_t s, cudaEvent_t *ev,
                                int *launches) {
  if (f64)
    return run_multi<double>(p, static_cast<const double *>(panels), static_cast<const double *>(vdata),
                             static_cast<double *>(xt), static_cast<const double *>(X), ldx, nr,
                             static_cast<double *>(Y), ldy, grid_v, grid_du, s, ev, launches);
  return run_multi<float>(p, static_cast<const float *>(panels), static_cast<const float *>(vdata),
                          static_cast<float *>(xt), static_cast<const float *>(X), ldx, nr,
                          static_cast<float *>(Y), ldy, grid_v, grid_du, s, ev, launches);
}

}  // namespace hm
