// Multi-right-hand-side H-matrix product, plain form (FP32 or FP64 on the CUDA
// cores): Y = H X for up to kRhs right-hand sides per pass.
//
// A pass is W right-hand sides wide (W = 8, 16 or 32: the narrowest that holds
// the pass's columns). XT holds, for every permuted source index and every
// rank row, the W values of that row contiguously (row-major, 4W bytes per row
// in FP32). The matrix is read once per pass and every element feeds W FMAs,
// so the 32-wide form is bound by the CUDA cores' FMA rate and the 8-wide one
// by HBM.
//
// Both passes run the same register-tiled micro-kernel over panels of at most
// 128 rows (multi_panel below); partial sums of the column slices meet in
// shared memory in a fixed order, so results are deterministic.
#include <cuda_runtime.h>

#include "hm_device.h"

namespace hm {

constexpr int kRhs = 32;  // right-hand sides per pass at most (row length of XT)

template <typename T, int W>
struct Cols {
  static constexpr int value = 16384 / (W * sizeof(T));  // XT rows staged at once
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

template <typename T, int N>
__device__ __forceinline__ void ldsn(const T *p, T (&v)[N]) {
  if constexpr (sizeof(T) == 4) {
#pragma unroll
    for (int q = 0; q < N / 4; q++) {
      const float4 a = reinterpret_cast<const float4 *>(p)[q];
      v[4 * q] = a.x; v[4 * q + 1] = a.y; v[4 * q + 2] = a.z; v[4 * q + 3] = a.w;
    }
  } else {
#pragma unroll
    for (int q = 0; q < N / 2; q++) {
      const double2 a = reinterpret_cast<const double2 *>(p)[q];
      v[2 * q] = a.x;
      v[2 * q + 1] = a.y;
    }
  }
}

// XT rows from X in its own order: X[j + r ldx] goes to XT[sinv[j] W + r]
// (0 for r >= nr). Reads of X are coalesced along j and every XT row is written
// whole; the x-region rows that no source index maps to stay zero (every pass
// width has its own XT, zeroed once). Also re-arms both ticket counters.
template <typename T, int W>
__global__ void permute_multi_kernel(const T *__restrict__ X, int64_t ldx, int nr,
                                     const int32_t *__restrict__ sinv0, int64_t n_src,
                                     T *__restrict__ xt, int32_t *__restrict__ counter) {
  __shared__ T tile[64][W + 1];
  if (blockIdx.x == 0 && threadIdx.x < 2) counter[threadIdx.x] = 0;  // both ticket slots
  for (int64_t j0 = blockIdx.x * 64ll; j0 < n_src; j0 += gridDim.x * 64ll) {
    for (int e = threadIdx.x; e < 64 * W; e += blockDim.x) {
      const int r = e / 64, jj = e % 64;  // consecutive threads: consecutive j
      const int64_t j = j0 + jj;
      tile[jj][r] = (j < n_src && r < nr) ? X[j + r * ldx] : T(0);
    }
    __syncthreads();
    for (int e = threadIdx.x; e < 64 * W; e += blockDim.x) {
      const int jj = e / W, r = e % W;
      if (j0 + jj < n_src) xt[static_cast<int64_t>(sinv0[j0 + jj]) * W + r] = tile[jj][r];
    }
    __syncthreads();
  }
}

// 16-byte asynchronous copy global -> shared; zeros when `valid` is false
// (then nothing is read from `src`).
__device__ __forceinline__ void cp16(void *dst, const void *src, bool valid) {
  const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(dst));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(d), "l"(src), "r"(valid ? 16 : 0)
               : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// One panel of m <= 128 rows (row-major, stride lda, rows padded with zeros to
// a multiple of 4 columns) times the W-wide XT rows of its columns. A thread
// keeps TR rows x TW right-hand sides of accumulators (4 x 8 for W = 8, 2 x 16
// otherwise, so that fewer threads load the same A entries); the layout is
// ceil(m / TR) row groups x W / TW right-hand-side groups x S column slices,
// and a thread steps 4 columns at a time (TR 16-byte loads of A, 4 TW values
// of XT rows from shared memory, 4 TR TW FMAs). `stage(c0, cn, xs)` issues the asynchronous
// copies (cp16) of the XT rows of columns [c0, c0 + cn) into xs; the XT rows of
// the next CC columns are copied into the other half of `buf` while the FMAs
// of the current ones run. The slices meet in shared memory in slice order.
template <typename T, int W, typename Stage, typename Emit>
__device__ __forceinline__ void multi_panel(const T *A, int64_t lda, int m, int ncols_pad, T *buf,
                                            Stage stage, Emit emit) {
  constexpr int CC = Cols<T, W>::value;
  constexpr int TW = W == 8 ? 8 : 16;  // right-hand sides per thread
  constexpr int TR = 32 / TW;          // rows per thread
  constexpr int G = W / TW;            // threads sharing a row group (each loads its A)
  T *red = buf;
  const int tid = threadIdx.x;
  const int RQ = (m + TR - 1) / TR, per = RQ * G;
  int S = kThreads / per;
  if (S < 1) S = 1;
  const int ks = tid / per, r = tid - ks * per, rq = r % RQ, rg = r / RQ;
  const bool active = ks < S;
  T acc[TR][TW];
#pragma unroll
  for (int i = 0; i < TR; i++)
#pragma unroll
    for (int j = 0; j < TW; j++) acc[i][j] = T(0);
  bool ok[TR];
#pragma unroll
  for (int i = 0; i < TR; i++) ok[i] = rq * TR + i < m;
  const int nst = (ncols_pad + CC - 1) / CC;
  __syncthreads();  // buf free (the previous panel's slice sums are read)
  if (nst > 0) stage(0, min(CC, ncols_pad), buf);
  cp_commit();
  for (int st = 0; st < nst; st++) {
    const int c0 = st * CC, cn = min(CC, ncols_pad - c0);
    const T *xs = buf + (st & 1) * CC * W;
    cp_wait_all();
    __syncthreads();  // stage st in place everywhere; stage st - 1's half is free
    if (st + 1 < nst) stage(c0 + CC, min(CC, ncols_pad - c0 - CC), buf + ((st + 1) & 1) * CC * W);
    cp_commit();
    if (active) {
      // the A entries of the next step are loaded before this step's FMAs
      const int step = 4 * S;
      auto load = [&](int c, T (&d)[TR][4]) {
#pragma unroll
        for (int i = 0; i < TR; i++) {
          if (ok[i] && c < cn)
            ld4(A + static_cast<int64_t>(rq * TR + i) * lda + c0 + c, d[i]);
          else
            d[i][0] = d[i][1] = d[i][2] = d[i][3] = T(0);
        }
      };
      auto step_fma = [&](int c, const T (&a)[TR][4]) {
#pragma unroll
        for (int k = 0; k < 4; k++) {
          T b[TW];
          ldsn<T, TW>(xs + (c + k) * W + rg * TW, b);
#pragma unroll
          for (int i = 0; i < TR; i++)
#pragma unroll
            for (int j = 0; j < TW; j++) acc[i][j] = fma(a[i][k], b[j], acc[i][j]);
        }
      };
      T a0[TR][4], a1[TR][4];
      int c = 4 * ks;
      load(c, a0);
      while (c < cn) {
        load(c + step, a1);
        step_fma(c, a0);
        c += step;
        if (c >= cn) break;
        load(c + step, a0);
        step_fma(c, a1);
        c += step;
      }
    }
  }
  __syncthreads();  // red aliases xs
  if (active)
#pragma unroll
    for (int i = 0; i < TR; i++)
#pragma unroll
      for (int j = 0; j < TW; j++) red[((ks * RQ + rq) * TR + i) * W + rg * TW + j] = acc[i][j];
  __syncthreads();
  for (int o = tid; o < m * W; o += kThreads) {
    const int row = o / W, q = o % W;
    T s = T(0);
    for (int sl = 0; sl < S; sl++) s += red[(sl * RQ * TR + row) * W + q];
    emit(row, q, s);
  }
}

// V pass: for every multi-RHS V item (ticket order)
//   out[(I.out + k) * W + r] = sum_j V[k, j] XT[(I.x_off + j) * W + r],
// out = XT (t rows) or the partial rows P of a cut group.
template <typename T, int W>
__global__ void __launch_bounds__(kThreads) v_multi_kernel(const T *__restrict__ V,
                                                           const MVItem *__restrict__ items,
                                                           int32_t nitems, T *__restrict__ xt,
                                                           T *__restrict__ P, int32_t *counter) {
  extern __shared__ __align__(16) unsigned char dyn_smem[];
  T *buf = reinterpret_cast<T *>(dyn_smem);  // XT rows while streaming, slice sums after
  __shared__ int32_t s_ticket[2];
  for (int it = 0;; it++) {
    if (threadIdx.x == 0) s_ticket[it & 1] = atomicAdd(counter, 1);
    __syncthreads();
    const int32_t u = s_ticket[it & 1];
    if (u >= nitems) break;
    const MVItem I = items[u];
    const T *src = xt + static_cast<int64_t>(I.x_off) * W;
    T *out = I.kind == 0 ? xt : P;
    multi_panel<T, W>(
        V + I.v_off, I.stride, I.nrows, I.ncols, buf,
        [&](int c0, int cn, T *xs) {  // contiguous XT rows
          constexpr int kV = 16 / sizeof(T);  // values per 16-byte copy
          for (int e = threadIdx.x; e < cn * W / kV; e += kThreads)
            cp16(xs + e * kV, src + static_cast<int64_t>(c0) * W + e * kV, true);
        },
        [&](int row, int q, T s) { out[static_cast<int64_t>(I.out + row) * W + q] = s; });
  }
}

// t rows of cut groups: pieces summed in order (one warp per row, lane = RHS).
template <typename T, int W>
__global__ void reduce_multi_kernel(const MVReduce *__restrict__ red, int32_t nred, const T *__restrict__ P,
                                    T *__restrict__ xt) {
  const int lane = threadIdx.x & 31;
  if (lane >= W) return;
  for (int32_t e = static_cast<int32_t>(blockIdx.x); e < nred; e += gridDim.x) {
    const MVReduce R = red[e];
    for (int row = threadIdx.x >> 5; row < R.nrows; row += blockDim.x >> 5) {
      T s = T(0);
      for (int j = 0; j < R.npieces; j++)
        s += P[(static_cast<int64_t>(R.p_row) + static_cast<int64_t>(j) * R.nrows + row) * W + lane];
      xt[static_cast<int64_t>(R.t_row + row) * W + lane] = s;
    }
  }
}

// Near/U pass: one whole row tile per CTA (tiles from a ticket counter).
template <typename T>
struct DuMultiArgs {
  const T *panels;
  const TileDesc *tiles;
  const int32_t *order;  // tiles by decreasing work
  int32_t ntiles;
  const Seg *segs;
  const T *xt;
  const int32_t *tmap0;
  T *y;
  int64_t ldy;
  int nr;
  int32_t *counter;
};

template <typename T, int W>
__global__ void __launch_bounds__(kThreads) du_multi_kernel(DuMultiArgs<T> a) {
  extern __shared__ __align__(16) unsigned char dyn_smem[];
  T *buf = reinterpret_cast<T *>(dyn_smem);  // two halves of staged XT rows, slice sums after
  __shared__ int32_t s_ticket[2];
  const int tid = threadIdx.x;
  for (int it = 0;; it++) {
    if (tid == 0) s_ticket[it & 1] = atomicAdd(a.counter, 1);
    __syncthreads();
    const int32_t u = s_ticket[it & 1];
    if (u >= a.ntiles) break;
    const TileDesc d = a.tiles[a.order[u]];
    const Seg *S = a.segs + d.seg0;
    multi_panel<T, W>(
        a.panels + d.data_off, d.ld, d.m, d.ld, buf,
        [&](int c0, int cn, T *xs) {  // one thread per column: its XT row, then its copies
          constexpr int kP = W * static_cast<int>(sizeof(T)) / 16;  // 16-byte pieces per XT row
          for (int j = threadIdx.x; j < cn; j += kThreads) {
            const int c = c0 + j;
            int v = -1;
            if (c < d.ncols) {
              int lo = 0, hi = d.nseg - 1;
              while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (S[mid].col0 <= c)
                  lo = mid;
                else
                  hi = mid - 1;
              }
              v = S[lo].vec_off + (c - S[lo].col0);
            }
            const T *src = a.xt + static_cast<int64_t>(v >= 0 ? v : 0) * W;
#pragma unroll
            for (int q = 0; q < kP; q++) cp16(xs + j * W + q * (16 / sizeof(T)), src + q * (16 / sizeof(T)), v >= 0);
          }
        },
        [&](int row, int q, T s) {
          if (q < a.nr) a.y[a.tmap0[d.row0 + row] + q * a.ldy] = s;
        });
  }
}

// Dynamic shared memory of the multi-RHS kernels: 32 accumulators per thread
// for the slice reduction (also holds the staged XT rows).
template <typename T>
constexpr size_t multi_smem() {
  return static_cast<size_t>(kThreads) * 32 * sizeof(T);
}

template <typename T, int W>
static void multi_attrs() {
  static bool done = false;  // once per process (the attribute is per function)
  if (done) return;
  cudaFuncSetAttribute(v_multi_kernel<T, W>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       static_cast<int>(multi_smem<T>()));
  cudaFuncSetAttribute(du_multi_kernel<T, W>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       static_cast<int>(multi_smem<T>()));
  done = true;
}

template <typename T, int W>
static cudaError_t run_multi(const DevPlan &p, const T *panels, const T *vdata, T *xt, T *P, const T *X,
                             int64_t ldx, int nr, T *Y, int64_t ldy, int grid_du,
                             cudaStream_t s, cudaEvent_t *ev, int *launches) {
  multi_attrs<T, W>();
  int gp = static_cast<int>((p.n_src + 63) / 64);
  if (gp > 2048) gp = 2048;
  int nl = 0;
  if (ev) cudaEventRecord(ev[0], s);
  permute_multi_kernel<T, W><<<gp, kThreads, 0, s>>>(X, ldx, nr, p.sinv0, p.n_src, xt, p.counter);
  nl++;
  if (ev) cudaEventRecord(ev[1], s);
  if (p.nmv > 0) {
    v_multi_kernel<T, W><<<grid_du, kThreads, multi_smem<T>(), s>>>(vdata, p.mv_items, p.nmv, xt, P, p.counter);
    nl++;
    if (p.nmvr > 0) {
      reduce_multi_kernel<T, W><<<p.nmvr < 4096 ? p.nmvr : 4096, kThreads, 0, s>>>(p.mv_reduce, p.nmvr, P, xt);
      nl++;
    }
  }
  if (ev) cudaEventRecord(ev[2], s);
  DuMultiArgs<T> a{panels, p.tiles, p.tile_order, p.ntiles, p.segs, xt, p.tmap0, Y, ldy, nr, p.counter + 1};
  du_multi_kernel<T, W><<<grid_du, kThreads, multi_smem<T>(), s>>>(a);
  nl++;
  if (ev) cudaEventRecord(ev[3], s);
  if (launches) *launches = nl;
  return cudaGetLastError();
}

int rhs_per_pass() { return kRhs; }

int multi_width(int nr) { return nr <= 8 ? 8 : nr <= 16 ? 16 : kRhs; }

int occupancy_du_multi(bool f64) {
  int n = 0;
  if (f64) {
    multi_attrs<double, kRhs>();
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, du_multi_kernel<double, kRhs>, kThreads, multi_smem<double>());
  } else {
    multi_attrs<float, kRhs>();
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, du_multi_kernel<float, kRhs>, kThreads, multi_smem<float>());
  }
  return n > 0 ? n : 1;
}

template <typename T>
static cudaError_t run_multi_w(const DevPlan &p, const T *panels, const T *vdata, T *xt, T *P, const T *X,
                               int64_t ldx, int nr, T *Y, int64_t ldy, int grid_du, cudaStream_t s,
                               cudaEvent_t *ev, int *launches) {
  switch (multi_width(nr)) {
    case 8: return run_multi<T, 8>(p, panels, vdata, xt, P, X, ldx, nr, Y, ldy, grid_du, s, ev, launches);
    case 16: return run_multi<T, 16>(p, panels, vdata, xt, P, X, ldx, nr, Y, ldy, grid_du, s, ev, launches);
    default: return run_multi<T, kRhs>(p, panels, vdata, xt, P, X, ldx, nr, Y, ldy, grid_du, s, ev, launches);
  }
}

cudaError_t launch_matvec_multi(bool f64, const DevPlan &p, const void *panels, const void *vdata,
                                void *xt, void *P, const void *X, int64_t ldx, int nr, void *Y,
                                int64_t ldy, int grid_du, cudaStream_t s, cudaEvent_t *ev,
                                int *launches) {
  if (f64)
    return run_multi_w<double>(p, static_cast<const double *>(panels), static_cast<const double *>(vdata),
                             static_cast<double *>(xt), static_cast<double *>(P),
                             static_cast<const double *>(X), ldx, nr, static_cast<double *>(Y), ldy,
                             grid_du, s, ev, launches);
  return run_multi_w<float>(p, static_cast<const float *>(panels), static_cast<const float *>(vdata),
                          static_cast<float *>(xt), static_cast<float *>(P), static_cast<const float *>(X),
                          ldx, nr, static_cast<float *>(Y), ldy, grid_du, s, ev, launches);
}

}  // namespace hm
