// Single-right-hand-side H-matrix product kernels (sm_103a).
//
// Replaces the reference's device product (src/mult.jl:41-189):
//   V_mult_vec_kernel!  (:41-78)  -> v_pass_kernel: t = V x, one 16-byte-load
//                                    stream per rank row, sub-warp shuffle sums.
//   DU_mult_vec_kernel! (:80-146) -> du_rows_kernel: y = D x + U t, one warp per
//                                    row of a row tile; the row concatenates the
//                                    row's dense and low-rank columns, so each
//                                    output is one dot product with a fixed
//                                    summation order and no atomics.
// Both passes are bound by HBM bandwidth: every matrix byte is read once with
// 16-byte non-allocating loads; the vectors (x permuted into XT, t) are small
// and stay in L2.
#include <cuda_runtime.h>

#include "hm_device.h"

namespace hm {

template <typename T>
struct Vec16;
template <>
struct Vec16<float> {
  using type = float4;
  static constexpr int N = 4;
};
template <>
struct Vec16<double> {
  using type = double2;
  static constexpr int N = 2;
};

// Streaming 16-byte load of matrix data: read once, do not keep in L1.
__device__ __forceinline__ float4 ld_stream(const float4 *p) {
  float4 v;
  asm volatile("ld.global.nc.L1::no_allocate.v4.f32 {%0,%1,%2,%3}, [%4];"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
               : "l"(p));
  return v;
}
__device__ __forceinline__ double2 ld_stream(const double2 *p) {
  double2 v;
  asm volatile("ld.global.nc.L1::no_allocate.v2.f64 {%0,%1}, [%2];"
               : "=d"(v.x), "=d"(v.y)
               : "l"(p));
  return v;
}

__device__ __forceinline__ float fma_(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_(double a, double b, double c) { return __fma_rn(a, b, c); }

// Dot2 step (Ogita, Rump & Oishi, "Accurate sum and dot product", 2005):
// s + c carries the running dot product with the rounding errors of every
// product (TwoProduct via FMA) and every addition (TwoSum) collected in c.
template <typename T>
__device__ __forceinline__ void dot2_step(T &s, T &c, T a, T b) {
  T p = a * b;
  T pe = fma_(a, b, -p);
  T t = s + p;
  T z = t - s;
  T e = (s - (t - z)) + (p - z);
  s = t;
  c += e + pe;
}

// Lane partials of a row: plain or compensated.
template <typename T, bool COMP>
struct RowAcc {
  T s = T(0), c = T(0);
  __device__ __forceinline__ void add(const typename Vec16<T>::type &a,
                                      const typename Vec16<T>::type &b) {
    const T *ea = reinterpret_cast<const T *>(&a), *eb = reinterpret_cast<const T *>(&b);
#pragma unroll
    for (int q = 0; q < Vec16<T>::N; q++) {
      if (COMP)
        dot2_step(s, c, ea[q], eb[q]);
      else
        s = fma_(ea[q], eb[q], s);
    }
  }
  // Butterfly over the warp (fixed order); every lane ends with the total.
  __device__ __forceinline__ T total() {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const T s2 = __shfl_xor_sync(0xffffffffu, s, o);
      if (COMP) {
        const T c2 = __shfl_xor_sync(0xffffffffu, c, o);
        const T t = s + s2, z = t - s;
        c += c2 + ((s - (t - z)) + (s2 - z));
        s = t;
      } else {
        s += s2;
      }
    }
    return COMP ? s + c : s;
  }
};

// ---------------------------------------------------------------------------
// x permutation: XT[j] = x[smap[j]] for j < n (zero where smap[j] < 0), zero
// padding up to x_len.
// Also re-arms the unit ticket of the near/U pass.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void permute_x_kernel(const T *__restrict__ x, const int32_t *__restrict__ smap0,
                                 int64_t n, int64_t x_len, T *__restrict__ xt,
                                 int32_t *__restrict__ counter) {
  int64_t j = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (j == 0) {
    counter[0] = 0;  // near/U row units
    counter[8] = 0;  // V units (dynamic schedule)
  }
  for (; j < x_len; j += static_cast<int64_t>(gridDim.x) * blockDim.x)
    xt[j] = (j < n && smap0[j] >= 0) ? x[smap0[j]] : T(0);  // negative: padding between batch members
}

// ---------------------------------------------------------------------------
// V pass. A unit is a run of rank rows of one block; `lanes` lanes share a
// row and 32/lanes rows run side by side. Row storage is phase-aligned with
// XT, so element p of the row pairs with XT[x_off + p]. Two schedules, picked
// per matrix by the autotuner: each warp owns a contiguous, byte-balanced
// range of units (planned on the host), or warps take units one at a time
// from a ticket counter (the next ticket is drawn before the current unit
// runs), which evens out uneven speeds on matrices with long rows.
// ---------------------------------------------------------------------------
// Six CTAs per SM (40 registers) and four loads in flight per lane: the pass
// is bound by memory latency, like the near/U pass.
template <typename T>
__device__ __forceinline__ void v_unit(const T *__restrict__ V, const VUnit U, T *__restrict__ xt, int lane) {
  using VT = typename Vec16<T>::type;
  constexpr int VEC = Vec16<T>::N;
  const int g = U.lanes, slot = lane / g, sub = lane - slot * g, per = 32 / g;
  const int nv = U.stride / VEC;
  const VT *X = reinterpret_cast<const VT *>(xt + U.x_off);
  for (int k0 = 0; k0 < U.nrows; k0 += per) {
    const int k = k0 + slot;
    T acc = T(0);
    if (k < U.nrows) {
      const VT *row = reinterpret_cast<const VT *>(V + U.v_off + static_cast<int64_t>(k) * U.stride);
      int p = sub;
      for (; p + 3 * g < nv; p += 4 * g) {  // four 16-byte loads of V in flight per lane
        VT a0 = ld_stream(row + p), a1 = ld_stream(row + p + g);
        VT a2 = ld_stream(row + p + 2 * g), a3 = ld_stream(row + p + 3 * g);
        VT b0 = __ldg(X + p), b1 = __ldg(X + p + g), b2 = __ldg(X + p + 2 * g), b3 = __ldg(X + p + 3 * g);
        const T *ea0 = reinterpret_cast<const T *>(&a0), *eb0 = reinterpret_cast<const T *>(&b0);
        const T *ea1 = reinterpret_cast<const T *>(&a1), *eb1 = reinterpret_cast<const T *>(&b1);
        const T *ea2 = reinterpret_cast<const T *>(&a2), *eb2 = reinterpret_cast<const T *>(&b2);
        const T *ea3 = reinterpret_cast<const T *>(&a3), *eb3 = reinterpret_cast<const T *>(&b3);
#pragma unroll
        for (int q = 0; q < VEC; q++) acc = fma_(ea0[q], eb0[q], acc);
#pragma unroll
        for (int q = 0; q < VEC; q++) acc = fma_(ea1[q], eb1[q], acc);
#pragma unroll
        for (int q = 0; q < VEC; q++) acc = fma_(ea2[q], eb2[q], acc);
#pragma unroll
        for (int q = 0; q < VEC; q++) acc = fma_(ea3[q], eb3[q], acc);
      }
      for (; p + g < nv; p += 2 * g) {
        VT a0 = ld_stream(row + p), a1 = ld_stream(row + p + g);
        VT b0 = __ldg(X + p), b1 = __ldg(X + p + g);
        const T *ea0 = reinterpret_cast<const T *>(&a0), *eb0 = reinterpret_cast<const T *>(&b0);
        const T *ea1 = reinterpret_cast<const T *>(&a1), *eb1 = reinterpret_cast<const T *>(&b1);
#pragma unroll
        for (int q = 0; q < VEC; q++) acc = fma_(ea0[q], eb0[q], acc);
#pragma unroll
        for (int q = 0; q < VEC; q++) acc = fma_(ea1[q], eb1[q], acc);
      }
      if (p < nv) {
        VT a0 = ld_stream(row + p);
        VT b0 = __ldg(X + p);
        const T *ea0 = reinterpret_cast<const T *>(&a0), *eb0 = reinterpret_cast<const T *>(&b0);
#pragma unroll
        for (int q = 0; q < VEC; q++) acc = fma_(ea0[q], eb0[q], acc);
      }
    }
    for (int o = g >> 1; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (sub == 0 && k < U.nrows) xt[U.t_off + k] = acc;
  }
}

template <typename T>
__global__ void __launch_bounds__(kThreads, 6) v_pass_kernel(const T *__restrict__ V,
                                                          const VUnit *__restrict__ units,
                                                          const int32_t *__restrict__ warp_begin,
                                                          T *__restrict__ xt) {
  using VT = typename Vec16<T>::type;
  constexpr int VEC = Vec16<T>::N;
  const int warp = static_cast<int>((blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  const int u0 = warp_begin[warp], u1 = warp_begin[warp + 1];
  for (int u = u0; u < u1; u++) {
    const VUnit U = units[u];
    const int g = U.lanes, slot = lane / g, sub = lane - slot * g, per = 32 / g;
    const int nv = U.stride / VEC;
    const VT *X = reinterpret_cast<const VT *>(xt + U.x_off);
    for (int k0 = 0; k0 < U.nrows; k0 += per) {
      const int k = k0 + slot;
      T acc = T(0);
      if (k < U.nrows) {
        const VT *row = reinterpret_cast<const VT *>(V + U.v_off + static_cast<int64_t>(k) * U.stride);
        int p = sub;
        for (; p + 3 * g < nv; p += 4 * g) {  // four 16-byte loads of V in flight per lane
          VT a0 = ld_stream(row + p), a1 = ld_stream(row + p + g);
          VT a2 = ld_stream(row + p + 2 * g), a3 = ld_stream(row + p + 3 * g);
          VT b0 = __ldg(X + p), b1 = __ldg(X + p + g), b2 = __ldg(X + p + 2 * g), b3 = __ldg(X + p + 3 * g);
          const T *ea0 = reinterpret_cast<const T *>(&a0), *eb0 = reinterpret_cast<const T *>(&b0);
          const T *ea1 = reinterpret_cast<const T *>(&a1), *eb1 = reinterpret_cast<const T *>(&b1);
          const T *ea2 = reinterpret_cast<const T *>(&a2), *eb2 = reinterpret_cast<const T *>(&b2);
          const T *ea3 = reinterpret_cast<const T *>(&a3), *eb3 = reinterpret_cast<const T *>(&b3);
#pragma unroll
          for (int q = 0; q < VEC; q++) acc = fma_(ea0[q], eb0[q], acc);
#pragma unroll
          for (int q = 0; q < VEC; q++) acc = fma_(ea1[q], eb1[q], acc);
#pragma unroll
          for (int q = 0; q < VEC; q++) acc = fma_(ea2[q], eb2[q], acc);
#pragma unroll
          for (int q = 0; q < VEC; q++) acc = fma_(ea3[q], eb3[q], acc);
        }
        for (; p + g < nv; p += 2 * g) {
          VT a0 = ld_stream(row + p), a1 = ld_stream(row + p + g);
          VT b0 = __ldg(X + p), b1 = __ldg(X + p + g);
          const T *ea0 = reinterpret_cast<const T *>(&a0), *eb0 = reinterpret_cast<const T *>(&b0);
          const T *ea1 = reinterpret_cast<const T *>(&a1), *eb1 = reinterpret_cast<const T *>(&b1);
#pragma unroll
          for (int q = 0; q < VEC; q++) acc = fma_(ea0[q], eb0[q], acc);
#pragma unroll
          for (int q = 0; q < VEC; q++) acc = fma_(ea1[q], eb1[q], acc);
        }
        if (p < nv) {
          VT a0 = ld_stream(row + p);
          VT b0 = __ldg(X + p);
          const T *ea0 = reinterpret_cast<const T *>(&a0), *eb0 = reinterpret_cast<const T *>(&b0);
#pragma unroll
          for (int q = 0; q < VEC; q++) acc = fma_(ea0[q], eb0[q], acc);
        }
      }
      for (int o = g >> 1; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
      if (sub == 0 && k < U.nrows) xt[U.t_off + k] = acc;
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(kThreads, 6) v_pass_dyn_kernel(const T *__restrict__ V,
                                                              const VUnit *__restrict__ units,
                                                              int32_t nunits, T *__restrict__ xt,
                                                              int32_t *__restrict__ ticket) {
  const int lane = threadIdx.x & 31;
  int u = 0;
  if (lane == 0) u = atomicAdd(ticket, 1);
  u = __shfl_sync(0xffffffffu, u, 0);
  while (u < nunits) {
    int next = 0;
    if (lane == 0) next = atomicAdd(ticket, 1);
    v_unit(V, units[u], xt, lane);
    u = __shfl_sync(0xffffffffu, next, 0);
  }
}

// ---------------------------------------------------------------------------
// Near/U pass. CTAs take row units (rows of one tile) from a ticket counter,
// tiles with the most columns first. The CTA gathers the tile's vector
// entries (x for dense columns, t for rank columns) into shared memory once
// per unit (once per 16 rows when the tile needs several chunks of entries);
// then each warp streams one or two whole rows of the tile's
// row-major panel with 16-byte loads (up to 8 in flight per lane) against
// 16-byte shared-memory loads of the entries, and reduces across lanes with a
// fixed butterfly. Every lane adds its vectors in increasing column order in
// every loop form, so a row's sum does not depend on the unit it is in.
// ---------------------------------------------------------------------------
template <typename T>
struct DuArgs {
  const T *panels;
  const TileDesc *tiles;
  const RowUnit *units;
  int32_t nunits;
  const Seg *segs;
  const T *xt;
  const int32_t *tmap0;
  T *y;
  int32_t *counter;
};

template <typename T>
struct DuCols {
  static constexpr int value = 16384 / sizeof(T);  // vector entries cached per column chunk
};
constexpr int kDuSegs = 512;

// Six CTAs per SM (40 registers, a few spilled to L1) keep more rows, and so
// more 16-byte loads, in flight than five CTAs without spills: the pass is
// bound by memory latency, not by the instructions the spills add.
template <typename T, bool COMP>
__global__ void __launch_bounds__(kThreads, 6) du_rows_kernel(DuArgs<T> a) {
  using VT = typename Vec16<T>::type;
  constexpr int VEC = Vec16<T>::N;
  constexpr int CH = DuCols<T>::value;
  __shared__ __align__(16) T vals[CH];
  __shared__ Seg ssegs[kDuSegs];
  __shared__ int32_t s_ticket[2];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int it = 0;; it++) {
    if (tid == 0) s_ticket[it & 1] = atomicAdd(a.counter, 1);
    __syncthreads();
    const int32_t u = s_ticket[it & 1];
    if (u >= a.nunits) break;
    const RowUnit U = a.units[u];
    const TileDesc d = a.tiles[U.tile];
    const bool seg_smem = d.nseg <= kDuSegs;
    if (seg_smem)
      for (int s = tid; s < d.nseg; s += kThreads) ssegs[s] = a.segs[d.seg0 + s];
    const Seg *S = seg_smem ? ssegs : a.segs + d.seg0;
    // Rows 16 at a time (a warp per row pair); a unit has more than 16 rows
    // only when its tile fits one chunk of entries, which are then gathered
    // once for all its rows.
    const bool single = d.ld <= CH;
    for (int r0 = U.i0; r0 < U.i1; r0 += kThreads / 16) {
      const int ia = r0 + warp, ib = ia + kThreads / 32;
      const bool ha = ia < U.i1, hb = ib < U.i1;
      RowAcc<T, COMP> ra, rb;
      for (int c0 = 0; c0 < d.ld; c0 += CH) {
        const int cn = min(CH, d.ld - c0);
        if (!single || r0 == U.i0) {
          __syncthreads();  // segments loaded / previous chunk's entries no longer read
          for (int j = tid; j < cn; j += kThreads) {
            const int c = c0 + j;
            T v = T(0);
            if (c < d.ncols) {
              int lo = 0, hi = d.nseg - 1;  // last segment with col0 <= c
              while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (S[mid].col0 <= c)
                  lo = mid;
                else
                  hi = mid - 1;
              }
              v = a.xt[S[lo].vec_off + (c - S[lo].col0)];
            }
            vals[j] = v;
          }
          __syncthreads();
        }
        const int nv = cn / VEC;
        const VT *E = reinterpret_cast<const VT *>(vals);
        const VT *RA = reinterpret_cast<const VT *>(a.panels + d.data_off + static_cast<int64_t>(ia) * d.ld + c0);
        const VT *RB = reinterpret_cast<const VT *>(a.panels + d.data_off + static_cast<int64_t>(ib) * d.ld + c0);
        if (ha && hb) {
          int p = lane;
          for (; p + 96 < nv; p += 128) {
            const VT x0 = ld_stream(RA + p), x1 = ld_stream(RA + p + 32);
            const VT x2 = ld_stream(RA + p + 64), x3 = ld_stream(RA + p + 96);
            const VT z0 = ld_stream(RB + p), z1 = ld_stream(RB + p + 32);
            const VT z2 = ld_stream(RB + p + 64), z3 = ld_stream(RB + p + 96);
            const VT e0 = E[p], e1 = E[p + 32], e2 = E[p + 64], e3 = E[p + 96];
            ra.add(x0, e0);
            ra.add(x1, e1);
            ra.add(x2, e2);
            ra.add(x3, e3);
            rb.add(z0, e0);
            rb.add(z1, e1);
            rb.add(z2, e2);
            rb.add(z3, e3);
          }
          for (; p + 32 < nv; p += 64) {
            const VT x0 = ld_stream(RA + p), x1 = ld_stream(RA + p + 32);
            const VT z0 = ld_stream(RB + p), z1 = ld_stream(RB + p + 32);
            const VT e0 = E[p], e1 = E[p + 32];
            ra.add(x0, e0);
            ra.add(x1, e1);
            rb.add(z0, e0);
            rb.add(z1, e1);
          }
          if (p < nv) {
            const VT e0 = E[p];
            ra.add(ld_stream(RA + p), e0);
            rb.add(ld_stream(RB + p), e0);
          }
        } else if (ha) {
          int p = lane;
          for (; p + 96 < nv; p += 128) {
            const VT x0 = ld_stream(RA + p), x1 = ld_stream(RA + p + 32);
            const VT x2 = ld_stream(RA + p + 64), x3 = ld_stream(RA + p + 96);
            ra.add(x0, E[p]);
            ra.add(x1, E[p + 32]);
            ra.add(x2, E[p + 64]);
            ra.add(x3, E[p + 96]);
          }
          for (; p < nv; p += 32) ra.add(ld_stream(RA + p), E[p]);
        }
      }
      const T ya = ra.total(), yb = rb.total();
      if (lane == 0) {
        if (ha) a.y[a.tmap0[d.row0 + ia]] = ya;
        if (hb) a.y[a.tmap0[d.row0 + ib]] = yb;
      }
    }
  }
}

int occupancy_v(bool f64) {
  int n = 0;
  if (f64)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, v_pass_kernel<double>, kThreads, 0);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, v_pass_kernel<float>, kThreads, 0);
  return n > 0 ? n : 1;
}

int occupancy_du(bool f64, bool comp) {
  int n = 0;
  if (f64)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, du_rows_kernel<double, false>, kThreads, 0);
  else if (comp)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, du_rows_kernel<float, true>, kThreads, 0);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, du_rows_kernel<float, false>, kThreads, 0);
  return n > 0 ? n : 1;
}

template <typename T, bool COMP>
static cudaError_t run(const DevPlan &p, const T *panels, const T *vdata, T *xt, const T *x, T *y,
                       int grid_v, int grid_du, cudaStream_t s, cudaEvent_t *ev, int *launches) {
  int gp = static_cast<int>((p.x_len + kThreads - 1) / kThreads);
  if (gp > 4096) gp = 4096;
  int nl = 0;
  if (ev) cudaEventRecord(ev[0], s);
  permute_x_kernel<T><<<gp, kThreads, 0, s>>>(x, p.smap0, p.n, p.x_len, xt, p.counter);
  nl++;
  if (ev) cudaEventRecord(ev[1], s);
  if (!p.warp_begin_empty) {
    if (p.v_dynamic)
      v_pass_dyn_kernel<T><<<grid_v, kThreads, 0, s>>>(vdata, p.vunits, p.nvunits, xt, p.counter + 8);
    else
      v_pass_kernel<T><<<grid_v, kThreads, 0, s>>>(vdata, p.vunits, p.warp_begin, xt);
    nl++;
  }
  if (ev) cudaEventRecord(ev[2], s);
  DuArgs<T> a{panels, p.tiles, p.units, p.nunits, p.segs, xt, p.tmap0, y, p.counter};
  du_rows_kernel<T, COMP><<<grid_du, kThreads, 0, s>>>(a);
  nl++;
  if (ev) cudaEventRecord(ev[3], s);
  if (launches) *launches = nl;
  return cudaGetLastError();
}

cudaError_t launch_matvec(bool f64, bool comp, const DevPlan &p, const void *panels,
                          const void *vdata, void *xt, const void *x, void *y, int grid_v,
                          int grid_du, cudaStream_t stream, cudaEvent_t *ev, int *launches) {
  if (f64)
    return run<double, false>(p, static_cast<const double *>(panels),
                              static_cast<const double *>(vdata), static_cast<double *>(xt),
                              static_cast<const double *>(x), static_cast<double *>(y), grid_v,
                              grid_du, stream, ev, launches);
  if (comp)
    return run<float, true>(p, static_cast<const float *>(panels), static_cast<const float *>(vdata),
                            static_cast<float *>(xt), static_cast<const float *>(x),
                            static_cast<float *>(y), grid_v, grid_du, stream, ev, launches);
  return run<float, false>(p, static_cast<const float *>(panels), static_cast<const float *>(vdata),
                           static_cast<float *>(xt), static_cast<const float *>(x),
                           static_cast<float *>(y), grid_v, grid_du, stream, ev, launches);
}

// ---------------------------------------------------------------------------
// packing: row-major factors (FP64, or FP32 for FP32 storage) -> product
// layout (one warp per job)
// ---------------------------------------------------------------------------
template <typename T, typename S>
__global__ void pack_panels_kernel(const PackJob *__restrict__ jobs, int64_t njobs, const S *__restrict__ dsrc,
                                   const S *__restrict__ usrc, T *__restrict__ panels) {
  const int lane = threadIdx.x & 31;
  const int64_t w0 = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
  const int64_t nw = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
  for (int64_t w = w0; w < njobs; w += nw) {
    const PackJob j = jobs[w];
    if (j.kind == 2) continue;
    const S *src = (j.kind == 0 ? dsrc : usrc) + j.src_off;
    for (int i = 0; i < j.m; i++)
      for (int c = lane; c < j.ncols; c += 32)
        panels[j.dst_off + static_cast<int64_t>(i) * j.dst_ld + c] =
            static_cast<T>(src[static_cast<int64_t>(i) * j.src_ld + c]);
  }
}

template <typename T, typename S>
__global__ void pack_v_kernel(const VPackJob *__restrict__ jobs, int64_t njobs, const S *__restrict__ vsrc,
                              T *__restrict__ vdata) {
  const int lane = threadIdx.x & 31;
  const int64_t w0 = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
  const int64_t nw = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
  for (int64_t w = w0; w < njobs; w += nw) {
    const VPackJob j = jobs[w];
    const int64_t total = static_cast<int64_t>(j.r) * j.n;
    for (int64_t e = lane; e < total; e += 32) {
      const int64_t k = e / j.n, c = e - k * j.n;
      vdata[j.dst_off + k * j.stride + j.phase + c] = static_cast<T>(vsrc[j.src_off + e]);
    }
  }
}

cudaError_t launch_pack_panels(bool f64, bool src32, const PackJob *jobs, int64_t njobs, const void *dsrc,
                               const void *usrc, void *panels, cudaStream_t s) {
  if (njobs == 0) return cudaSuccess;
  int grid = static_cast<int>((njobs + 7) / 8);
  if (grid > 65535) grid = 65535;
  if (src32)  // FP32 factors go to FP32 storage only
    pack_panels_kernel<float, float><<<grid, kThreads, 0, s>>>(jobs, njobs, static_cast<const float *>(dsrc),
                                                               static_cast<const float *>(usrc),
                                                               static_cast<float *>(panels));
  else if (f64)
    pack_panels_kernel<double, double><<<grid, kThreads, 0, s>>>(jobs, njobs, static_cast<const double *>(dsrc),
                                                                 static_cast<const double *>(usrc),
                                                                 static_cast<double *>(panels));
  else
    pack_panels_kernel<float, double><<<grid, kThreads, 0, s>>>(jobs, njobs, static_cast<const double *>(dsrc),
                                                                static_cast<const double *>(usrc),
                                                                static_cast<float *>(panels));
  return cudaGetLastError();
}

cudaError_t launch_pack_v(bool f64, bool src32, const VPackJob *jobs, int64_t njobs, const void *vsrc, void *vdata,
                          cudaStream_t s) {
  if (njobs == 0) return cudaSuccess;
  int grid = static_cast<int>((njobs + 7) / 8);
  if (grid > 65535) grid = 65535;
  if (src32)
    pack_v_kernel<float, float><<<grid, kThreads, 0, s>>>(jobs, njobs, static_cast<const float *>(vsrc),
                                                          static_cast<float *>(vdata));
  else if (f64)
    pack_v_kernel<double, double><<<grid, kThreads, 0, s>>>(jobs, njobs, static_cast<const double *>(vsrc),
                                                            static_cast<double *>(vdata));
  else
    pack_v_kernel<float, double><<<grid, kThreads, 0, s>>>(jobs, njobs, static_cast<const double *>(vsrc),
                                                           static_cast<float *>(vdata));
  return cudaGetLastError();
}

}  // namespace hm
