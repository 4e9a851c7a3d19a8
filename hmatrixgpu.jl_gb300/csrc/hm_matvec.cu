// Single-right-hand-side H-matrix product kernels (sm_103a).
//
// Replaces the reference's device product (src/mult.jl:41-189):
//   V_mult_vec_kernel!  (:41-78)  -> v_pass_kernel: t = V x, one 16-byte-load
//                                    stream per rank row, sub-warp shuffle sums.
//   DU_mult_vec_kernel! (:80-146) -> du_pass_kernel: y = D x + U t over row
//                                    tiles; each tile owns its rows of y, so the
//                                    sums have a fixed order and need no atomics.
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

// ---------------------------------------------------------------------------
// x permutation: XT[j] = x[smap[j]] for j < n, zero padding up to x_len.
// Also re-arms the tile ticket of the near/U pass.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void permute_x_kernel(const T *__restrict__ x, const int32_t *__restrict__ smap0,
                                 int64_t n, int64_t x_len, T *__restrict__ xt,
                                 int32_t *__restrict__ counter) {
  int64_t j = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (j == 0) *counter = 0;
  for (; j < x_len; j += static_cast<int64_t>(gridDim.x) * blockDim.x)
    xt[j] = j < n ? x[smap0[j]] : T(0);
}

// ---------------------------------------------------------------------------
// V pass. Each warp owns a contiguous, byte-balanced range of units (planned on
// the host). A unit is a run of rank rows of one block; `lanes` lanes share a
// row and 32/lanes rows run side by side. Row storage is phase-aligned with
// XT, so element p of the row pairs with XT[x_off + p].
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(kThreads) v_pass_kernel(const T *__restrict__ V,
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
        for (; p + 3 * g < nv; p += 4 * g) {  // four 16-byte loads in flight per lane
          VT a[4], b[4];
#pragma unroll
          for (int s = 0; s < 4; s++) a[s] = ld_stream(row + p + s * g);
#pragma unroll
          for (int s = 0; s < 4; s++) b[s] = __ldg(X + p + s * g);
#pragma unroll
          for (int s = 0; s < 4; s++) {
            const T *ea = reinterpret_cast<const T *>(&a[s]), *eb = reinterpret_cast<const T *>(&b[s]);
#pragma unroll
            for (int q = 0; q < VEC; q++) acc = fma_(ea[q], eb[q], acc);
          }
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

// ---------------------------------------------------------------------------
// Near/U pass. CTAs take units (column slices of a row tile) from a ticket
// counter, largest tiles first. A tile of m rows is a column-major panel; the
// CTA's threads form G groups of m threads. Thread t of group g loads the
// 16-byte vectors f = t + m*q, q = g (mod G). Because a vector holds VEC
// elements and the group spans VEC*m elements per step, element u of every
// vector the thread loads belongs to the same row (VEC*t + u) mod m: the
// thread keeps VEC fixed-row accumulators, and the column of element u is
// (VEC*t + u)/m + VEC*q. The vector entries of the unit's columns are
// gathered into shared memory first. A tile cut into several units writes
// one partial row-sum vector per unit; the unit that arrives last adds them
// in slot order, so the result does not depend on the schedule.
// ---------------------------------------------------------------------------
template <typename T>
struct DuArgs {
  const T *panels;
  const TileDesc *tiles;
  const DuUnit *units;
  int32_t nunits;
  const Seg *segs;
  const T *xt;
  const int32_t *tmap0;
  T *y;
  int32_t *counter;
  T *part;            // partial row sums of split tiles (x2 when compensated)
  int32_t *tile_cnt;  // arrivals per tile, returned to zero by the last unit
};

template <typename T>
struct DuChunk {
  static constexpr int value = 16384 / sizeof(T);  // columns of vector entries per unit
};
constexpr int kDuSegs = 512;

template <typename T, bool COMP>
__global__ void __launch_bounds__(kThreads) du_pass_kernel(DuArgs<T> a) {
  using VT = typename Vec16<T>::type;
  constexpr int VEC = Vec16<T>::N;
  __shared__ T vals[DuChunk<T>::value];
  __shared__ Seg ssegs[kDuSegs];
  __shared__ T part[kThreads * VEC];
  __shared__ T partc[COMP ? kThreads * VEC : 1];
  __shared__ int32_t s_ticket, s_last;
  const int tid = threadIdx.x;
  for (;;) {
    if (tid == 0) s_ticket = atomicAdd(a.counter, 1);
    __syncthreads();
    const int32_t ticket = s_ticket;
    if (ticket >= a.nunits) break;
    const DuUnit U = a.units[ticket];
    const TileDesc d = a.tiles[U.tile];
    const int m = d.m, c0 = U.c0, c1 = U.c1;
    for (int s = tid; s < U.nseg; s += kThreads) ssegs[s] = a.segs[U.seg0 + s];
    __syncthreads();
    for (int c = c0 + tid; c < c1; c += kThreads) {
      int lo = 0, hi = U.nseg - 1;  // last segment with col0 <= c
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (ssegs[mid].col0 <= c)
          lo = mid;
        else
          hi = mid - 1;
      }
      vals[c - c0] = a.xt[ssegs[lo].vec_off + (c - ssegs[lo].col0)];
    }
    __syncthreads();
    int G = kThreads / m;
    if (G > 16) G = 16;
    const int g = tid / m, t = tid - g * m;
    const bool active = g < G;
    T acc[VEC], cmp[VEC];
#pragma unroll
    for (int u = 0; u < VEC; u++) acc[u] = cmp[u] = T(0);
    if (active) {
      int base[VEC];
#pragma unroll
      for (int u = 0; u < VEC; u++) base[u] = (VEC * t + u) / m;
      const VT *P = reinterpret_cast<const VT *>(a.panels + d.data_off);
      const int64_t f_lo = (static_cast<int64_t>(c0) * m) / VEC;
      const int64_t f_hi = (static_cast<int64_t>(c1) * m + VEC - 1) / VEC;
      int64_t q = f_lo > t ? (f_lo - t + m - 1) / m : 0;
      q += ((g - static_cast<int>(q % G)) % G + G) % G;
      auto consume = [&](const VT &v, int64_t qq) {
        const T *e = reinterpret_cast<const T *>(&v);
#pragma unroll
        for (int u = 0; u < VEC; u++) {
          const int c = base[u] + static_cast<int>(VEC * qq);
          if (c >= c0 && c < c1) {
            if (COMP)
              dot2_step(acc[u], cmp[u], e[u], vals[c - c0]);
            else
              acc[u] = fma_(e[u], vals[c - c0], acc[u]);
          }
        }
      };
      const int64_t step = static_cast<int64_t>(m) * G;
      int64_t f = t + m * q;
      for (; f + 3 * step < f_hi; f += 4 * step, q += 4 * G) {
        VT v0 = ld_stream(P + f), v1 = ld_stream(P + f + step);
        VT v2 = ld_stream(P + f + 2 * step), v3 = ld_stream(P + f + 3 * step);
        consume(v0, q);
        consume(v1, q + G);
        consume(v2, q + 2 * G);
        consume(v3, q + 3 * G);
      }
      for (; f < f_hi; f += step, q += G) consume(ld_stream(P + f), q);
#pragma unroll
      for (int u = 0; u < VEC; u++) {
        part[g * VEC * m + VEC * t + u] = acc[u];
        if (COMP) partc[g * VEC * m + VEC * t + u] = cmp[u];
      }
    }
    __syncthreads();
    T s = T(0), c = T(0);
    if (tid < m) {
      for (int gg = 0; gg < G; gg++)
#pragma unroll
        for (int k = 0; k < VEC; k++) {
          const int idx = gg * VEC * m + tid + k * m;
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
      if (tid < m) a.y[a.tmap0[d.row0 + tid]] = COMP ? s + c : s;
      continue;  // the ticket read at the top of the loop is behind a barrier
    }
    const int64_t pbase = U.part_off + static_cast<int64_t>(U.slot) * m + tid;
    if (tid < m) {
      if (COMP) {
        a.part[2 * pbase] = s;
        a.part[2 * pbase + 1] = c;
      } else {
        a.part[pbase] = s;
      }
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) s_last = atomicAdd(&a.tile_cnt[U.tile], 1) == U.nslots - 1;
    __syncthreads();
    if (s_last) {
      __threadfence();
      if (tid < m) {
        T ts = T(0), tc = T(0);
        for (int sl = 0; sl < U.nslots; sl++) {
          const int64_t idx = U.part_off + static_cast<int64_t>(sl) * m + tid;
          if (COMP) {
            const T p = __ldcg(a.part + 2 * idx), tt = ts + p, z = tt - ts;
            tc += ((ts - (tt - z)) + (p - z)) + __ldcg(a.part + 2 * idx + 1);
            ts = tt;
          } else {
            ts += __ldcg(a.part + idx);
          }
        }
        a.y[a.tmap0[d.row0 + tid]] = COMP ? ts + tc : ts;
      }
      if (tid == 0) a.tile_cnt[U.tile] = 0;
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
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, du_pass_kernel<double, false>, kThreads, 0);
  else if (comp)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, du_pass_kernel<float, true>, kThreads, 0);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, du_pass_kernel<float, false>, kThreads, 0);
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
  if (p.vunits && !p.warp_begin_empty) {
    v_pass_kernel<T><<<grid_v, kThreads, 0, s>>>(vdata, p.vunits, p.warp_begin, xt);
    nl++;
  }
  if (ev) cudaEventRecord(ev[2], s);
  if (p.du_variant == 1) {
    cudaError_t e = launch_du_tma(sizeof(T) == 8, COMP, p, panels, xt, y, p.grid_tma, s);
    if (e != cudaSuccess) return e;
  } else {
    DuArgs<T> a{panels, p.tiles, p.units, p.nunits, p.segs, xt, p.tmap0, y, p.counter,
                static_cast<T *>(p.part), p.tile_cnt};
    du_pass_kernel<T, COMP><<<grid_du, kThreads, 0, s>>>(a);
  }
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
// packing: FP64 row-major factors -> product layout (one warp per job)
// ---------------------------------------------------------------------------
template <typename T>
__global__ void pack_panels_kernel(const PackJob *__restrict__ jobs, int64_t njobs,
                                   const double *__restrict__ dsrc, const double *__restrict__ usrc,
                                   T *__restrict__ panels) {
  const int lane = threadIdx.x & 31;
  const int64_t w0 = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
  const int64_t nw = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
  for (int64_t w = w0; w < njobs; w += nw) {
    const PackJob j = jobs[w];
    if (j.kind == 2) continue;
    const double *src = (j.kind == 0 ? dsrc : usrc) + j.src_off;
    const int64_t total = static_cast<int64_t>(j.m) * j.ncols;
    for (int64_t e = lane; e < total; e += 32) {
      const int64_t c = e / j.m, i = e - c * j.m;
      panels[j.dst_off + e] = static_cast<T>(src[i * j.src_ld + c]);
    }
  }
}

template <typename T>
__global__ void pack_v_kernel(const VPackJob *__restrict__ jobs, int64_t njobs,
                              const double *__restrict__ vsrc, T *__restrict__ vdata) {
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

cudaError_t launch_pack_panels(bool f64, const PackJob *jobs, int64_t njobs, const double *dsrc,
                               const double *usrc, void *panels, cudaStream_t s) {
  if (njobs == 0) return cudaSuccess;
  int grid = static_cast<int>((njobs + 7) / 8);
  if (grid > 65535) grid = 65535;
  if (f64)
    pack_panels_kernel<double><<<grid, kThreads, 0, s>>>(jobs, njobs, dsrc, usrc,
                                                         static_cast<double *>(panels));
  else
    pack_panels_kernel<float><<<grid, kThreads, 0, s>>>(jobs, njobs, dsrc, usrc,
                                                        static_cast<float *>(panels));
  return cudaGetLastError();
}

cudaError_t launch_pack_v(bool f64, const VPackJob *jobs, int64_t njobs, const double *vsrc,
                          void *vdata, cudaStream_t s) {
  if (njobs == 0) return cudaSuccess;
  int grid = static_cast<int>((njobs + 7) / 8);
  if (grid > 65535) grid = 65535;
  if (f64)
    pack_v_kernel<double><<<grid, kThreads, 0, s>>>(jobs, njobs, vsrc, static_cast<double *>(vdata));
  else
    pack_v_kernel<float><<<grid, kThreads, 0, s>>>(jobs, njobs, vsrc, static_cast<float *>(vdata));
  return cudaGetLastError();
}

}  // namespace hm
