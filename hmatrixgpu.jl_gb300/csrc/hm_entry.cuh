// Matrix entries and the device kernels that evaluate them: the entry
// generators (kentry), batched ACA+ (src/aca.jl:36-106, aca_kernel), the
// dense blocks of the product layout (gen_dense_kernel) and
// sparsify_hmatrix's entries (sparsify_kernel).
//
// The header is compiled twice: into the library, with the built-in kernels,
// and at run time by NVRTC for a user's kernel (hmgpu_user_kernel_compile),
// with HM_USER_ENTRY defined and the user's
//   __device__ double hmgpu_entry(const double *x, const double *y, const double *p, int a, int b)
// (target point x, source point y, both 3 coordinates; p the kernel's
// parameters; a and b the components of a vector or tensor kernel, 0 for a
// scalar one) placed before it. It therefore includes nothing that NVRTC
// lacks; under NVRTC the integer types and the HMGPU_KERNEL_* kinds come from
// a prelude the library writes from its own definitions.
#pragma once
#ifndef __CUDACC_RTC__
#include <cstdint>

#include "../../include/hmgpu.h"
#endif
#include "hm_packjob.h"

// FP64 quiet NaN (the bits of CUDA's CUDART_NAN)
#define HM_NAN __longlong_as_double(0xfff8000000000000ULL)

namespace hm {

// ---------------------------------------------------------------------------
// matrix entries
// ---------------------------------------------------------------------------
struct KDev {
  int32_t kind;
  const double *X, *Y;  // 3 x N column-major
  const double *A;      // explicit matrix, column-major
  int64_t lda;
  const double *P;      // user kernel: its parameters (device)
  int32_t dx, dy;       // user kernel: entries per target / source point (tree dims)
};

__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }

// LinearAlgebra.generic_norm2 of a 3-vector (see hm_tree.cpp).
__device__ double norm3_dev(double a, double b, double c) {
  if (isnan(a) || isnan(b) || isnan(c)) return HM_NAN;
  double mx = fabs(a);
  if (fabs(b) > mx) mx = fabs(b);
  if (fabs(c) > mx) mx = fabs(c);
  if (mx == 0.0 || isinf(mx)) return mx;
  if (isfinite(dmul(dmul(3.0, mx), mx)) && dmul(mx, mx) != 0.0)
    return __dsqrt_rn(dadd(dadd(dmul(a, a), dmul(b, b)), dmul(c, c)));
  double qa = ddiv(fabs(a), mx), qb = ddiv(fabs(b), mx), qc = ddiv(fabs(c), mx);
  return dmul(mx, __dsqrt_rn(dadd(dadd(dmul(qa, qa), dmul(qb, qb)), dmul(qc, qc))));
}

// examples/hmatrix_vector.jl:12-28
__device__ double dip_xx(double x, double y, double z) {
  double R = dadd(dadd(dmul(x, x), dmul(y, y)), dmul(z, z));
  if (R == 0.0) return 0.0;
  double num = dsub(dsub(dmul(dmul(2.0, x), x), dmul(y, y)), dmul(z, z));
  return ddiv(ddiv(-num, dmul(dmul(R, R), __dsqrt_rn(R))), 4.0 * 3.141592653589793);
}
__device__ double dip_xy(double x, double y, double z) {
  double R = dadd(dadd(dmul(x, x), dmul(y, y)), dmul(z, z));
  if (R == 0.0) return 0.0;
  return ddiv(ddiv(dmul(dmul(-3.0, x), y), dmul(dmul(R, R), __dsqrt_rn(R))), 4.0 * 3.141592653589793);
}

// K[i, j] for 0-based original (unpermuted) indices.
__device__ double kentry(const KDev &K, int64_t i, int64_t j) {
#ifdef HM_USER_ENTRY
  // a user's kernel (kind HMGPU_KERNEL_USER): its function of the two points
  // and the two components (row i is component i mod dx of point i / dx)
  const int64_t pi = i / K.dx, pj = j / K.dy;
  return hmgpu_entry(K.X + 3 * pi, K.Y + 3 * pj, K.P, static_cast<int>(i - pi * K.dx),
                     static_cast<int>(j - pj * K.dy));
#else
  switch (K.kind) {
    case HMGPU_KERNEL_EXPLICIT:
      return K.A[i + j * K.lda];
    case HMGPU_KERNEL_LAPLACE3D:
    case HMGPU_KERNEL_YUKAWA: {
      const double *p = K.X + 3 * i, *q = K.Y + 3 * j;
      double dx = dsub(p[0], q[0]), dy = dsub(p[1], q[1]), dz = dsub(p[2], q[2]);
      double r = __dsqrt_rn(dadd(dadd(dmul(dx, dx), dmul(dy, dy)), dmul(dz, dz)));
      if (r == 0.0) return 0.0;
      if (K.kind == HMGPU_KERNEL_LAPLACE3D) return ddiv(0.07957747154594767, r);
      return ddiv(exp(-r), r);
    }
    case HMGPU_KERNEL_LOG2D: {  // test/test_hmatrix.jl:170-173
      const double *p = K.X + 3 * i, *q = K.Y + 3 * j;
      double d = norm3_dev(dsub(p[0], q[0]), dsub(p[1], q[1]), dsub(p[2], q[2]));
      return d < 1e-12 ? 1.0 : dmul(-0.5 / 3.141592653589793, log(d));
    }
    case HMGPU_KERNEL_VECTOR_R: {  // test/test_hmatrix_vector.jl:334-340
      const int64_t J = j / 3, c = j - 3 * J;
      const double *p = K.X + 3 * i, *q = K.Y + 3 * J;
      double R[3] = {dsub(p[0], q[0]), dsub(p[1], q[1]), dsub(p[2], q[2])};
      double r = norm3_dev(R[0], R[1], R[2]);
      return r < 1e-12 ? 1.0 : ddiv(R[c], dmul(r, r));
    }
    case HMGPU_KERNEL_DIPOLAR: {  // examples/hmatrix_vector.jl:46-80
      const int64_t pi_ = i / 3, a = i - 3 * pi_, pj = j / 3, b = j - 3 * pj;
      const double *p = K.X + 3 * pi_, *q = K.Y + 3 * pj;
      double x = dsub(p[0], q[0]), y = dsub(p[1], q[1]), z = dsub(p[2], q[2]);
      const int ab = a < b ? a * 3 + b : b * 3 + a;
      switch (ab) {
        case 0: return dip_xx(x, y, z);
        case 1: return dip_xy(x, y, z);
        case 2: return dip_xy(x, z, y);
        case 4: return dip_xx(y, x, z);
        case 5: return dip_xy(y, z, x);
        default: return dip_xx(z, y, x);
      }
    }
  }
  return HM_NAN;
#endif
}

// ---------------------------------------------------------------------------
// teams: one block of the matrix is worked on by a warp (NT = 32) or, for the
// large blocks, by a whole CTA (NT = kBuildThreads)
// ---------------------------------------------------------------------------
constexpr int kBuildThreads = 256;  // threads per CTA of the assembly kernels
constexpr int kBuildWarps = kBuildThreads / 32;
constexpr int64_t kTeamMinMN = 4096;  // blocks with m + n at least this get a CTA
constexpr int kCols = 8;             // columns per pass of the QR and Q applications

struct TeamScratch {  // shared memory of the CTA teams
  double v[kCols][kBuildWarps];
  int64_t key[kBuildWarps];
  int idx[kBuildWarps];
  int ticket;
};

template <int NT>
__device__ __forceinline__ int trank() {
  return NT == 32 ? static_cast<int>(threadIdx.x & 31) : static_cast<int>(threadIdx.x);
}
template <int NT>
__device__ __forceinline__ void tsync() {
  if (NT == 32)
    __syncwarp();
  else
    __syncthreads();
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Team sums of NV values per thread: each value is reduced across the warp by
// the butterfly above and then across the CTA's warps in warp order.
template <int NT, int NV>
__device__ __forceinline__ void tsum(double (&v)[NV], TeamScratch *sc) {
#pragma unroll
  for (int q = 0; q < NV; q++) v[q] = warp_sum(v[q]);
  if (NT == 32) return;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();  // earlier readers of the scratch are done
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < NV; q++) sc->v[q][w] = v[q];
  __syncthreads();
#pragma unroll
  for (int q = 0; q < NV; q++) {
    double s = sc->v[q][0];
    for (int u = 1; u < NT / 32; u++) s += sc->v[q][u];
    v[q] = s;
  }
}
template <int NT>
__device__ __forceinline__ double tsum1(double x, TeamScratch *sc) {
  double v[1] = {x};
  tsum<NT, 1>(v, sc);
  return v[0];
}

// Order of argmax_not_in_list (src/aca.jl:9-17): sortperm(rev=true) is stable,
// so the largest |value| wins, NaN above all numbers, ties to the lowest index.
// Compared as integers: the bits of |value| order the numbers, every NaN maps
// to one key above +Inf. This is a total order, so any reduction tree gives the
// same winner.
__device__ __forceinline__ int64_t am_key(double v) {
  const int64_t b = __double_as_longlong(v) & 0x7fffffffffffffffll;
  return b > 0x7ff0000000000000ll ? 0x7ff8000000000000ll : b;
}
__device__ __forceinline__ bool am_better(int64_t ka, int ia, int64_t kb, int ib) {
  if (ib < 0) return ia >= 0;
  if (ia < 0) return false;
  if (ka != kb) return ka > kb;
  return ia < ib;
}

template <int NT>
__device__ int team_argmax_unused(const double *r, const uint8_t *used, int len, TeamScratch *sc) {
  int64_t bk = 0;
  int bi = -1;
  for (int j = trank<NT>(); j < len; j += NT) {
    if (used[j]) continue;
    const int64_t kj = am_key(r[j]);
    if (am_better(kj, j, bk, bi)) {
      bk = kj;
      bi = j;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const int64_t ok = __shfl_xor_sync(0xffffffffu, bk, o);
    const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
    if (am_better(ok, oi, bk, bi)) {
      bk = ok;
      bi = oi;
    }
  }
  if (NT == 32) return bi;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) {
    sc->key[w] = bk;
    sc->idx[w] = bi;
  }
  __syncthreads();
  bk = sc->key[0];
  bi = sc->idx[0];
  for (int u = 1; u < NT / 32; u++)
    if (am_better(sc->key[u], sc->idx[u], bk, bi)) {
      bk = sc->key[u];
      bi = sc->idx[u];
    }
  return bi;
}

// Jobs of one kernel: jobs [0, nbig) by whole CTAs, then [nbig, njobs) by
// single warps; both from ticket counters tk[0] and tk[1], largest first.
template <typename Big, typename Small>
__device__ void run_teams(int nbig, int njobs, int32_t *tk, TeamScratch *sc, Big big, Small small) {
  for (;;) {
    if (threadIdx.x == 0) sc->ticket = atomicAdd(tk, 1);
    __syncthreads();
    const int j = sc->ticket;
    __syncthreads();
    if (j >= nbig) break;
    big(j);
    __syncthreads();
  }
  const int lane = threadIdx.x & 31;
  for (;;) {
    int j = 0;
    if (lane == 0) j = nbig + atomicAdd(tk + 1, 1);
    j = __shfl_sync(0xffffffffu, j, 0);
    if (j >= njobs) return;
    small(j);
  }
}

// ---------------------------------------------------------------------------
// per-block workspace
// ---------------------------------------------------------------------------
struct AcaJob {
  int32_t rs, m, cs, n;  // permuted ranges: rows rs..rs+m-1, columns cs..cs+n-1
  int64_t ws;            // workspace offset in doubles
  int32_t kcap;          // U columns / V rows available
  int32_t max_iter;      // min(m, n, max_iter)
  // continuation: k0 > 0 resumes an ACA that stopped with k0 terms when its
  // workspace (at `carry`, kcap0 terms) was full; its state is copied over
  int32_t k0, kcap0;
  int64_t carry;
};

struct AcaRes {
  int32_t k;      // ACA rank
  int32_t r;      // rank after recompression
  int32_t flags;  // 1 zero pivot, 2 workspace exhausted, 4 Jacobi not converged
  int32_t pad;
};

struct WS {
  double *U, *V, *rrow, *rcol, *tauU, *tauV, *M, *Z, *sig;
  int32_t *ord;
  uint8_t *used_r, *used_c;
};

__host__ __device__ inline int64_t ws_doubles(int64_t m, int64_t n, int64_t kcap) {
  return m * kcap + kcap * n + n + m + 2 * kcap + 2 * kcap * kcap + kcap + (kcap + 1) / 2 +
         (m + n + 7) / 8 + 4;
}

__device__ inline WS ws_view(double *base, int m, int n, int kcap) {
  WS w;
  w.U = base;
  w.V = w.U + static_cast<int64_t>(m) * kcap;
  w.rrow = w.V + static_cast<int64_t>(kcap) * n;
  w.rcol = w.rrow + n;
  w.tauU = w.rcol + m;
  w.tauV = w.tauU + kcap;
  w.M = w.tauV + kcap;
  w.Z = w.M + kcap * kcap;
  w.sig = w.Z + kcap * kcap;
  w.ord = reinterpret_cast<int32_t *>(w.sig + kcap);
  w.used_r = reinterpret_cast<uint8_t *>(w.sig + kcap + (kcap + 1) / 2);
  w.used_c = w.used_r + m;
  return w;
}

__host__ __device__ inline bool team_job(const AcaJob &j) { return int64_t{j.m} + j.n >= kTeamMinMN; }

// ---------------------------------------------------------------------------
// ACA+ (src/aca.jl:36-106), one team per block
// ---------------------------------------------------------------------------
// Residual entries K[i, j] - sum_q U[i, q] V[q, j], one term at a time
// (:43-58); E entries per thread at once so that their dependency chains
// interleave. `col` selects a column (fixed j, entries over i) or a row.
template <int NT, int E, bool COL>
__device__ __forceinline__ void residual(const KDev &K, const int32_t *trow, const int32_t *scol, const WS &w,
                                         int m, int n, int k, int fixed, double *out) {
  const int len = COL ? m : n;
  const int64_t fixed_ix = COL ? scol[fixed] : trow[fixed];
  for (int p0 = trank<NT>(); p0 < len; p0 += E * NT) {
    double v[E];
    int pp[E];
#pragma unroll
    for (int e = 0; e < E; e++) {
      pp[e] = min(p0 + e * NT, len - 1);
      v[e] = COL ? kentry(K, trow[pp[e]], fixed_ix) : kentry(K, fixed_ix, scol[pp[e]]);
    }
    for (int q = 0; q < k; q++) {
      if (COL) {
        const double vq = w.V[static_cast<int64_t>(q) * n + fixed];
        const double *uq = w.U + static_cast<int64_t>(q) * m;
#pragma unroll
        for (int e = 0; e < E; e++) v[e] = dsub(v[e], dmul(uq[pp[e]], vq));
      } else {
        const double uq = w.U[fixed + static_cast<int64_t>(q) * m];
        const double *vq = w.V + static_cast<int64_t>(q) * n;
#pragma unroll
        for (int e = 0; e < E; e++) v[e] = dsub(v[e], dmul(uq, vq[pp[e]]));
      }
    }
#pragma unroll
    for (int e = 0; e < E; e++)
      if (p0 + e * NT < len) out[p0 + e * NT] = v[e];
  }
}

template <int NT, bool COL>
__device__ void residual_any(const KDev &K, const int32_t *trow, const int32_t *scol, const WS &w, int m, int n,
                             int k, int fixed) {
  const int len = COL ? m : n;
  double *out = COL ? w.rcol : w.rrow;
  if (len >= 4 * NT)
    residual<NT, 4, COL>(K, trow, scol, w, m, n, k, fixed, out);
  else if (len > NT)
    residual<NT, 2, COL>(K, trow, scol, w, m, n, k, fixed, out);
  else
    residual<NT, 1, COL>(K, trow, scol, w, m, n, k, fixed, out);
  tsync<NT>();
}

template <int NT>
__device__ void aca_team(const KDev &K, const int32_t *tmap0, const int32_t *smap0, const AcaJob &jb,
                         double eps, double *wsbase, AcaRes *res, TeamScratch *sc) {
  const int t = trank<NT>();
  const int m = jb.m, n = jb.n, kcap = jb.kcap;
  WS w = ws_view(wsbase + jb.ws, m, n, kcap);
  const int32_t *trow = tmap0 + jb.rs, *scol = smap0 + jb.cs;
  if (jb.k0 > 0) {
    // a continuation: the first k0 terms, the last residual row and column
    // and the used pivots, exactly as the stopped run left them, so the run
    // goes on as if its workspace had been large enough
    const WS o = ws_view(wsbase + jb.carry, m, n, jb.kcap0);
    for (int64_t e = t; e < static_cast<int64_t>(m) * jb.k0; e += NT) w.U[e] = o.U[e];
    for (int64_t e = t; e < static_cast<int64_t>(jb.k0) * n; e += NT) w.V[e] = o.V[e];
    for (int j = t; j < n; j += NT) {
      w.rrow[j] = o.rrow[j];
      w.used_c[j] = o.used_c[j];
    }
    for (int i = t; i < m; i += NT) {
      w.rcol[i] = o.rcol[i];
      w.used_r[i] = o.used_r[i];
    }
  } else {
    for (int j = t; j < n; j += NT) {
      w.rrow[j] = 0.0;
      w.used_c[j] = 0;
    }
    for (int i = t; i < m; i += NT) {
      w.rcol[i] = 0.0;
      w.used_r[i] = 0;
    }
  }
  tsync<NT>();
  int k = jb.k0 > 0 ? jb.k0 : 0, flags = 0;
  for (int it = k + 1; it <= jb.max_iter; it++) {
    int rp = 0, cp = 0;
    if (it > 1) {  // :72-73
      cp = team_argmax_unused<NT>(w.rrow, w.used_c, n, sc);
      rp = team_argmax_unused<NT>(w.rcol, w.used_r, m, sc);
    }
    const double cval = fabs(w.rrow[cp]), rval = fabs(w.rcol[rp]);
    if (rval > cval) {  // :79-82
      residual_any<NT, false>(K, trow, scol, w, m, n, k, rp);
      cp = team_argmax_unused<NT>(w.rrow, w.used_c, n, sc);
      residual_any<NT, true>(K, trow, scol, w, m, n, k, cp);
    } else {  // :83-87
      residual_any<NT, true>(K, trow, scol, w, m, n, k, cp);
      rp = team_argmax_unused<NT>(w.rcol, w.used_r, m, sc);
      residual_any<NT, false>(K, trow, scol, w, m, n, k, rp);
    }
    const double piv = w.rrow[cp];
    if (piv == 0.0 || !isfinite(piv)) {  // the reference would divide by zero here
      flags |= 1;
      break;
    }
    double s2[2] = {0.0, 0.0};  // sum(v.^2), sum(u.^2)
    for (int j = t; j < n; j += NT) {  // v_k = row / row[cp] (:92)
      double v = ddiv(w.rrow[j], piv);
      w.V[static_cast<int64_t>(k) * n + j] = v;
      s2[0] = dadd(s2[0], dmul(v, v));
    }
    for (int i = t; i < m; i += NT) {  // u_k = col (:93)
      double u = w.rcol[i];
      w.U[i + static_cast<int64_t>(k) * m] = u;
      s2[1] = dadd(s2[1], dmul(u, u));
    }
    if (t == 0) {
      w.used_r[rp] = 1;
      w.used_c[cp] = 1;
    }
    k++;
    tsum<NT, 2>(s2, sc);
    tsync<NT>();
    if (sqrt(s2[1] * s2[0]) < eps) break;  // :95-99
    if (k == kcap && it < jb.max_iter) {
      flags |= 2;
      break;
    }
  }
  if (t == 0) {
    res->k = k;
    res->flags = flags;
  }
}

__global__ void __launch_bounds__(kBuildThreads, 3) aca_kernel(KDev K, const int32_t *__restrict__ tmap0,
                                                            const int32_t *__restrict__ smap0,
                                                            const AcaJob *__restrict__ jobs, int32_t nbig,
                                                            int32_t njobs, double eps, double *ws, AcaRes *res,
                                                            int32_t *ticket) {
  __shared__ TeamScratch sc;
  run_teams(
      nbig, njobs, ticket, &sc,
      [&](int j) { aca_team<kBuildThreads>(K, tmap0, smap0, jobs[j], eps, ws, res + j, &sc); },
      [&](int j) { aca_team<32>(K, tmap0, smap0, jobs[j], eps, ws, res + j, &sc); });
}

// Dense blocks generated straight into the product layout (kind-2 pack jobs).
template <typename T>
__global__ void gen_dense_kernel(KDev K, const int32_t *__restrict__ tmap0,
                                 const int32_t *__restrict__ smap0, const PackJob *__restrict__ jobs,
                                 int64_t njobs, T *__restrict__ panels) {
  const int lane = threadIdx.x & 31;
  const int64_t w0 = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
  const int64_t nw = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
  for (int64_t wi = w0; wi < njobs; wi += nw) {
    const PackJob j = jobs[wi];
    if (j.kind != 2) continue;
    for (int i = 0; i < j.m; i++) {  // rows of the row-major tile panel
      const int64_t ti = tmap0[j.row0 + i];
      T *dst = panels + j.dst_off + static_cast<int64_t>(i) * j.dst_ld;
      for (int c = lane; c < j.ncols; c += 32) dst[c] = static_cast<T>(kentry(K, ti, smap0[j.col0 + c]));
    }
  }
}

// sparsify_hmatrix: block j's entries K[tmap[row0 + i], smap[col0 + c]] at
// out[off + i n + c] (row by row, as the reference pushes them); a warp per block.
struct SpJob {
  int32_t row0, m, col0, n;
  int64_t off;
};

__global__ void sparsify_kernel(KDev K, const int32_t *__restrict__ tmap0, const int32_t *__restrict__ smap0,
                                const SpJob *__restrict__ jobs, int64_t njobs, double *__restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t w0 = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
  const int64_t nw = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
  for (int64_t wi = w0; wi < njobs; wi += nw) {
    const SpJob j = jobs[wi];
    for (int i = 0; i < j.m; i++) {
      const int64_t ti = tmap0[j.row0 + i];
      double *dst = out + j.off + static_cast<int64_t>(i) * j.n;
      for (int c = lane; c < j.n; c += 32) dst[c] = kentry(K, ti, smap0[j.col0 + c]);
    }
  }
}

}  // namespace hm
