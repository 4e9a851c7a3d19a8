// On-device H-matrix assembly: entry generation, batched ACA+ and batched
// QR + SVD recompression (all FP64), replacing the reference's host loop in
// build_matrices (src/hmatrix.jl:170-217), ACA_plus (src/aca.jl:36-106) and
// SVD_recompress (src/aca.jl:123-143).
//
// A warp owns one admissible block at a time, or a whole CTA for the large
// blocks; teams take blocks from ticket counters, largest first. The Jacobi
// SVD of the small k x k core runs one block per thread.  The ACA follows the reference's pivot and
// stopping rules exactly; matrix entries and residual updates use explicitly
// rounded FP64 operations in the reference's order, so for kernels built from
// +,-,*,/ and sqrt the pivots match the oracle bit for bit.  The only reduction
// whose order differs from the reference is the step-size norm
// sqrt(sum(u.^2) * sum(v.^2)) (Julia sums with SIMD reassociation).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <memory>
#include <type_traits>

#include "hm_api.h"
#include "hm_entry.cuh"
#include "hm_user.h"

namespace hm {

// ---------------------------------------------------------------------------
// QR + SVD recompression (src/aca.jl:123-143)
// ---------------------------------------------------------------------------
// Applies the reflector I - tau v v' (v = [1; x[1..len)]) to NC columns:
// entry i of column q at y0[i*si + q*scs]. The NC dot products are reduced
// together, each exactly as a single one would be.
template <int NT, int NC>
__device__ __forceinline__ void reflect_cols(const double *x, int len, double tau, double *y0, int64_t si,
                                             int64_t scs, TeamScratch *sc) {
  const int t = trank<NT>();
  double d[NC];
#pragma unroll
  for (int q = 0; q < NC; q++) d[q] = 0.0;
  for (int i = 1 + t; i < len; i += NT) {
    const double xi = x[i];
#pragma unroll
    for (int q = 0; q < NC; q++) d[q] += xi * y0[i * si + q * scs];
  }
  tsum<NT, NC>(d, sc);
  double wv[NC];
#pragma unroll
  for (int q = 0; q < NC; q++) wv[q] = (d[q] + y0[q * scs]) * tau;
  for (int i = 1 + t; i < len; i += NT) {
    const double xi = x[i];
#pragma unroll
    for (int q = 0; q < NC; q++) y0[i * si + q * scs] -= wv[q] * xi;
  }
  tsync<NT>();
  if (t == 0)
#pragma unroll
    for (int q = 0; q < NC; q++) y0[q * scs] -= wv[q];
  tsync<NT>();
}

template <int NT>
__device__ void reflect_any(int nc, const double *x, int len, double tau, double *y0, int64_t si, int64_t scs,
                            TeamScratch *sc) {
  switch (nc) {
    case 1: reflect_cols<NT, 1>(x, len, tau, y0, si, scs, sc); break;
    case 2: reflect_cols<NT, 2>(x, len, tau, y0, si, scs, sc); break;
    case 3: reflect_cols<NT, 3>(x, len, tau, y0, si, scs, sc); break;
    case 4: reflect_cols<NT, 4>(x, len, tau, y0, si, scs, sc); break;
    case 5: reflect_cols<NT, 5>(x, len, tau, y0, si, scs, sc); break;
    case 6: reflect_cols<NT, 6>(x, len, tau, y0, si, scs, sc); break;
    case 7: reflect_cols<NT, 7>(x, len, tau, y0, si, scs, sc); break;
    default: reflect_cols<NT, 8>(x, len, tau, y0, si, scs, sc); break;
  }
}

// Householder QR (LAPACK dgeqr2 conventions) of A (rows x cols, column-major,
// leading dimension ld), in place; tau[j] per reflector. The trailing columns
// are updated kCols at a time (their dot products reduced together).
template <int NT>
__device__ void team_qr(double *A, int64_t ld, int rows, int cols, double *tau, TeamScratch *sc) {
  const int t = trank<NT>();
  for (int j = 0; j < cols; j++) {
    double *x = A + j + j * ld;
    const int len = rows - j;
    double s = 0.0;
    for (int i = 1 + t; i < len; i += NT) s += x[i] * x[i];
    const double xn = sqrt(tsum1<NT>(s, sc));
    const double alpha = x[0];
    double tj = 0.0;
    if (xn != 0.0) {
      const double beta = -copysign(sqrt(alpha * alpha + xn * xn), alpha);
      tj = (beta - alpha) / beta;
      const double scl = 1.0 / (alpha - beta);
      for (int i = 1 + t; i < len; i += NT) x[i] *= scl;
      tsync<NT>();
      if (t == 0) x[0] = beta;
    }
    if (t == 0) tau[j] = tj;
    tsync<NT>();
    for (int c0 = j + 1; c0 < cols; c0 += kCols)
      reflect_any<NT>(min(kCols, cols - c0), x, len, tj, A + j + c0 * ld, 1, ld, sc);
  }
}

// QR of both factors and M = RU * RV' (k x k column-major), Z = I.
template <int NT>
__device__ void qr_team(const AcaJob &jb, const AcaRes &rs, int svd, double *ws, TeamScratch *sc) {
  const int k = rs.k;
  if (!svd || k == 0) return;
  const int t = trank<NT>();
  WS w = ws_view(ws + jb.ws, jb.m, jb.n, jb.kcap);
  const int m = jb.m, n = jb.n;
  team_qr<NT>(w.U, m, m, k, w.tauU, sc);  // qr(U) (:125)
  team_qr<NT>(w.V, n, n, k, w.tauV, sc);  // qr(V') (:126): V row-major k x n == V' column-major
  for (int e = t; e < k * k; e += NT) {   // M = RU * RV' (:129)
    const int r = e % k, c = e / k;
    double s = 0.0;
    for (int q = max(r, c); q < k; q++) s += w.U[r + static_cast<int64_t>(q) * m] * w.V[c + static_cast<int64_t>(q) * n];
    w.M[r + c * k] = s;
    w.Z[r + c * k] = r == c ? 1.0 : 0.0;
  }
  tsync<NT>();
}

__global__ void __launch_bounds__(kBuildThreads) qr_kernel(const AcaJob *__restrict__ jobs, int32_t nbig,
                                                           int32_t njobs, int svd, double *ws,
                                                           const AcaRes *res, int32_t *ticket) {
  __shared__ TeamScratch sc;
  run_teams(
      nbig, njobs, ticket, &sc, [&](int j) { qr_team<kBuildThreads>(jobs[j], res[j], svd, ws, &sc); },
      [&](int j) { qr_team<32>(jobs[j], res[j], svd, ws, &sc); });
}

// One-sided (Hestenes) Jacobi SVD of M, one thread per block: columns of M
// rotated into W*Sigma, Z collects the rotations; then the singular values in
// decreasing order and the truncation rank from the tail norms (:130-136).
__global__ void __launch_bounds__(kBuildThreads) jacobi_kernel(const AcaJob *__restrict__ jobs, int32_t njobs,
                                                               double eps, int svd, double *ws, AcaRes *res) {
  const int jj = blockIdx.x * blockDim.x + threadIdx.x;
  if (jj >= njobs) return;
  const int k = res[jj].k;
  if (!svd || k == 0) {
    res[jj].r = k;
    return;
  }
  const AcaJob jb = jobs[jj];
  WS w = ws_view(ws + jb.ws, jb.m, jb.n, jb.kcap);
  double *M = w.M, *Z = w.Z;
  int converged = 0;
  for (int sweep = 0; sweep < 80 && !converged; sweep++) {
    int rotated = 0;
    for (int p = 0; p < k - 1; p++)
      for (int q = p + 1; q < k; q++) {
        double *mp = M + p * k, *mq = M + q * k;
        double a = 0.0, b = 0.0, g = 0.0;
        for (int i = 0; i < k; i++) {
          const double u = mp[i], v = mq[i];
          a += u * u;
          b += v * v;
          g += u * v;
        }
        if (g == 0.0 || fabs(g) <= 1e-15 * sqrt(a * b)) continue;
        rotated = 1;
        const double zeta = (b - a) / (2.0 * g);
        const double tt = copysign(1.0, zeta) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
        const double c = 1.0 / sqrt(1.0 + tt * tt), s = c * tt;
        double *zp = Z + p * k, *zq = Z + q * k;
        for (int i = 0; i < k; i++) {
          const double u = mp[i], v = mq[i];
          mp[i] = c * u - s * v;
          mq[i] = s * u + c * v;
          const double zu = zp[i], zv = zq[i];
          zp[i] = c * zu - s * zv;
          zq[i] = s * zu + c * zv;
        }
      }
    converged = !rotated;
  }
  for (int j = 0; j < k; j++) {
    double s = 0.0;
    for (int i = 0; i < k; i++) s += M[i + j * k] * M[i + j * k];
    w.sig[j] = sqrt(s);
    w.ord[j] = j;
  }
  for (int i = 1; i < k; i++) {  // stable, decreasing sigma
    const int v = w.ord[i];
    int j = i - 1;
    while (j >= 0 && w.sig[w.ord[j]] < w.sig[v]) {
      w.ord[j + 1] = w.ord[j];
      j--;
    }
    w.ord[j + 1] = v;
  }
  // tail norms accumulated from the smallest singular value (:132-136); they
  // grow as i falls, so the first i with tail < eps is where the downward scan
  // last sees tail < eps.
  int r = k;
  double acc = 0.0;
  for (int i = k - 1; i >= 0; i--) {
    acc += w.sig[w.ord[i]] * w.sig[w.ord[i]];
    if (sqrt(acc) < eps)
      r = i;
    else
      break;
  }
  res[jj].r = r;
  if (!converged) res[jj].flags |= 4;
}

// out(i, c) for c < r := (Q [C(:, ord[c]); 0])(i) with Q's k reflectors in QR
// (rows x k, ld) and tau; C is k x k; out(i, c) lives at out[i*si + c*scs].
// kCols output columns per pass.
template <int NT>
__device__ void team_apply_q(const double *QR, int64_t ld, int rows, int k, const double *tau, const double *C,
                             const int32_t *ord, int r, double *out, int64_t si, int64_t scs, TeamScratch *sc) {
  const int t = trank<NT>();
  for (int c0 = 0; c0 < r; c0 += kCols) {
    const int nc = min(kCols, r - c0);
    double *o = out + c0 * scs;
    for (int i = t; i < rows; i += NT)
#pragma unroll
      for (int q = 0; q < kCols; q++)
        if (q < nc) o[i * si + q * scs] = i < k ? C[i + ord[c0 + q] * k] : 0.0;
    tsync<NT>();
    for (int j = k - 1; j >= 0; j--)
      reflect_any<NT>(nc, QR + j + j * ld, rows - j, tau[j], o + j * si, si, scs, sc);
  }
}

// Final factors of one block, row-major: U' (m x r) at uo, V' (r x n) at vo.
template <int NT>
__device__ void form_team(const AcaJob &jb, const AcaRes &rs, int svd, double *ws, int64_t uo, int64_t vo,
                          double *ustore, double *vstore, TeamScratch *sc) {
  if (uo < 0) return;  // block stored dense
  const int t = trank<NT>();
  const int m = jb.m, n = jb.n, k = rs.k, r = rs.r;
  WS w = ws_view(ws + jb.ws, m, n, jb.kcap);
  double *U = ustore + uo, *V = vstore + vo;
  if (!svd) {
    for (int64_t e = t; e < static_cast<int64_t>(m) * k; e += NT) {
      const int64_t i = e / k, q = e - i * k;
      U[e] = w.U[i + q * m];
    }
    for (int64_t e = t; e < static_cast<int64_t>(k) * n; e += NT) V[e] = w.V[e];
    return;
  }
  team_apply_q<NT>(w.U, m, m, k, w.tauU, w.M, w.ord, r, U, r, 1, sc);  // U' = QU * (W_r Sigma_r) (:139)
  team_apply_q<NT>(w.V, n, n, k, w.tauV, w.Z, w.ord, r, V, 1, n, sc);  // V' = Z_r' * QV' (:140)
}

__global__ void __launch_bounds__(kBuildThreads) form_kernel(const AcaJob *__restrict__ jobs, int32_t nbig,
                                                             int32_t njobs, int svd, double *ws,
                                                             const AcaRes *res, const int64_t *uo,
                                                             const int64_t *vo, double *ustore, double *vstore,
                                                             int32_t *ticket) {
  __shared__ TeamScratch sc;
  run_teams(
      nbig, njobs, ticket, &sc,
      [&](int j) { form_team<kBuildThreads>(jobs[j], res[j], svd, ws, uo[j], vo[j], ustore, vstore, &sc); },
      [&](int j) { form_team<32>(jobs[j], res[j], svd, ws, uo[j], vo[j], ustore, vstore, &sc); });
}

// The entry kernels run from the library's own build, or, for a user's
// kernel, from the module compiled with the user's entry function (the same
// source, the same argument lists).
static cudaError_t launch_aca(const UserFns *uf, int grid, KDev K, const int32_t *tmap0, const int32_t *smap0,
                              const AcaJob *jobs, int32_t nbig, int32_t njobs, double eps, double *ws, AcaRes *res,
                              int32_t *ticket) {
  if (!uf) {
    aca_kernel<<<grid, kBuildThreads>>>(K, tmap0, smap0, jobs, nbig, njobs, eps, ws, res, ticket);
    return cudaGetLastError();
  }
  void *args[] = {&K, &tmap0, &smap0, &jobs, &nbig, &njobs, &eps, &ws, &res, &ticket};
  return launch_user(uf->aca, grid, kBuildThreads, args);
}

template <typename T>
static cudaError_t launch_gen_dense(const UserFns *uf, int grid, KDev K, const int32_t *tmap0, const int32_t *smap0,
                                    const PackJob *jobs, int64_t njobs, T *panels) {
  if (!uf) {
    gen_dense_kernel<T><<<grid, 256>>>(K, tmap0, smap0, jobs, njobs, panels);
    return cudaGetLastError();
  }
  void *args[] = {&K, &tmap0, &smap0, &jobs, &njobs, &panels};
  return launch_user(std::is_same<T, double>::value ? uf->gen_d : uf->gen_f, grid, 256, args);
}

static cudaError_t launch_sparsify(const UserFns *uf, int grid, KDev K, const int32_t *tmap0, const int32_t *smap0,
                                   const SpJob *jobs, int64_t njobs, double *out) {
  if (!uf) {
    sparsify_kernel<<<grid, 256>>>(K, tmap0, smap0, jobs, njobs, out);
    return cudaGetLastError();
  }
  void *args[] = {&K, &tmap0, &smap0, &jobs, &njobs, &out};
  return launch_user(uf->sparsify, grid, 256, args);
}

struct KernelGen : DenseGenerator {
  KDev K;
  const UserFns *uf = nullptr;
  int generate(HMatrix &H, const PackJob *djobs, int64_t njobs) override {
    if (njobs == 0) return HMGPU_OK;
    int grid = static_cast<int>(std::min<int64_t>((njobs + 7) / 8, 65535));
    cudaError_t e;
    if (H.opt.precision == HMGPU_F64)
      e = launch_gen_dense<double>(uf, grid, K, H.dp.tmap0, H.dp.smap0, djobs, njobs,
                                   static_cast<double *>(H.panels));
    else
      e = launch_gen_dense<float>(uf, grid, K, H.dp.tmap0, H.dp.smap0, djobs, njobs,
                                  static_cast<float *>(H.panels));
    return e == cudaSuccess ? HMGPU_OK : cuda_fail(e, "dense generation");
  }
};

// Gather of the kept blocks' factors from the per-batch buffers into one
// store: one warp per copy.
template <typename E>
struct CopyJob {
  const E *src;
  E *dst;
  int64_t n;
};

// FP64 factors of one batch rounded to FP32 (FP32 storage keeps no FP64 copy).
__global__ void __launch_bounds__(256) round_kernel(const double *__restrict__ src, float *__restrict__ dst,
                                                   int64_t n) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    dst[i] = static_cast<float>(src[i]);
}

template <typename E>
__global__ void __launch_bounds__(256) gather_kernel(const CopyJob<E> *__restrict__ jobs, int64_t njobs) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
  for (int64_t w = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; w < njobs; w += warps) {
    const CopyJob<E> j = jobs[w];
    for (int64_t i = lane; i < j.n; i += 32) j.dst[i] = j.src[i];
  }
}

// ---------------------------------------------------------------------------
// host orchestration
// ---------------------------------------------------------------------------
struct DevBuf {
  void *p = nullptr;
  size_t cap = 0;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
  int alloc(size_t bytes) {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    cudaError_t e = cudaMalloc(&p, bytes ? bytes : 16);
    if (e != cudaSuccess) {
      cudaGetLastError();
      p = nullptr;
      return fail(HMGPU_ERR_NOMEM, "cudaMalloc of " + std::to_string(bytes) + " bytes failed");
    }
    cap = bytes ? bytes : 16;
    return HMGPU_OK;
  }
  // Keeps the current allocation when it is large enough.
  int reserve(size_t bytes) { return p && cap >= bytes ? HMGPU_OK : alloc(bytes); }
  template <typename V>
  V *as() const {
    return static_cast<V *>(p);
  }
};

// Resident CTAs of a persistent assembly kernel on the whole device.
template <typename F>
static int persistent_grid(F kernel) {
  int dev = 0, sms = 0, occ = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, kBuildThreads, 0);
  return std::max(1, sms) * std::max(1, occ);
}

// Runs ACA (+ recompression) on `jobs` (workspace offsets filled here) in
// batches that fit `budget` doubles. Returns per-job results; the caller picks
// which blocks to keep and receives row-major factors through `emit`.
struct BatchOut {
  std::vector<AcaRes> res;
};

struct Compressor {
  KDev K;
  const UserFns *uf = nullptr;  // a user's kernel: its compiled entry kernels
  const int32_t *tmap0, *smap0;
  double eps_aca, eps_svd;
  int svd;
  int64_t budget;  // doubles of workspace per batch
  int grid_aca = 1, grid_qr = 1, grid_form = 1;
  // continuation: the workspace holds a quarter more than a batch fills, and a
  // block that fills its own goes on there, from its state, in the same batch
  bool resume = false;
  int64_t batches = 0, ws_bytes = 0, continued = 0;  // statistics of all run() calls

  // Processes jobs[idx] for idx in `sel`, writing results into res (indexed like jobs).
  // keep(jj, k, r) -> bool decides whether low-rank factors are written; factors
  // of kept blocks go to (ustore + uoff[jj], vstore + voff[jj]) allocated by `place`.
  // The blocks of a batch that filled their workspace before converging go
  // on in the free part of the workspace, from the state they stopped in,
  // with room for half as many terms again (at least 8 more, at most
  // min(m, n)), round after round while blocks still fill up and room is
  // left; the batch's jobs and results on the device are updated to the
  // continued runs. Blocks that do not fit are left to the restart after all
  // batches.
  int continue_full(std::vector<AcaJob> &batch, int64_t used, DevBuf &ws, DevBuf &djobs, DevBuf &dres, DevBuf &dcj,
                    DevBuf &dcr, int32_t *tk) {
    const int nb = static_cast<int>(batch.size());
    std::vector<AcaRes> hr(nb);
    cudaError_t e = cudaMemcpy(hr.data(), dres.p, nb * sizeof(AcaRes), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "ACA kernel");
    const int64_t room = static_cast<int64_t>(ws.cap / sizeof(double));
    int64_t extra = used;
    bool changed = false;
    for (;;) {
      std::vector<AcaJob> cj;
      std::vector<int> cidx;
      for (int b = 0; b < nb; b++) {  // team jobs stay first: the batch lists them first
        if (!(hr[b].flags & 2)) continue;
        AcaJob j2 = batch[b];
        const int32_t cap2 = std::min(j2.max_iter, std::max(j2.kcap + 8, j2.kcap + j2.kcap / 2));
        const int64_t need = ws_doubles(j2.m, j2.n, cap2);
        if (extra + need > room) continue;
        j2.k0 = hr[b].k;
        j2.kcap0 = j2.kcap;
        j2.carry = j2.ws;
        j2.kcap = cap2;
        j2.ws = extra;
        extra += need;
        cj.push_back(j2);
        cidx.push_back(b);
      }
      if (cj.empty()) break;
      const int nc = static_cast<int>(cj.size());
      int nbig = 0;
      while (nbig < nc && team_job(cj[nbig])) nbig++;
      int rc;
      if ((rc = dcj.reserve(nc * sizeof(AcaJob))) || (rc = dcr.reserve(nc * sizeof(AcaRes)))) return rc;
      cudaMemcpy(dcj.p, cj.data(), nc * sizeof(AcaJob), cudaMemcpyHostToDevice);
      cudaMemset(dcr.p, 0, nc * sizeof(AcaRes));
      cudaMemset(tk, 0, 2 * sizeof(int32_t));
      if ((e = launch_aca(uf, grid_aca, K, tmap0, smap0, dcj.as<AcaJob>(), nbig, nc, eps_aca, ws.as<double>(),
                          dcr.as<AcaRes>(), tk)) != cudaSuccess)
        return cuda_fail(e, "ACA continuation launch");
      std::vector<AcaRes> cr(nc);
      e = cudaMemcpy(cr.data(), dcr.p, nc * sizeof(AcaRes), cudaMemcpyDeviceToHost);
      if (e != cudaSuccess) return cuda_fail(e, "ACA continuation");
      for (int q = 0; q < nc; q++) {
        batch[cidx[q]] = cj[q];
        hr[cidx[q]] = cr[q];
      }
      continued += nc;
      changed = true;
    }
    if (!changed) return HMGPU_OK;
    cudaMemcpy(djobs.p, batch.data(), nb * sizeof(AcaJob), cudaMemcpyHostToDevice);
    cudaMemcpy(dres.p, hr.data(), nb * sizeof(AcaRes), cudaMemcpyHostToDevice);
    ws_bytes += (extra - used) * static_cast<int64_t>(sizeof(double));
    return HMGPU_OK;
  }

  template <typename Keep, typename Place, typename After>
  int run(std::vector<AcaJob> &jobs, std::vector<AcaRes> &res, const std::vector<int> &sel,
          Keep keep, Place place, After after) {
    size_t pos = 0;
    DevBuf ws, djobs, dres, dtick, duo, dvo, dcj, dcr;
    if (int rc = dtick.alloc(8 * sizeof(int32_t))) return rc;
    const int64_t fill = budget;
    if (resume)  // a quarter more than the batches fill, for the continued blocks
      if (int rc = ws.reserve((budget + budget / 4) * sizeof(double))) return rc;
    while (pos < sel.size()) {
      std::vector<AcaJob> batch;
      std::vector<int> ids;
      int64_t used = 0;
      while (pos < sel.size()) {
        AcaJob jb = jobs[sel[pos]];
        int64_t need = ws_doubles(jb.m, jb.n, jb.kcap);
        if (!batch.empty() && used + need > fill) break;
        jb.ws = used;
        used += need;
        batch.push_back(jb);
        ids.push_back(sel[pos]);
        pos++;
      }
      // blocks worked on by whole CTAs first (the kernels take them before the rest)
      {
        std::vector<AcaJob> b2;
        std::vector<int> i2;
        b2.reserve(batch.size());
        i2.reserve(ids.size());
        for (int pass = 0; pass < 2; pass++)
          for (size_t q = 0; q < batch.size(); q++)
            if (team_job(batch[q]) == (pass == 0)) {
              b2.push_back(batch[q]);
              i2.push_back(ids[q]);
            }
        batch.swap(b2);
        ids.swap(i2);
      }
      const int nb = static_cast<int>(batch.size());
      int nbig = 0;
      while (nbig < nb && team_job(batch[nbig])) nbig++;
      batches++;
      ws_bytes += used * static_cast<int64_t>(sizeof(double));
      int rc;
      if ((rc = ws.reserve(used * sizeof(double))) || (rc = djobs.reserve(nb * sizeof(AcaJob))) ||
          (rc = dres.reserve(nb * sizeof(AcaRes))))
        return rc;
      cudaMemcpy(djobs.p, batch.data(), nb * sizeof(AcaJob), cudaMemcpyHostToDevice);
      cudaMemset(dres.p, 0, nb * sizeof(AcaRes));
      cudaMemset(dtick.p, 0, 8 * sizeof(int32_t));
      int32_t *tk = dtick.as<int32_t>();
      if (cudaError_t le = launch_aca(uf, grid_aca, K, tmap0, smap0, djobs.as<AcaJob>(), nbig, nb, eps_aca,
                                      ws.as<double>(), dres.as<AcaRes>(), tk))
        return cuda_fail(le, "ACA launch");
      if (resume && (rc = continue_full(batch, used, ws, djobs, dres, dcj, dcr, tk + 6))) return rc;
      qr_kernel<<<grid_qr, kBuildThreads>>>(djobs.as<AcaJob>(), nbig, nb, svd, ws.as<double>(), dres.as<AcaRes>(),
                                         tk + 2);
      jacobi_kernel<<<(nb + kBuildThreads - 1) / kBuildThreads, kBuildThreads>>>(
          djobs.as<AcaJob>(), nb, eps_svd, svd, ws.as<double>(), dres.as<AcaRes>());
      std::vector<AcaRes> hr(nb);
      cudaError_t e = cudaMemcpy(hr.data(), dres.p, nb * sizeof(AcaRes), cudaMemcpyDeviceToHost);
      if (e != cudaSuccess) return cuda_fail(e, "ACA / recompression kernels");
      std::vector<int64_t> uo(nb, -1), vo(nb, -1);
      int64_t ulen = 0, vlen = 0;
      for (int b = 0; b < nb; b++) {
        res[ids[b]] = hr[b];
        if ((hr[b].flags & 2) == 0 && keep(ids[b], hr[b].k, hr[b].r)) {
          uo[b] = ulen;
          vo[b] = vlen;
          ulen += static_cast<int64_t>(batch[b].m) * hr[b].r;
          vlen += static_cast<int64_t>(batch[b].n) * hr[b].r;
        }
      }
      double *ust = nullptr, *vst = nullptr;
      if ((rc = place(ids, uo, vo, ulen, vlen, &ust, &vst))) return rc;
      if ((rc = duo.reserve(nb * sizeof(int64_t))) || (rc = dvo.reserve(nb * sizeof(int64_t)))) return rc;
      cudaMemcpy(duo.p, uo.data(), nb * sizeof(int64_t), cudaMemcpyHostToDevice);
      cudaMemcpy(dvo.p, vo.data(), nb * sizeof(int64_t), cudaMemcpyHostToDevice);
      form_kernel<<<grid_form, kBuildThreads>>>(djobs.as<AcaJob>(), nbig, nb, svd, ws.as<double>(), dres.as<AcaRes>(),
                                           duo.as<int64_t>(), dvo.as<int64_t>(), ust, vst, tk + 4);
      e = cudaDeviceSynchronize();
      if (e != cudaSuccess) return cuda_fail(e, "factor formation");
      if ((rc = after())) return rc;
    }
    return HMGPU_OK;
  }
};

static int upload_coords(const double *src, int64_t npts, DevBuf &dst) {
  if (int rc = dst.alloc(static_cast<size_t>(3 * npts) * sizeof(double))) return rc;
  cudaError_t e = cudaMemcpy(dst.p, src, 3 * npts * sizeof(double), cudaMemcpyDefault);
  return e == cudaSuccess ? HMGPU_OK : cuda_fail(e, "copying coordinates");
}

// size(K) must match the trees (the reference indexes K through the trees' maps).
static int check_kernel(const hmgpu_kernel *kd, int64_t m, int64_t n) {
  int64_t km = 0, kn = 0;
  switch (kd->kind) {
    case HMGPU_KERNEL_EXPLICIT:
      if (!kd->A || kd->lda < m) return fail(HMGPU_ERR_INVALID, "explicit kernel needs A with lda >= rows");
      km = m;
      kn = n;
      break;
    case HMGPU_KERNEL_LAPLACE3D:
    case HMGPU_KERNEL_YUKAWA:
    case HMGPU_KERNEL_LOG2D:
      km = kd->nX;
      kn = kd->nY;
      break;
    case HMGPU_KERNEL_USER:  // dims entries per point, as the trees have them
      if (kd->nX <= 0 || kd->nY <= 0 || m % kd->nX != 0 || n % kd->nY != 0)
        return fail(HMGPU_ERR_INVALID, "a user kernel's rows and columns must be whole multiples of its points");
      km = m;
      kn = n;
      break;
    case HMGPU_KERNEL_VECTOR_R:
      km = kd->nX;
      kn = 3 * kd->nY;
      break;
    case HMGPU_KERNEL_DIPOLAR:
      km = 3 * kd->nX;
      kn = 3 * kd->nY;
      break;
    default:
      return fail(HMGPU_ERR_INVALID, "unknown kernel kind");
  }
  if (km != m || kn != n)
    return fail(HMGPU_ERR_INVALID, "size(K) = (" + std::to_string(km) + ", " + std::to_string(kn) +
                                       ") does not match the trees (" + std::to_string(m) + ", " +
                                       std::to_string(n) + ")");
  if (kd->kind != HMGPU_KERNEL_EXPLICIT && (!kd->X || !kd->Y))
    return fail(HMGPU_ERR_INVALID, "kernel points are NULL");
  if (kd->kind == HMGPU_KERNEL_USER) {
    if (!kd->user) return fail(HMGPU_ERR_INVALID, "a user kernel needs its compiled entry function");
    if (kd->nparams < 0 || kd->nparams > kUserMaxParams || (kd->nparams > 0 && !kd->params))
      return fail(HMGPU_ERR_INVALID, "user kernel parameters: 0 to " + std::to_string(kUserMaxParams) +
                                         " values, and a pointer when there are any");
  }
  return HMGPU_OK;
}

// The kernel's points (or explicit matrix, and a user kernel's parameters) on
// the device; `uf` the user kernel's entry kernels, or NULL.
static int upload_kernel(const hmgpu_kernel *kd, int64_t m, int64_t n, DevBuf &dX, DevBuf &dY, DevBuf &dA,
                         DevBuf &dP, KDev &K, const UserFns *&uf) {
  K = KDev{kd->kind, nullptr, nullptr, nullptr, kd->lda, nullptr, 1, 1};
  uf = nullptr;
  int rc;
  if (kd->kind == HMGPU_KERNEL_USER) {
    if ((rc = user_functions(kd->user, &uf))) return rc;
    if ((rc = dP.alloc(static_cast<size_t>(std::max<int64_t>(kd->nparams, 1)) * sizeof(double)))) return rc;
    if (kd->nparams > 0) {
      cudaError_t e = cudaMemcpy(dP.p, kd->params, kd->nparams * sizeof(double), cudaMemcpyDefault);
      if (e != cudaSuccess) return cuda_fail(e, "copying the user kernel's parameters");
    }
    K.P = dP.as<double>();
    K.dx = static_cast<int32_t>(m / kd->nX);
    K.dy = static_cast<int32_t>(n / kd->nY);
  }
  if (kd->kind == HMGPU_KERNEL_EXPLICIT) {
    if ((rc = dA.alloc(static_cast<size_t>(kd->lda) * n * sizeof(double)))) return rc;
    cudaError_t e = cudaMemcpy(dA.p, kd->A, kd->lda * n * sizeof(double), cudaMemcpyDefault);
    if (e != cudaSuccess) return cuda_fail(e, "copying the explicit matrix");
    K.A = dA.as<double>();
  } else {
    if ((rc = upload_coords(kd->X, kd->nX, dX)) || (rc = upload_coords(kd->Y, kd->nY, dY))) return rc;
    K.X = dX.as<double>();
    K.Y = dY.as<double>();
  }
  return HMGPU_OK;
}

}  // namespace hm

using namespace hm;

// ---------------------------------------------------------------------------
// HMatrix(K, X, Y; eta, eps, svd_recompress) on the device
// ---------------------------------------------------------------------------
extern "C" int hmgpu_hmatrix_build(const hmgpu_options *opt, const hmgpu_kernel *kd,
                                   const hmgpu_tree *Xh, const hmgpu_tree *Yh, double eta,
                                   double eps, int svd_recompress, hmgpu_hmatrix **out) {
  auto t0 = std::chrono::steady_clock::now();
  if (!kd || !Xh || !Yh || !out) return fail(HMGPU_ERR_INVALID, "NULL argument");
  *out = nullptr;
  const Tree &X = Xh->t;
  const Tree &Y = Yh->t;
  hmgpu_options o{HMGPU_F32, 0, 0, 0, nullptr};
  if (opt) o = *opt;
  if (o.precision != HMGPU_F64 && o.precision != HMGPU_F32 && o.precision != HMGPU_MIXED)
    return fail(HMGPU_ERR_INVALID, "unknown precision mode");
  if (!(eps >= 0.0)) return fail(HMGPU_ERR_INVALID, "eps must be >= 0");
  const int64_t m = static_cast<int64_t>(X.index_map.size()), n = static_cast<int64_t>(Y.index_map.size());
  if (m >= (int64_t(1) << 31) || n >= (int64_t(1) << 31)) return fail(HMGPU_ERR_INVALID, "too many rows or columns");
  if (int rc = check_kernel(kd, m, n)) return rc;

  auto Hp = std::make_unique<HMatrix>();
  HMatrix &H = *Hp;
  H.opt = o;
  cudaGetDevice(&H.device);
  PhaseClock clk;
  Blocks blk;
  try {
    // src/hmatrix.jl:74-78, on the device (bit-identical to the host build)
    if (int rc = build_blocks_device(X, Y, eta, true, blk)) return rc;
  } catch (const std::bad_alloc &) {
    return fail(HMGPU_ERR_NOMEM, "host allocation failed");
  }
  BlockSet &bs = H.bs;
  bs.m = m;
  bs.n = n;
  bs.tmap = X.index_map;
  bs.smap = Y.index_map;
  H.build_phase[0] = clk.lap();

  // device copies of the geometry and the maps
  DevBuf dX, dY, dA, dP, dt, ds;
  KDev K;
  const UserFns *uf;
  int rc;
  if ((rc = upload_kernel(kd, m, n, dX, dY, dA, dP, K, uf))) return rc;
  {
    std::vector<int32_t> t0v(m), s0v(n);
    for (int64_t i = 0; i < m; i++) t0v[i] = static_cast<int32_t>(X.index_map[i] - 1);
    for (int64_t j = 0; j < n; j++) s0v[j] = static_cast<int32_t>(Y.index_map[j] - 1);
    if ((rc = dt.alloc(m * 4)) || (rc = ds.alloc(n * 4))) return rc;
    cudaMemcpy(dt.p, t0v.data(), m * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(ds.p, s0v.data(), n * 4, cudaMemcpyHostToDevice);
  }

  // candidate low-rank blocks (traversal order)
  const size_t na = blk.approx.size() / 2;
  std::vector<AcaJob> jobs(na);
  for (size_t a = 0; a < na; a++) {
    const Node &x = X.nodes[blk.approx[2 * a]], &y = Y.nodes[blk.approx[2 * a + 1]];
    AcaJob &j = jobs[a];
    j.rs = static_cast<int32_t>(x.start - 1);
    j.m = static_cast<int32_t>(x.end - x.start);
    j.cs = static_cast<int32_t>(y.start - 1);
    j.n = static_cast<int32_t>(y.end - y.start);
    j.max_iter = std::min(j.m, j.n);
    j.kcap = std::min(j.max_iter, 48);
    j.ws = 0;
  }
  std::vector<int> order(na);
  for (size_t a = 0; a < na; a++) order[a] = static_cast<int>(a);
  if (o.rank_model && na > 0) {
    // learned bucketing: workspace for 1.5 x the predicted rank + 6 terms,
    // blocks of equal predicted workspace batched together
    std::vector<float> feats(na * HMGPU_RANK_FEATURES), pred(na);
    for (size_t a = 0; a < na; a++)
      block_features(X.nodes[blk.approx[2 * a]], Y.nodes[blk.approx[2 * a + 1]], eps,
                     &feats[a * HMGPU_RANK_FEATURES]);
    if ((rc = hmgpu_rank_model_predict(const_cast<hmgpu_rank_model *>(o.rank_model), feats.data(),
                                       static_cast<int64_t>(na), pred.data())))
      return rc;
    for (size_t a = 0; a < na; a++) {
      const float p = std::isfinite(pred[a]) ? std::max(pred[a], 0.0f) : 1e9f;
      const int64_t cap = static_cast<int64_t>(std::ceil(1.5 * p)) + 6;
      // never above the fixed cap: a prediction can only shrink the workspace
      // (a block that needs more is rerun with room for min(m, n) terms either way)
      jobs[a].kcap = static_cast<int32_t>(std::max<int64_t>(1, std::min<int64_t>(cap, jobs[a].kcap)));
    }
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
      if (jobs[a].kcap != jobs[b].kcap) return jobs[a].kcap > jobs[b].kcap;
      return jobs[a].m + jobs[a].n > jobs[b].m + jobs[b].n;
    });
  } else {
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
      return static_cast<int64_t>(jobs[a].m + jobs[a].n) * jobs[a].kcap >
             static_cast<int64_t>(jobs[b].m + jobs[b].n) * jobs[b].kcap;
    });
  }
  size_t free_b = 0, total_b = 0;
  cudaMemGetInfo(&free_b, &total_b);
  Compressor C;
  C.K = K;
  C.uf = uf;
  C.tmap0 = dt.as<int32_t>();
  C.smap0 = ds.as<int32_t>();
  C.eps_aca = eps / 10.0;  // src/hmatrix.jl:196
  C.eps_svd = eps;         // src/hmatrix.jl:198
  C.svd = svd_recompress ? 1 : 0;
  C.budget = static_cast<int64_t>(std::min<size_t>(free_b / 4, size_t(16) << 30) / sizeof(double));
  C.grid_aca = persistent_grid(aca_kernel);
  C.grid_qr = persistent_grid(qr_kernel);
  C.grid_form = persistent_grid(form_kernel);
  // with learned caps, a block that outgrows its cap continues in its batch
  C.resume = o.rank_model != nullptr;

  H.build_phase[1] = clk.lap();
  std::vector<AcaRes> res(na);
  std::vector<char> kept(na, 0);
  std::vector<std::unique_ptr<DevBuf>> ubufs, vbufs;
  std::vector<int> buf_of(na, -1);
  std::vector<int64_t> loc_u(na, -1), loc_v(na, -1);
  auto keep = [&](int a, int /*k*/, int r) {  // src/hmatrix.jl:202-203
    const int64_t mm = jobs[a].m, nn = jobs[a].n;
    bool ok = r * mm + r * nn < mm * nn;
    kept[a] = ok;
    return ok;
  };
  auto place = [&](const std::vector<int> &ids, const std::vector<int64_t> &uo,
                   const std::vector<int64_t> &vo, int64_t ulen, int64_t vlen, double **ust,
                   double **vst) {
    ubufs.emplace_back(new DevBuf);
    vbufs.emplace_back(new DevBuf);
    int r2;
    if ((r2 = ubufs.back()->alloc(ulen * 8)) || (r2 = vbufs.back()->alloc(vlen * 8))) return r2;
    const int bi = static_cast<int>(ubufs.size()) - 1;
    for (size_t q = 0; q < ids.size(); q++)
      if (uo[q] >= 0) {
        buf_of[ids[q]] = bi;
        loc_u[ids[q]] = uo[q];
        loc_v[ids[q]] = vo[q];
      }
    *ust = ubufs.back()->as<double>();
    *vst = vbufs.back()->as<double>();
    return HMGPU_OK;
  };
  // FP32 storage keeps no FP64 factors: each batch's factors are rounded to
  // FP32 as soon as they are formed (half the memory of the build's factors)
  const bool f32_factors = o.precision != HMGPU_F64 && !o.keep_factors;
  std::vector<std::unique_ptr<DevBuf>> ubufs32, vbufs32;
  size_t rounded = 0;  // batches already rounded
  auto after = [&]() {
    if (!f32_factors) return HMGPU_OK;
    for (; rounded < ubufs.size(); rounded++) {
      DevBuf *src[2] = {ubufs[rounded].get(), vbufs[rounded].get()};
      for (int h = 0; h < 2; h++) {
        std::unique_ptr<DevBuf> d(new DevBuf);
        const int64_t len = static_cast<int64_t>(src[h]->cap / sizeof(double));
        int r2;
        if ((r2 = d->alloc(len * sizeof(float)))) return r2;
        const int grid = static_cast<int>(std::min<int64_t>((len + 255) / 256, 152 * 32));
        if (len > 0) round_kernel<<<grid, 256>>>(src[h]->as<double>(), d->as<float>(), len);
        cudaError_t e = cudaDeviceSynchronize();
        if (e != cudaSuccess) return cuda_fail(e, "rounding factors");
        src[h]->alloc(0);  // the FP64 copy is no longer needed
        (h == 0 ? ubufs32 : vbufs32).push_back(std::move(d));
      }
    }
    return HMGPU_OK;
  };
  if ((rc = C.run(jobs, res, order, keep, place, after))) return rc;
  // blocks that exhausted their workspace are rerun, first with the fixed cap
  // (blocks whose learned cap was below it), then with room for min(m, n) terms
  int64_t reruns = 0;
  for (int round = 0; round < 2; round++) {
    std::vector<int> again;
    for (int a : order)
      if (res[a].flags & 2) {
        const int32_t fixed = std::min(jobs[a].max_iter, 48);
        jobs[a].kcap = jobs[a].kcap < fixed ? fixed : jobs[a].max_iter;
        again.push_back(a);
      }
    if (again.empty()) break;
    reruns += static_cast<int64_t>(again.size());
    if ((rc = C.run(jobs, res, again, keep, place, after))) return rc;
  }
  H.aca_batches = C.batches;
  H.aca_reruns = reruns;
  H.aca_continued = C.continued;
  H.aca_ws_bytes = C.ws_bytes;
  H.build_phase[2] = clk.lap();

  // block lists in the reference's order (src/hmatrix.jl:180-213)
  for (size_t d = 0; d < blk.dense.size() / 2; d++) {
    const Node &x = X.nodes[blk.dense[2 * d]], &y = Y.nodes[blk.dense[2 * d + 1]];
    bs.d_rs.push_back(static_cast<int32_t>(x.start - 1));
    bs.d_re.push_back(static_cast<int32_t>(x.end - 1));
    bs.d_cs.push_back(static_cast<int32_t>(y.start - 1));
    bs.d_ce.push_back(static_cast<int32_t>(y.end - 1));
  }
  bs.aca_rank.assign(na, 0);
  bs.final_rank.assign(na, -1);
  int64_t ulen = 0, vlen = 0;
  std::vector<int64_t> usrc, vsrc;
  for (size_t a = 0; a < na; a++) {
    const AcaJob &j = jobs[a];
    bs.aca_rank[a] = res[a].k;
    if (kept[a]) {
      bs.final_rank[a] = res[a].r;
      bs.a_rs.push_back(j.rs);
      bs.a_re.push_back(j.rs + j.m);
      bs.a_cs.push_back(j.cs);
      bs.a_ce.push_back(j.cs + j.n);
      bs.a_r.push_back(res[a].r);
      usrc.push_back(ulen);
      vsrc.push_back(vlen);
      ulen += static_cast<int64_t>(j.m) * res[a].r;
      vlen += static_cast<int64_t>(j.n) * res[a].r;
    } else {
      bs.d_rs.push_back(j.rs);
      bs.d_re.push_back(j.rs + j.m);
      bs.d_cs.push_back(j.cs);
      bs.d_ce.push_back(j.cs + j.n);
    }
  }
  // gather the factors into one store in block order (FP32 or FP64)
  void *ust = nullptr, *vst = nullptr;
  const size_t fes = f32_factors ? sizeof(float) : sizeof(double);
  if ((rc = H.dalloc(&ust, ulen * fes)) || (rc = H.dalloc(&vst, vlen * fes))) return rc;
  {
    auto gather = [&](auto *ud, auto *vd, auto getu, auto getv) -> int {
      using E = std::remove_pointer_t<decltype(ud)>;
      std::vector<CopyJob<E>> cj;
      cj.reserve(2 * usrc.size());
      size_t q = 0;
      for (size_t a = 0; a < na; a++) {
        if (!kept[a]) continue;
        const int64_t r = res[a].r;
        const int64_t un = static_cast<int64_t>(jobs[a].m) * r, vn = static_cast<int64_t>(jobs[a].n) * r;
        if (un) cj.push_back(CopyJob<E>{getu(buf_of[a]) + loc_u[a], ud + usrc[q], un});
        if (vn) cj.push_back(CopyJob<E>{getv(buf_of[a]) + loc_v[a], vd + vsrc[q], vn});
        q++;
      }
      DevBuf dcj;
      int r3;
      if ((r3 = dcj.alloc(cj.size() * sizeof(CopyJob<E>)))) return r3;
      cudaError_t e = cudaMemcpy(dcj.p, cj.data(), cj.size() * sizeof(CopyJob<E>), cudaMemcpyHostToDevice);
      if (e == cudaSuccess && !cj.empty()) {
        const int grid = static_cast<int>(std::min<int64_t>((static_cast<int64_t>(cj.size()) + 7) / 8, 152 * 16));
        gather_kernel<E><<<grid, 256>>>(dcj.as<CopyJob<E>>(), static_cast<int64_t>(cj.size()));
        e = cudaGetLastError();
      }
      if (e == cudaSuccess) e = cudaDeviceSynchronize();
      return e == cudaSuccess ? HMGPU_OK : cuda_fail(e, "gathering factors");
    };
    if (f32_factors)
      rc = gather(static_cast<float *>(ust), static_cast<float *>(vst),
                  [&](int b) { return ubufs32[b]->as<float>(); }, [&](int b) { return vbufs32[b]->as<float>(); });
    else
      rc = gather(static_cast<double *>(ust), static_cast<double *>(vst),
                  [&](int b) { return ubufs[b]->as<double>(); }, [&](int b) { return vbufs[b]->as<double>(); });
    if (rc) return rc;
  }
  ubufs32.clear();
  vbufs32.clear();
  ubufs.clear();
  vbufs.clear();
  H.build_phase[3] = clk.lap();
  std::vector<int64_t> dsrc(bs.d_rs.size(), -1);
  KernelGen gen;
  gen.K = K;
  gen.uf = uf;
  if ((rc = finalize_layout(H, nullptr, dsrc, ust, usrc, vst, vsrc, &gen, f32_factors))) return rc;
  if (o.keep_factors) {
    H.u64 = static_cast<double *>(ust);
    H.v64 = static_cast<double *>(vst);
    H.u_src_off = usrc;
    H.v_src_off = vsrc;
  } else {
    H.dfree(ust);
    H.dfree(vst);
    H.device_bytes -= (ulen + vlen) * static_cast<int64_t>(fes);
  }
  H.build_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  *out = reinterpret_cast<hmgpu_hmatrix *>(Hp.release());
  return HMGPU_OK;
}

// ---------------------------------------------------------------------------
// single-block ACA_plus and SVD_recompress through the batched kernels
// ---------------------------------------------------------------------------
extern "C" int hmgpu_aca_plus(const double *A, int64_t lda, int64_t m, int64_t n, double eps,
                              int64_t max_iter, int64_t cap, double *U, double *V, int64_t *rank) {
  if (!A || !U || !V || !rank) return fail(HMGPU_ERR_INVALID, "NULL argument");
  if (m <= 0 || n <= 0 || lda < m) return fail(HMGPU_ERR_INVALID, "bad block size");
  if (m >= (int64_t(1) << 31) || n >= (int64_t(1) << 31)) return fail(HMGPU_ERR_INVALID, "block too large");
  if (max_iter <= 0) max_iter = m;  // default max_iter = n_rows (src/aca.jl:36)
  const int64_t mi = std::min(std::min(m, n), max_iter);
  if (cap < mi) return fail(HMGPU_ERR_INVALID, "cap < min(m, n, max_iter)");
  DevBuf dA, dt, ds, dj, dr, dws, dtk;
  int rc;
  if ((rc = dA.alloc(lda * n * 8)) || (rc = dt.alloc(m * 4)) || (rc = ds.alloc(n * 4)) ||
      (rc = dj.alloc(sizeof(AcaJob))) || (rc = dr.alloc(sizeof(AcaRes))) || (rc = dtk.alloc(16)))
    return rc;
  cudaMemcpy(dA.p, A, lda * n * 8, cudaMemcpyDefault);
  std::vector<int32_t> id(std::max(m, n));
  for (size_t i = 0; i < id.size(); i++) id[i] = static_cast<int32_t>(i);
  cudaMemcpy(dt.p, id.data(), m * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(ds.p, id.data(), n * 4, cudaMemcpyHostToDevice);
  AcaJob j{0, static_cast<int32_t>(m), 0, static_cast<int32_t>(n), 0, static_cast<int32_t>(mi),
           static_cast<int32_t>(mi), 0, 0, 0};
  if ((rc = dws.alloc(ws_doubles(m, n, mi) * 8))) return rc;
  cudaMemcpy(dj.p, &j, sizeof j, cudaMemcpyHostToDevice);
  cudaMemset(dr.p, 0, sizeof(AcaRes));
  cudaMemset(dtk.p, 0, 16);
  KDev K{HMGPU_KERNEL_EXPLICIT, nullptr, nullptr, dA.as<double>(), lda};
  aca_kernel<<<1, kBuildThreads>>>(K, dt.as<int32_t>(), ds.as<int32_t>(), dj.as<AcaJob>(), team_job(j) ? 1 : 0, 1,
                                   eps, dws.as<double>(), dr.as<AcaRes>(), dtk.as<int32_t>());
  AcaRes r;
  cudaError_t e = cudaMemcpy(&r, dr.p, sizeof r, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "ACA kernel");
  std::vector<double> ws(static_cast<size_t>(m * mi + mi * n));
  cudaMemcpy(ws.data(), dws.p, ws.size() * 8, cudaMemcpyDeviceToHost);
  for (int64_t q = 0; q < r.k; q++) {
    for (int64_t i = 0; i < m; i++) U[i + q * m] = ws[i + q * m];
    for (int64_t c = 0; c < n; c++) V[q + c * cap] = ws[m * mi + q * n + c];
  }
  *rank = r.k;
  return HMGPU_OK;
}

extern "C" int hmgpu_svd_recompress(int64_t m, int64_t n, int64_t k, const double *U,
                                    const double *V, double eps, double *U_out, double *V_out,
                                    int64_t *r_out) {
  if (!U || !V || !U_out || !V_out || !r_out) return fail(HMGPU_ERR_INVALID, "NULL argument");
  if (m <= 0 || n <= 0 || k < 0 || k > m || k > n) return fail(HMGPU_ERR_INVALID, "bad sizes (need k <= m, n)");
  if (k == 0) {
    *r_out = 0;
    return HMGPU_OK;
  }
  DevBuf dj, dr, dws, dtk, duo, dvo, dus, dvs;
  int rc;
  if ((rc = dj.alloc(sizeof(AcaJob))) || (rc = dr.alloc(sizeof(AcaRes))) || (rc = dtk.alloc(16)) ||
      (rc = dws.alloc(ws_doubles(m, n, k) * 8)) || (rc = duo.alloc(8)) || (rc = dvo.alloc(8)) ||
      (rc = dus.alloc(m * k * 8)) || (rc = dvs.alloc(k * n * 8)))
    return rc;
  std::vector<double> w(static_cast<size_t>(m * k + k * n));
  for (int64_t i = 0; i < m * k; i++) w[i] = U[i];
  for (int64_t q = 0; q < k; q++)
    for (int64_t c = 0; c < n; c++) w[m * k + q * n + c] = V[q + c * k];
  cudaMemcpy(dws.p, w.data(), w.size() * 8, cudaMemcpyHostToDevice);
  AcaJob j{0, static_cast<int32_t>(m), 0, static_cast<int32_t>(n), 0, static_cast<int32_t>(k),
           static_cast<int32_t>(k), 0, 0, 0};
  AcaRes r0{static_cast<int32_t>(k), 0, 0, 0};
  cudaMemcpy(dj.p, &j, sizeof j, cudaMemcpyHostToDevice);
  cudaMemcpy(dr.p, &r0, sizeof r0, cudaMemcpyHostToDevice);
  cudaMemset(dtk.p, 0, 16);
  int64_t zero = 0;
  cudaMemcpy(duo.p, &zero, 8, cudaMemcpyHostToDevice);
  cudaMemcpy(dvo.p, &zero, 8, cudaMemcpyHostToDevice);
  const int big = team_job(j) ? 1 : 0;
  qr_kernel<<<1, kBuildThreads>>>(dj.as<AcaJob>(), big, 1, 1, dws.as<double>(), dr.as<AcaRes>(), dtk.as<int32_t>());
  jacobi_kernel<<<1, 32>>>(dj.as<AcaJob>(), 1, eps, 1, dws.as<double>(), dr.as<AcaRes>());
  form_kernel<<<1, kBuildThreads>>>(dj.as<AcaJob>(), big, 1, 1, dws.as<double>(), dr.as<AcaRes>(),
                                    duo.as<int64_t>(), dvo.as<int64_t>(), dus.as<double>(), dvs.as<double>(),
                                    dtk.as<int32_t>() + 2);
  AcaRes r;
  cudaError_t e = cudaMemcpy(&r, dr.p, sizeof r, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "recompression kernels");
  std::vector<double> uo(static_cast<size_t>(m * r.r)), vo(static_cast<size_t>(r.r * n));
  cudaMemcpy(uo.data(), dus.p, uo.size() * 8, cudaMemcpyDeviceToHost);
  cudaMemcpy(vo.data(), dvs.p, vo.size() * 8, cudaMemcpyDeviceToHost);
  for (int64_t i = 0; i < m; i++)
    for (int64_t c = 0; c < r.r; c++) U_out[i + c * m] = uo[i * r.r + c];
  for (int64_t c = 0; c < r.r; c++)
    for (int64_t q = 0; q < n; q++) V_out[c + q * r.r] = vo[c * n + q];
  *r_out = r.r;
  return HMGPU_OK;
}

// ---------------------------------------------------------------------------
// sparsify_hmatrix(K, X, Y; eta) (src/hmatrix.jl:234-274)
// ---------------------------------------------------------------------------
extern "C" int hmgpu_sparsify(const hmgpu_kernel *kd, const hmgpu_tree *Xh, const hmgpu_tree *Yh, double eta,
                              int64_t *I, int64_t *J, double *V, int64_t *nnz) {
  if (!kd || !Xh || !Yh) return fail(HMGPU_ERR_INVALID, "NULL argument");
  const Tree &X = Xh->t;
  const Tree &Y = Yh->t;
  const int64_t m = static_cast<int64_t>(X.index_map.size()), n = static_cast<int64_t>(Y.index_map.size());
  if (m >= (int64_t(1) << 31) || n >= (int64_t(1) << 31)) return fail(HMGPU_ERR_INVALID, "too many rows or columns");
  if (int rc = check_kernel(kd, m, n)) return rc;
  Blocks blk;
  try {
    // BlockTree + merge_dense_matrices! + traverse (:236-239), on the device
    if (int rc = build_blocks_device(X, Y, eta, true, blk)) return rc;
  } catch (const std::bad_alloc &) {
    return fail(HMGPU_ERR_NOMEM, "host allocation failed");
  }
  const size_t nd = blk.dense.size() / 2;
  int64_t count = 0;
  for (size_t b = 0; b < nd; b++) {
    const Node &x = X.nodes[blk.dense[2 * b]], &y = Y.nodes[blk.dense[2 * b + 1]];
    count += (x.end - x.start) * (y.end - y.start);
  }
  if (nnz) *nnz = count;
  if (!I && !J && !V) return HMGPU_OK;
  if (!I || !J || !V) return fail(HMGPU_ERR_INVALID, "I, J and V must all be given, or all be NULL to count");
  // indices on the host (1-based original indices, :251-263)
  int64_t k = 0;
  for (size_t b = 0; b < nd; b++) {
    const Node &x = X.nodes[blk.dense[2 * b]], &y = Y.nodes[blk.dense[2 * b + 1]];
    for (int64_t i = x.start; i < x.end; i++)
      for (int64_t j = y.start; j < y.end; j++, k++) {
        I[k] = X.index_map[i - 1];
        J[k] = Y.index_map[j - 1];
      }
  }
  // values on the device, in pieces of at most kPiece entries
  constexpr int64_t kPiece = int64_t(32) << 20;
  DevBuf dX, dY, dA, dP, dt, ds, dout, djobs;
  KDev K;
  const UserFns *uf;
  int rc;
  if ((rc = upload_kernel(kd, m, n, dX, dY, dA, dP, K, uf))) return rc;
  {
    std::vector<int32_t> t0v(m), s0v(n);
    for (int64_t i = 0; i < m; i++) t0v[i] = static_cast<int32_t>(X.index_map[i] - 1);
    for (int64_t j = 0; j < n; j++) s0v[j] = static_cast<int32_t>(Y.index_map[j] - 1);
    if ((rc = dt.alloc(m * 4)) || (rc = ds.alloc(n * 4))) return rc;
    cudaMemcpy(dt.p, t0v.data(), m * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(ds.p, s0v.data(), n * 4, cudaMemcpyHostToDevice);
  }
  int64_t largest = 0;
  for (size_t b = 0; b < nd; b++) {
    const Node &x = X.nodes[blk.dense[2 * b]], &y = Y.nodes[blk.dense[2 * b + 1]];
    largest = std::max<int64_t>(largest, (x.end - x.start) * (y.end - y.start));
  }
  const int64_t piece = std::max(kPiece, largest);
  if ((rc = dout.alloc(static_cast<size_t>(std::min(piece, std::max<int64_t>(count, 1))) * sizeof(double)))) return rc;
  int64_t base = 0;
  for (size_t b0 = 0; b0 < nd;) {
    std::vector<SpJob> jobs;
    int64_t used = 0;
    size_t b = b0;
    for (; b < nd; b++) {
      const Node &x = X.nodes[blk.dense[2 * b]], &y = Y.nodes[blk.dense[2 * b + 1]];
      const int64_t e = (x.end - x.start) * (y.end - y.start);
      if (!jobs.empty() && used + e > piece) break;
      jobs.push_back(SpJob{static_cast<int32_t>(x.start - 1), static_cast<int32_t>(x.end - x.start),
                           static_cast<int32_t>(y.start - 1), static_cast<int32_t>(y.end - y.start), used});
      used += e;
    }
    if ((rc = djobs.alloc(jobs.size() * sizeof(SpJob)))) return rc;
    cudaMemcpy(djobs.p, jobs.data(), jobs.size() * sizeof(SpJob), cudaMemcpyHostToDevice);
    const int grid = static_cast<int>(std::min<int64_t>((static_cast<int64_t>(jobs.size()) + 7) / 8, 65535));
    cudaError_t e = launch_sparsify(uf, grid, K, dt.as<int32_t>(), ds.as<int32_t>(), djobs.as<SpJob>(),
                                    static_cast<int64_t>(jobs.size()), dout.as<double>());
    if (e != cudaSuccess) return cuda_fail(e, "sparsify launch");
    e = cudaMemcpy(V + base, dout.p, used * sizeof(double), cudaMemcpyDefault);
    if (e != cudaSuccess) return cuda_fail(e, "sparsify entries");
    base += used;
    b0 = b;
  }
  return HMGPU_OK;
}
