// Batches of H-matrices, CUDA-graph products and the product autotuner.
//
// A batch is the block-diagonal operator diag(H_1, ..., H_k) as one H-matrix:
// the members' device layouts are concatenated and every index of their
// tables is shifted, so a product of the batch runs all members in the same
// (persistent, ticket-scheduled) kernel launches: three launches for any
// number of members instead of three per member.
//
// XT of a batch is [x regions of all members | t regions of all members]; a
// member's own XT index v maps to x_base + v in its x region (v < x_len) or to
// T0 + t_base + (v - x_len) in its t region.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <memory>
#include <numeric>
#include <string>
#include <vector>

#include "hm_api.h"

using hm::HMatrix;

extern "C" int hmgpu_hmatrix_batch(hmgpu_hmatrix *const *members, int32_t count, hmgpu_hmatrix **out) {
  auto t_start = std::chrono::steady_clock::now();
  if (!out) return hm::fail(HMGPU_ERR_INVALID, "out is NULL");
  *out = nullptr;
  if (count < 1 || !members) return hm::fail(HMGPU_ERR_INVALID, "a batch needs at least one member");
  std::vector<const HMatrix *> M(count);
  for (int32_t k = 0; k < count; k++) {
    if (!members[k]) return hm::fail(HMGPU_ERR_INVALID, "member " + std::to_string(k) + " is NULL");
    M[k] = reinterpret_cast<const HMatrix *>(members[k]);
    if (M[k]->is_shard) return hm::fail(HMGPU_ERR_INVALID, "a shard cannot be a batch member");
    if (M[k]->lean) return hm::fail(HMGPU_ERR_INVALID, "a lean mixed H-matrix keeps only its tensor-core copy; a batch is built from the FP32 layouts");
  }
  int dev = 0;
  cudaGetDevice(&dev);
  for (int32_t k = 0; k < count; k++) {
    if (M[k]->device != M[0]->device || M[k]->device != dev)
      return hm::fail(HMGPU_ERR_INVALID, "batch members must live on the current device");
    if (M[k]->opt.precision != M[0]->opt.precision || M[k]->opt.compensated != M[0]->opt.compensated)
      return hm::fail(HMGPU_ERR_INVALID, "batch members must share precision and compensation");
  }
  auto B = std::make_unique<HMatrix>();
  B->device = dev;
  B->opt = M[0]->opt;
  B->opt.keep_factors = 0;
  B->opt.rank_model = nullptr;
  const bool f64 = B->opt.precision == HMGPU_F64;
  const size_t es = f64 ? 8 : 4;
  int rc;
  if ((rc = hm::setup_grids(*B))) return rc;

  std::vector<const hm::Plan *> plans(count);
  std::vector<const hm::BlockSet *> sets(count);
  for (int32_t k = 0; k < count; k++) {
    plans[k] = &M[k]->plan;
    sets[k] = &M[k]->bs;
    B->build_seconds += M[k]->build_seconds;
    B->aca_batches += M[k]->aca_batches;
    B->aca_reruns += M[k]->aca_reruns;
  }
  hm::Plan &P = B->plan;
  std::vector<int32_t> tmap0, smap0;
  std::vector<int64_t> panel_base, v_base;
  if ((rc = hm::combine_plans(plans, sets, B->grid_v * (hm::kThreads / 32), P, B->bs, tmap0, smap0,
                              panel_base, v_base)))
    return rc;
  B->multi_from = M[0]->multi_from;
  B->member_rows.assign(1, 0);
  B->member_cols.assign(1, 0);
  for (int32_t k = 0; k < count; k++) {
    B->member_rows.push_back(B->member_rows.back() + M[k]->bs.m);
    B->member_cols.push_back(B->member_cols.back() + M[k]->bs.n);
  }

  // device data: the members' panels and V rows, copied in order
  if ((rc = B->dalloc(&B->panels, P.panel_len * es))) return rc;
  if ((rc = B->dalloc(&B->vdata, P.v_len * es))) return rc;
  for (int32_t k = 0; k < count; k++) {
    const hm::Plan &q = M[k]->plan;
    cudaError_t e = cudaMemcpy(static_cast<char *>(B->panels) + panel_base[k] * es, M[k]->panels,
                               q.panel_len * es, cudaMemcpyDeviceToDevice);
    if (e == cudaSuccess)
      e = cudaMemcpy(static_cast<char *>(B->vdata) + v_base[k] * es, M[k]->vdata, q.v_len * es,
                     cudaMemcpyDeviceToDevice);
    if (e != cudaSuccess) return hm::cuda_fail(e, "copying a batch member");
  }
  // the padding entry after member 0's x is always zero
  if ((rc = hm::upload_plan(*B, tmap0, smap0, M[0]->bs.n))) return rc;
  if (B->opt.precision == HMGPU_MIXED && (rc = hm::build_tc(*B))) return rc;
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return hm::cuda_fail(e, "assembling the batch");
  B->build_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
  *out = reinterpret_cast<hmgpu_hmatrix *>(B.release());
  return HMGPU_OK;
}

// ---------------------------------------------------------------------------
// CUDA graphs
// ---------------------------------------------------------------------------
struct hmgpu_graph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

extern "C" int hmgpu_graph_create(hmgpu_hmatrix *h, const void *x, void *y, int64_t nrhs, int64_t ldx,
                                  int64_t ldy, hmgpu_graph **out) {
  if (!h || !out) return hm::fail(HMGPU_ERR_INVALID, "NULL argument");
  *out = nullptr;
  if (nrhs < 1) return hm::fail(HMGPU_ERR_INVALID, "a graph needs at least one right-hand side");
  HMatrix &H = *reinterpret_cast<HMatrix *>(h);
  cudaStream_t s;
  cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  if (e != cudaSuccess) return hm::cuda_fail(e, "cudaStreamCreate");
  const bool prof = H.profiling;
  H.profiling = false;
  // one product outside the capture allocates the scratch and sets the kernel
  // attributes, so that the captured product only launches kernels
  int rc = hmgpu_matvec(h, x, y, nrhs, ldx, ldy, s);
  if (rc == HMGPU_OK) {
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) rc = hm::cuda_fail(e, "product before capture");
  }
  auto g = std::make_unique<hmgpu_graph>();
  if (rc == HMGPU_OK) {
    e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
      rc = hm::cuda_fail(e, "cudaStreamBeginCapture");
    } else {
      rc = hmgpu_matvec(h, x, y, nrhs, ldx, ldy, s);
      e = cudaStreamEndCapture(s, &g->graph);
      if (rc == HMGPU_OK && e != cudaSuccess) rc = hm::cuda_fail(e, "cudaStreamEndCapture");
      if (rc == HMGPU_OK) {
        e = cudaGraphInstantiate(&g->exec, g->graph, 0);
        if (e != cudaSuccess) rc = hm::cuda_fail(e, "cudaGraphInstantiate");
      }
    }
  }
  H.profiling = prof;
  cudaStreamDestroy(s);
  if (rc != HMGPU_OK) {
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    cudaGetLastError();
    return rc;
  }
  *out = g.release();
  return HMGPU_OK;
}

extern "C" int hmgpu_graph_launch(hmgpu_graph *G, void *stream) {
  if (!G || !G->exec) return hm::fail(HMGPU_ERR_INVALID, "graph is NULL");
  cudaError_t e = cudaGraphLaunch(G->exec, static_cast<cudaStream_t>(stream));
  return e == cudaSuccess ? HMGPU_OK : hm::cuda_fail(e, "cudaGraphLaunch");
}

extern "C" int hmgpu_graph_free(hmgpu_graph *G) {
  if (!G) return HMGPU_OK;
  if (G->exec) cudaGraphExecDestroy(G->exec);
  if (G->graph) cudaGraphDestroy(G->graph);
  delete G;
  return HMGPU_OK;
}

// ---------------------------------------------------------------------------
// autotuner
// ---------------------------------------------------------------------------
namespace {

uint64_t structure_hash(const HMatrix &H) {
  cudaDeviceProp prop;
  std::memset(&prop, 0, sizeof prop);
  cudaGetDeviceProperties(&prop, H.device);
  uint64_t h = 1469598103934665603ull;
  auto mix = [&](uint64_t v) {
    for (int i = 0; i < 8; i++) {
      h ^= (v >> (8 * i)) & 0xff;
      h *= 1099511628211ull;
    }
  };
  int64_t R = 0;
  for (int32_t r : H.bs.a_r) R += r;
  mix(static_cast<uint64_t>(H.bs.m));
  mix(static_cast<uint64_t>(H.bs.n));
  mix(H.bs.d_rs.size());
  mix(H.bs.a_rs.size());
  mix(static_cast<uint64_t>(R));
  mix(static_cast<uint64_t>(H.plan.dense_entries));
  mix(static_cast<uint64_t>(H.plan.far_entries));
  mix(static_cast<uint64_t>(H.opt.precision * 2 + H.opt.compensated));
  mix(static_cast<uint64_t>(prop.multiProcessorCount));
  for (const char *c = prop.name; *c; c++) mix(static_cast<unsigned char>(*c));
  return h;
}

bool cache_lookup(const char *path, uint64_t key, int32_t (&v)[4]) {
  if (!path) return false;
  FILE *f = std::fopen(path, "r");
  if (!f) return false;
  char line[256];
  bool found = false;
  while (std::fgets(line, sizeof line, f)) {
    unsigned long long k;
    int a, b, c, d;
    if (std::sscanf(line, "hmgpu-tune %llx %d %d %d %d", &k, &a, &b, &c, &d) == 5 && k == key) {
      v[0] = a;
      v[1] = b;
      v[2] = c;
      v[3] = d;
      found = true;  // the last line for a key wins
    }
  }
  std::fclose(f);
  return found;
}

void cache_store(const char *path, uint64_t key, const int32_t (&v)[4]) {
  if (!path) return;
  FILE *f = std::fopen(path, "a");
  if (!f) return;
  std::fprintf(f, "hmgpu-tune %016llx %d %d %d %d\n", static_cast<unsigned long long>(key), v[0], v[1], v[2],
               v[3]);
  std::fclose(f);
}

int apply(HMatrix &H, int32_t unit_rows, int32_t vunit_kib, int32_t multi_from, int32_t v_dynamic) {
  hm::make_units(H.plan, unit_rows);
  hm::make_vunits(H.plan, static_cast<int64_t>(vunit_kib) * 1024, H.grid_v * (hm::kThreads / 32));
  H.multi_from = multi_from;
  H.dp.v_dynamic = v_dynamic != 0;
  return hm::upload_units(H);
}

// Average device time in ms of `reps` products after `warm` untimed ones.
int time_products(hmgpu_hmatrix *h, const void *x, void *y, int64_t nrhs, int64_t ldx, int64_t ldy,
                  cudaStream_t s, cudaEvent_t e0, cudaEvent_t e1, int warm, int reps, float *ms) {
  for (int i = 0; i < warm; i++)
    if (int rc = hmgpu_matvec(h, x, y, nrhs, ldx, ldy, s)) return rc;
  cudaEventRecord(e0, s);
  for (int i = 0; i < reps; i++)
    if (int rc = hmgpu_matvec(h, x, y, nrhs, ldx, ldy, s)) return rc;
  cudaEventRecord(e1, s);
  cudaError_t e = cudaEventSynchronize(e1);
  if (e != cudaSuccess) return hm::cuda_fail(e, "autotune timing");
  cudaEventElapsedTime(ms, e0, e1);
  *ms /= reps;
  return HMGPU_OK;
}

}  // namespace

extern "C" int hmgpu_hmatrix_autotune(hmgpu_hmatrix *h, const char *cache_path, int32_t *result) {
  if (!h) return hm::fail(HMGPU_ERR_INVALID, "H is NULL");
  HMatrix &H = *reinterpret_cast<HMatrix *>(h);
  if (H.is_shard) return hm::fail(HMGPU_ERR_INVALID, "a shard multiplies through hmgpu_matvec_shard only");
  if (H.lean) {  // only the tensor-core pass, which has nothing to tune
    if (result) {
      const int32_t cur[4] = {H.plan.unit_rows, static_cast<int32_t>(H.plan.vunit_bytes / 1024), H.multi_from, 0};
      std::copy(cur, cur + 4, result);
    }
    return HMGPU_OK;
  }
  const uint64_t key = structure_hash(H);
  int32_t best[4];
  if (cache_lookup(cache_path, key, best)) {
    if (int rc = apply(H, best[0], best[1], best[2], best[3])) return rc;
    if (result) {
      std::copy(best, best + 3, result);
      result[3] = 1;
    }
    return HMGPU_OK;
  }
  const size_t es = H.opt.precision == HMGPU_F64 ? 8 : 4;
  const int64_t m = H.bs.m, n = H.bs.n, per = hm::rhs_per_pass();
  void *x = nullptr, *y = nullptr;
  cudaStream_t s = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = HMGPU_OK;
  const bool prof = H.profiling;
  H.profiling = false;
  auto cleanup = [&]() {
    if (x) cudaFree(x);
    if (y) cudaFree(y);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (s) cudaStreamDestroy(s);
    H.profiling = prof;
  };
  cudaError_t e = cudaMalloc(&x, n * per * es);
  if (e == cudaSuccess) e = cudaMalloc(&y, m * per * es);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  if (e == cudaSuccess) e = cudaMemsetAsync(x, 0, n * per * es, s);  // the timing does not depend on x
  if (e != cudaSuccess) {
    cleanup();
    cudaGetLastError();
    return hm::fail(HMGPU_ERR_NOMEM, std::string("autotune scratch: ") + cudaGetErrorString(e));
  }
  // single-RHS layout parameters and the V schedule
  const int32_t cand_rows[4] = {8, 16, 32, 64}, cand_kib[3] = {32, 64, 128};
  float t1 = 0.0f;
  best[0] = 16;
  best[1] = 64;
  best[3] = 0;
  for (int32_t ur : cand_rows)
    for (int32_t kib : cand_kib)
      for (int32_t vd = 0; vd < 2 && rc == HMGPU_OK; vd++) {
        if ((rc = apply(H, ur, kib, H.multi_from, vd))) break;
        float ms = 0.0f;
        if ((rc = time_products(h, x, y, 1, n, m, s, e0, e1, 2, 5, &ms))) break;
        if (t1 == 0.0f || ms < t1) {
          t1 = ms;
          best[0] = ur;
          best[1] = kib;
          best[3] = vd;
        }
      }
  // crossover: one multi-RHS pass (8, 16 or rhs_per_pass() wide) against
  // repeated single-RHS products; the threshold is the first k from which
  // every k' up to a full pass is faster as one pass of its width
  if (rc == HMGPU_OK && (rc = apply(H, best[0], best[1], 2, best[3])) == HMGPU_OK) {
    const int64_t widths[3] = {8, 16, per};
    float tw[3] = {0.0f, 0.0f, 0.0f};
    for (int i = 0; i < 3 && rc == HMGPU_OK; i++)
      rc = time_products(h, x, y, widths[i], n, m, s, e0, e1, 1, 3, &tw[i]);
    if (rc == HMGPU_OK) {
      int32_t from = 1 << 30;
      for (int64_t k = per; k >= 2; k--) {
        const int w = hm::multi_width(static_cast<int>(k));
        const float tm = tw[w == 8 ? 0 : w == 16 ? 1 : 2];
        if (static_cast<float>(k) * t1 > tm)
          from = static_cast<int32_t>(k);
        else
          break;
      }
      best[2] = from;
      rc = apply(H, best[0], best[1], best[2], best[3]);
    }
  }
  cleanup();
  if (rc != HMGPU_OK) return rc;
  cache_store(cache_path, key, best);
  if (result) {
    std::copy(best, best + 3, result);
    result[3] = 0;
  }
  return HMGPU_OK;
}

extern "C" int hmgpu_hmatrix_tuning(const hmgpu_hmatrix *h, int32_t *v, int32_t n) {
  if (!h || (!v && n > 0)) return hm::fail(HMGPU_ERR_INVALID, "NULL argument");
  const HMatrix &H = *reinterpret_cast<const HMatrix *>(h);
  const int32_t all[4] = {H.plan.unit_rows, static_cast<int32_t>(H.plan.vunit_bytes / 1024), H.multi_from,
                          H.dp.v_dynamic ? 1 : 0};
  for (int32_t i = 0; i < n && i < 4; i++) v[i] = all[i];
  return HMGPU_OK;
}

extern "C" int hmgpu_hmatrix_set_tuning(hmgpu_hmatrix *h, const int32_t *v, int32_t n) {
  if (!h || !v || n < 4) return hm::fail(HMGPU_ERR_INVALID, "need H and 4 values");
  HMatrix &H = *reinterpret_cast<HMatrix *>(h);
  if ((v[0] != 8 && v[0] != 16 && v[0] != 32 && v[0] != 64) || (v[1] != 32 && v[1] != 64 && v[1] != 128) || v[2] < 2 || (v[3] != 0 && v[3] != 1))
    return hm::fail(HMGPU_ERR_INVALID, "tuning values out of range (unit rows 8|16|32|64, V unit KiB 32|64|128, "
                                       "multi-RHS threshold >= 2, V schedule 0|1)");
  if (H.lean) return hm::fail(HMGPU_ERR_INVALID, "a lean mixed H-matrix keeps only its tensor-core copy: every product runs on the tensor cores");
  return apply(H, v[0], v[1], v[2], v[3]);
}
