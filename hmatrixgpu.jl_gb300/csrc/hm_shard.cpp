// Row shards of an H-matrix for products split over several GPUs.
//
// The reference's product owns every row of y in exactly one place: row I of
// the permuted output is written once, by the thread that sums it
// (src/mult.jl:144). Rows therefore split across GPUs with no reduction: a
// shard owns a contiguous range of row tiles (hence a contiguous range of
// permuted rows) and computes exactly those rows of y. What it reads is x in
// the permuted source order (every GPU needs the x entries of every source
// cluster its tiles touch, so x is all-gathered before the product, in that
// order) and the t = V x entries of the low-rank blocks in its tiles.
//
// A shard is an H-matrix handle of its own: the owned tiles' panels, the V
// rows of every source group that feeds one of its tiles (whole groups, so a
// group read by two shards is computed by both), and the single-RHS product
// tables rebuilt for that subset. Its product is the parent's single-RHS
// product restricted to the owned rows, so every owned row is bitwise the
// parent's (each row and each rank row keeps its summation order).
#include <algorithm>
#include <cstring>
#include <new>
#include <numeric>

#include "hm_api.h"

namespace hm {

namespace {

// Tiles [lo, hi) of shard `rank`: contiguous, balanced by panel entries.
void tile_range(const Plan &p, int32_t rank, int32_t world, size_t &lo, size_t &hi) {
  const size_t nt = p.tiles.size();
  std::vector<int64_t> pre(nt + 1, 0);
  for (size_t i = 0; i < nt; i++) pre[i + 1] = pre[i] + int64_t{p.tiles[i].m} * p.tiles[i].ld + 1;
  auto first_at = [&](int64_t goal) {
    return static_cast<size_t>(std::lower_bound(pre.begin(), pre.end(), goal) - pre.begin());
  };
  const int64_t total = pre[nt];
  lo = rank == 0 ? 0 : std::min(nt, first_at(total * rank / world));
  hi = rank == world - 1 ? nt : std::min(nt, first_at(total * (rank + 1) / world));
  if (hi < lo) hi = lo;
}

}  // namespace

static int make_shard(const HMatrix &H, int32_t rank, int32_t world, HMatrix &S) {
  const Plan &p = H.plan;
  const size_t es = H.opt.precision == HMGPU_F64 ? 8 : 4;
  size_t lo, hi;
  tile_range(p, rank, world, lo, hi);
  S.device = H.device;
  S.opt = H.opt;
  S.opt.keep_factors = 0;
  S.opt.rank_model = nullptr;
  if (S.opt.precision == HMGPU_MIXED) S.opt.precision = HMGPU_F32, S.opt.compensated = 1;
  S.bs = H.bs;
  S.is_shard = true;
  S.shard_rank = rank;
  S.shard_world = world;
  S.multi_from = 1 << 30;
  Plan &q = S.plan;
  q.vec = p.vec;
  q.x_len = p.x_len;
  q.R = p.R;
  q.xt_len = p.xt_len;
  q.dense_entries = p.dense_entries;
  q.far_entries = p.far_entries;
  // ---- owned tiles, their segments and panels ----------------------------------------
  const int64_t pbase = lo < hi ? p.tiles[lo].data_off : 0;
  const int32_t sbase = lo < hi ? p.tiles[lo].seg0 : 0;
  int64_t pend = pbase;
  int32_t send = sbase;
  S.shard_row0 = lo < hi ? p.tiles[lo].row0 : 0;
  S.shard_row1 = S.shard_row0;
  for (size_t i = lo; i < hi; i++) {
    TileDesc d = p.tiles[i];
    pend = std::max(pend, d.data_off + int64_t{d.m} * d.ld);
    send = std::max(send, d.seg0 + d.nseg);
    S.shard_row1 = std::max<int64_t>(S.shard_row1, int64_t{d.row0} + d.m);
    d.data_off -= pbase;
    d.seg0 -= sbase;
    q.tiles.push_back(d);
  }
  q.segs.assign(p.segs.begin() + sbase, p.segs.begin() + send);
  q.panel_len = std::max<int64_t>(pend - pbase, p.vec);
  // ---- t rows the owned tiles read, and the V groups that make them -------------------
  std::vector<uint8_t> need(static_cast<size_t>(std::max<int64_t>(p.R, 1)), 0);
  for (const Seg &g : q.segs)
    if (g.vec_off >= p.x_len)
      std::fill(need.begin() + (g.vec_off - p.x_len), need.begin() + (g.vec_off - p.x_len + g.ncols), 1);
  struct Copy {
    int64_t src, dst, len;
  };
  std::vector<Copy> copies;
  int64_t voff = 0;
  for (const VGroup &g : p.vgroups) {
    const int64_t t0 = g.t_off - p.x_len;
    if (!std::any_of(need.begin() + t0, need.begin() + t0 + g.rows, [](uint8_t v) { return v != 0; })) continue;
    VGroup h = g;
    h.v_off = voff;
    const int64_t len = int64_t{g.rows} * g.stride;
    if (!copies.empty() && copies.back().src + copies.back().len == g.v_off)
      copies.back().len += len;  // runs of consecutive groups: one copy
    else
      copies.push_back(Copy{g.v_off, voff, len});
    voff += len;
    q.vgroups.push_back(h);
  }
  q.v_len = std::max<int64_t>((voff + p.vec - 1) / p.vec * p.vec, p.vec);
  // ---- work partitions of the subset -------------------------------------------------
  q.tile_order.resize(q.tiles.size());
  std::iota(q.tile_order.begin(), q.tile_order.end(), 0);
  std::stable_sort(q.tile_order.begin(), q.tile_order.end(),
                   [&](int32_t a, int32_t b) { return q.tiles[a].ncols > q.tiles[b].ncols; });
  make_units(q, p.unit_rows);
  make_vunits(q, p.vunit_bytes, p.nwarps);
  // ---- device data -------------------------------------------------------------------
  int rc;
  if ((rc = S.dalloc(&S.panels, q.panel_len * es)) || (rc = S.dalloc(&S.vdata, q.v_len * es))) return rc;
  cudaError_t e = cudaMemset(S.vdata, 0, q.v_len * es);
  if (e == cudaSuccess && pend > pbase)
    e = cudaMemcpy(S.panels, static_cast<const char *>(H.panels) + pbase * es, (pend - pbase) * es,
                   cudaMemcpyDeviceToDevice);
  for (size_t c = 0; e == cudaSuccess && c < copies.size(); c++)
    e = cudaMemcpy(static_cast<char *>(S.vdata) + copies[c].dst * es,
                   static_cast<const char *>(H.vdata) + copies[c].src * es, copies[c].len * es,
                   cudaMemcpyDeviceToDevice);
  if (e != cudaSuccess) return cuda_fail(e, "copying the shard's panels and V rows");
  // x arrives in the permuted source order: XT row j is x[j]; owned y rows go
  // to a local vector, row row0 + i at i
  const int64_t n = H.dp.n, m = H.dp.m;
  std::vector<int32_t> smap0(static_cast<size_t>(n)), tmap0(static_cast<size_t>(m), -1);
  std::iota(smap0.begin(), smap0.end(), 0);
  for (int64_t r = S.shard_row0; r < S.shard_row1; r++) tmap0[r] = static_cast<int32_t>(r - S.shard_row0);
  if ((rc = upload_plan(S, tmap0, smap0, H.dp.zero_row))) return rc;
  S.dp.v_dynamic = H.dp.v_dynamic;
  S.plan.unit_rows = p.unit_rows;
  return setup_grids(S);
}

}  // namespace hm

using hm::HMatrix;

extern "C" int hmgpu_hmatrix_shard(const hmgpu_hmatrix *h, int32_t rank, int32_t world, hmgpu_hmatrix **out) {
  if (!h || !out) return hm::fail(HMGPU_ERR_INVALID, "NULL argument");
  *out = nullptr;
  const HMatrix &H = *reinterpret_cast<const HMatrix *>(h);
  if (H.is_shard) return hm::fail(HMGPU_ERR_INVALID, "H is itself a shard");
  if (H.lean) return hm::fail(HMGPU_ERR_INVALID, "a lean mixed H-matrix keeps only its tensor-core copy; shards take the FP32 layout");
  if (world < 1 || rank < 0 || rank >= world) return hm::fail(HMGPU_ERR_INVALID, "need 0 <= rank < world");
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return hm::cuda_fail(e, "cudaGetDevice");
  if (dev != H.device) return hm::fail(HMGPU_ERR_INVALID, "the current device is not the device H was created on");
  hm::PhaseClock clk;
  HMatrix *S = new (std::nothrow) HMatrix();
  if (!S) return hm::fail(HMGPU_ERR_NOMEM, "out of host memory");
  int rc = hm::make_shard(H, rank, world, *S);
  if (rc) {
    delete S;
    return rc;
  }
  S->build_seconds = clk.lap();
  *out = reinterpret_cast<hmgpu_hmatrix *>(S);
  return HMGPU_OK;
}

extern "C" int hmgpu_shard_rows(const hmgpu_hmatrix *s, int64_t *row_begin, int64_t *row_end) {
  if (!s || !row_begin || !row_end) return hm::fail(HMGPU_ERR_INVALID, "NULL argument");
  const HMatrix &S = *reinterpret_cast<const HMatrix *>(s);
  if (!S.is_shard) return hm::fail(HMGPU_ERR_INVALID, "not a shard (hmgpu_hmatrix_shard makes one)");
  *row_begin = S.shard_row0;
  *row_end = S.shard_row1;
  return HMGPU_OK;
}

extern "C" int hmgpu_matvec_shard(hmgpu_hmatrix *s, const void *x_perm, void *y_rows, void *stream) {
  if (!s) return hm::fail(HMGPU_ERR_INVALID, "shard is NULL");
  HMatrix &S = *reinterpret_cast<HMatrix *>(s);
  if (!S.is_shard) return hm::fail(HMGPU_ERR_INVALID, "not a shard (hmgpu_hmatrix_shard makes one)");
  if (!x_perm || !y_rows) return hm::fail(HMGPU_ERR_INVALID, "x or y is NULL");
  const bool f64 = S.opt.precision == HMGPU_F64;
  const bool comp = !f64 && S.opt.compensated;
  int nl = 0;
  cudaError_t e = hm::launch_matvec(f64, comp, S.dp, S.panels, S.vdata, S.xt, x_perm, y_rows, S.grid_v, S.grid_du,
                                    static_cast<cudaStream_t>(stream), nullptr, &nl);
  if (e != cudaSuccess) return hm::cuda_fail(e, "shard matvec launch");
  return HMGPU_OK;
}
