// C ABI of libhmgpu: H-matrix objects, import of the reference's flattened
// layout, the product entry points and the info/export queries.
#include <algorithm>
#include <chrono>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <numeric>

#include "hm_api.h"


namespace hm {

int cuda_fail(cudaError_t e, const char *what) {
  return fail(HMGPU_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

HMatrix::~HMatrix() {
  for (auto &q : prof_ev)
    for (cudaEvent_t e : q) cudaEventDestroy(e);
  if (io_stream) cudaStreamDestroy(io_stream);
  release();
}

void HMatrix::release() {
  for (void *p : dev_allocs) cudaFree(p);
  dev_allocs.clear();
}

int HMatrix::dalloc(void **p, size_t bytes) {
  *p = nullptr;
  if (bytes == 0) bytes = 16;
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(HMGPU_ERR_NOMEM, "cudaMalloc of " + std::to_string(bytes) + " bytes failed: " +
                                     cudaGetErrorString(e));
  }
  dev_allocs.push_back(*p);
  device_bytes += static_cast<int64_t>(bytes);
  return HMGPU_OK;
}

void HMatrix::dfree(void *p) {
  if (!p) return;
  for (size_t i = 0; i < dev_allocs.size(); i++)
    if (dev_allocs[i] == p) {
      dev_allocs.erase(dev_allocs.begin() + i);
      break;
    }
  cudaFree(p);
}

template <typename V>
static int upload(HMatrix &H, V **dst, const std::vector<V> &src) {
  int rc = H.dalloc(reinterpret_cast<void **>(dst), src.size() * sizeof(V));
  if (rc) return rc;
  if (src.empty()) return HMGPU_OK;
  cudaError_t e = cudaMemcpy(*dst, src.data(), src.size() * sizeof(V), cudaMemcpyHostToDevice);
  return e == cudaSuccess ? HMGPU_OK : cuda_fail(e, "cudaMemcpy");
}

int setup_grids(HMatrix &H) {
  const bool f64 = H.opt.precision == HMGPU_F64;
  const bool comp = !f64 && (H.opt.compensated || H.opt.precision == HMGPU_MIXED);
  cudaDeviceProp prop;
  cudaError_t e = cudaGetDeviceProperties(&prop, H.device);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDeviceProperties");
  H.num_sms = prop.multiProcessorCount;
  H.grid_v = H.num_sms * occupancy_v(f64);
  H.grid_du = H.num_sms * occupancy_du(f64, comp);
  return HMGPU_OK;
}

// Row units, V units and the static V split on the device (rebuilt by the autotuner).
int upload_units(HMatrix &H) {
  const Plan &p = H.plan;
  H.dfree(H.dp.units);
  H.dfree(H.dp.vunits);
  H.dfree(H.dp.warp_begin);
  int rc;
  if ((rc = upload(H, &H.dp.units, p.units))) return rc;
  if ((rc = upload(H, &H.dp.vunits, p.vunits))) return rc;
  if ((rc = upload(H, &H.dp.warp_begin, p.warp_begin))) return rc;
  H.dp.nunits = static_cast<int32_t>(p.units.size());
  H.dp.nvunits = static_cast<int32_t>(p.vunits.size());
  H.dp.nwarps = p.nwarps;
  H.dp.warp_begin_empty = p.vunits.empty();
  return HMGPU_OK;
}

// Every table of H.plan, the index maps (tmap0: length m; smap0: the x region,
// -1 for zero entries) and the ticket/status words; allocates XT.
int upload_plan(HMatrix &H, const std::vector<int32_t> &tmap0, const std::vector<int32_t> &smap0,
                int64_t zero_row) {
  const Plan &p = H.plan;
  const size_t es = H.opt.precision == HMGPU_F64 ? 8 : 4;
  int rc;
  if ((rc = H.dalloc(&H.xt, p.xt_len * es))) return rc;
  cudaMemset(H.xt, 0, p.xt_len * es);
  if ((rc = upload(H, &H.dp.tiles, p.tiles))) return rc;
  if ((rc = upload(H, &H.dp.tile_order, p.tile_order))) return rc;
  if ((rc = upload(H, &H.dp.segs, p.segs))) return rc;
  if ((rc = upload_units(H))) return rc;
  if ((rc = upload(H, &H.dp.tmap0, tmap0))) return rc;
  if ((rc = upload(H, &H.dp.smap0, smap0))) return rc;
  {
    int64_t n_src = 0;
    for (int32_t v : smap0) n_src = std::max<int64_t>(n_src, static_cast<int64_t>(v) + 1);
    std::vector<int32_t> sinv0(n_src, -1);
    for (size_t c = 0; c < smap0.size(); c++)
      if (smap0[c] >= 0) sinv0[smap0[c]] = static_cast<int32_t>(c);
    for (int32_t v : sinv0)
      if (v < 0) return fail(HMGPU_ERR_INVALID, "source map is not a permutation");
    if ((rc = upload(H, &H.dp.sinv0, sinv0))) return rc;
    H.dp.n_src = n_src;
  }
  if ((rc = H.dalloc(reinterpret_cast<void **>(&H.dp.counter), 64))) return rc;
  cudaMemset(H.dp.counter, 0, 64);
  H.dp.status = H.dp.counter + 4;  // its own 16-byte slot of the same allocation
  H.dp.ntiles = static_cast<int32_t>(p.tiles.size());
  {  // device order: by first XT row, so pieces reading the same x rows share them in L2
    std::vector<MVItem> ms = p.mv_items;
    std::stable_sort(ms.begin(), ms.end(), [](const MVItem &a, const MVItem &b) { return a.x_off < b.x_off; });
    if ((rc = upload(H, &H.dp.mv_items, ms))) return rc;
  }
  if ((rc = upload(H, &H.dp.mv_reduce, p.mv_reduce))) return rc;
  H.dp.nmv = static_cast<int32_t>(p.mv_items.size());
  H.dp.nmvr = static_cast<int32_t>(p.mv_reduce.size());
  H.dp.p_rows = p.p_rows;
  H.dp.m = static_cast<int64_t>(tmap0.size());
  H.dp.n = static_cast<int64_t>(smap0.size());
  H.dp.zero_row = zero_row;
  H.dp.x_len = p.x_len;
  H.dp.xt_len = p.xt_len;
  return HMGPU_OK;
}

// Builds the product layout from the block set and the row-major factors held
// on the device (d64: dense, u64/v64: low-rank; per-block offsets). The
// low-rank factors are FP64, or FP32 when src32 (FP32 storage with generated
// dense blocks only).
int finalize_layout(HMatrix &H, const double *d64, const std::vector<int64_t> &dense_src_off,
                    const void *u64, const std::vector<int64_t> &u_src_off, const void *v64,
                    const std::vector<int64_t> &v_src_off, DenseGenerator *gen, bool src32) {
  const bool f64 = H.opt.precision == HMGPU_F64;
  int rc;
  PhaseClock clk;
  if ((rc = setup_grids(H))) return rc;
  const int vec = f64 ? 2 : 4;
  make_plan(H.bs, vec, H.grid_v * (kThreads / 32), dense_src_off, u_src_off, H.plan);
  const Plan &p = H.plan;
  const size_t es = f64 ? 8 : 4;
  if ((rc = H.dalloc(&H.panels, p.panel_len * es))) return rc;
  if ((rc = H.dalloc(&H.vdata, p.v_len * es))) return rc;
  cudaMemset(H.vdata, 0, p.v_len * es);
  std::vector<int32_t> t0(H.bs.m), s0(H.bs.n);
  for (int64_t i = 0; i < H.bs.m; i++) t0[i] = static_cast<int32_t>(H.bs.tmap[i] - 1);
  for (int64_t j = 0; j < H.bs.n; j++) s0[j] = static_cast<int32_t>(H.bs.smap[j] - 1);
  if ((rc = upload_plan(H, t0, s0, H.bs.n))) return rc;
  H.build_phase[4] = clk.lap();
  cudaError_t e;

  // pack panels
  PackJob *djobs = nullptr;
  if ((rc = upload(H, &djobs, p.pjobs))) return rc;
  if (src32 && (f64 || d64)) return fail(HMGPU_ERR_INVALID, "FP32 factors need FP32 storage and generated dense blocks");
  e = launch_pack_panels(f64, src32, djobs, static_cast<int64_t>(p.pjobs.size()), d64, u64, H.panels, 0);
  if (e != cudaSuccess) return cuda_fail(e, "pack panels");
  if (gen) {
    rc = gen->generate(H, djobs, static_cast<int64_t>(p.pjobs.size()));
    if (rc) return rc;
  }
  // pack V rows
  std::vector<VPackJob> vj;
  for (size_t a = 0; a < H.bs.a_r.size(); a++) {
    if (H.bs.a_r[a] == 0) continue;
    VPackJob j;
    j.src_off = v_src_off[a];
    j.dst_off = p.v_off[a];
    j.n = H.bs.a_ce[a] - H.bs.a_cs[a];
    j.r = H.bs.a_r[a];
    j.stride = p.v_stride[a];
    j.phase = p.v_phase[a];
    vj.push_back(j);
  }
  VPackJob *dvj = nullptr;
  if ((rc = upload(H, &dvj, vj))) return rc;
  e = launch_pack_v(f64, src32, dvj, static_cast<int64_t>(vj.size()), v64, H.vdata, 0);
  if (e != cudaSuccess) return cuda_fail(e, "pack V");
  e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return cuda_fail(e, "layout packing");
  H.dfree(djobs);
  H.dfree(dvj);
  H.device_bytes -= static_cast<int64_t>(p.pjobs.size() * sizeof(PackJob) + vj.size() * sizeof(VPackJob));
  H.build_phase[5] = clk.lap();
  if (H.opt.precision == HMGPU_MIXED) {
    rc = build_tc(H);
    if (rc == HMGPU_OK && H.opt.lean) {
      // only the FP16 pairs stay: the FP32 panels, V rows and single-RHS XT go
      const size_t es = 4;
      H.dfree(H.panels);
      H.dfree(H.vdata);
      H.dfree(H.xt);
      H.device_bytes -= static_cast<int64_t>((H.plan.panel_len + H.plan.v_len + H.plan.xt_len) * es);
      H.panels = H.vdata = H.xt = nullptr;
      H.lean = true;
      H.multi_from = 1;  // every product on the tensor cores
    }
    H.build_phase[6] = clk.lap();
    return rc;
  }
  return HMGPU_OK;
}

// Tensor-core copy of a FP32 layout: canonical FP16 (hi, lo) chunks of every
// multi-RHS V item and every row tile (hm_tc.cu), packed from the FP32 panels
// and V rows with power-of-two scales: per rank row from its V row (max and
// 1-norm), then per panel row.
int build_tc(HMatrix &H) {
  TcPlan tp;
  make_tc_plan(H.plan, tp);
  DevTc &t = H.tc;
  int rc;
  if ((rc = H.dalloc(&t.adata, tp.bytes))) return rc;
  H.tc_bytes = tp.bytes;
  // V items run in order of their first XT row, so that the pieces of every
  // level that read the same x rows run close together and share them in L2
  // (the packing below keeps the plan's order).
  std::vector<TcItem> vs = tp.v_items;
  std::stable_sort(vs.begin(), vs.end(), [](const TcItem &a, const TcItem &b) { return a.map < b.map; });
  if ((rc = upload(H, &t.v_items, vs)) || (rc = upload(H, &t.du_items, tp.du_items)) ||
      (rc = upload(H, &t.colmap, tp.colmap)))
    return rc;
  t.reduce = H.dp.mv_reduce;
  t.n_v = static_cast<int32_t>(tp.v_items.size());
  t.n_du = static_cast<int32_t>(tp.du_items.size());
  t.n_reduce = H.dp.nmvr;
  t.ctas = H.num_sms;
  t.xt_rows = H.plan.xt_len;
  // XT row of every P row (the rows of V items cut into column pieces)
  std::vector<int32_t> p2t(static_cast<size_t>(std::max<int64_t>(H.plan.p_rows, 1)), 0);
  for (const MVReduce &D : H.plan.mv_reduce)
    for (int32_t j = 0; j < D.npieces; j++)
      for (int32_t r = 0; r < D.nrows; r++)
        p2t[static_cast<size_t>(D.p_row) + static_cast<size_t>(j) * D.nrows + r] = D.t_row + r;
  // batch members: contiguous source ranges (right-hand-side scales are per
  // member, so a batch's products equal its members' own) and row ranges
  std::vector<int64_t> mcol = H.member_cols, mrow = H.member_rows;
  if (mcol.size() < 2) mcol = {0, H.bs.n}, mrow = {0, H.bs.m};
  t.nmem = static_cast<int32_t>(mcol.size() - 1);
  if ((rc = upload(H, &t.mcol0, mcol))) return rc;
  std::vector<TcPack> vj, dj;
  for (size_t i = 0; i < tp.v_items.size(); i++) {
    const MVItem &it = H.plan.mv_items[i];
    const int32_t trow = it.kind == 0 ? it.out : p2t[static_cast<size_t>(it.out)];
    vj.push_back(TcPack{tp.v_src[i], tp.v_items[i].a_off, it.stride, it.nrows, it.ncols, 1, 0, trow, 0, 0});
  }
  for (size_t i = 0; i < tp.du_items.size(); i++) {
    const TcItem &ti = tp.du_items[i];
    const int64_t row = H.plan.tiles[ti.out].row0;
    const int32_t mem = static_cast<int32_t>(std::upper_bound(mrow.begin(), mrow.end(), row) - mrow.begin()) - 1;
    dj.push_back(TcPack{tp.du_src[i], ti.a_off, H.plan.tiles[ti.out].ld, ti.m, ti.ncols, 0, ti.map, 0,
                        std::max(0, std::min(mem, t.nmem - 1)), 0});
  }
  TcPack *dvj = nullptr, *ddj = nullptr;
  VGroup *dg = nullptr;
  float *sc = nullptr;  // nu | gam | colsc, xt_len each
  const int64_t xr = H.plan.xt_len;
  if ((rc = upload(H, &dvj, vj)) || (rc = upload(H, &ddj, dj)) || (rc = upload(H, &dg, H.plan.vgroups)) ||
      (rc = H.dalloc(reinterpret_cast<void **>(&sc), 3 * xr * sizeof(float))))
    return rc;
  cudaError_t e = cudaMemset(sc, 0, 3 * xr * sizeof(float));
  if (e == cudaSuccess)
    e = launch_tc_scales(dg, static_cast<int64_t>(H.plan.vgroups.size()), static_cast<const float *>(H.vdata), xr,
                         sc, sc + xr, sc + 2 * xr, 0);
  if (e == cudaSuccess)
    e = launch_pack_tc(dvj, static_cast<int64_t>(vj.size()), static_cast<const float *>(H.vdata), t.adata,
                       t.colmap, sc + 2 * xr, sc, sc + xr, 0);
  if (e == cudaSuccess)
    e = launch_pack_tc(ddj, static_cast<int64_t>(dj.size()), static_cast<const float *>(H.panels), t.adata,
                       t.colmap, sc + 2 * xr, sc, sc + xr, 0);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return cuda_fail(e, "tensor-core packing");
  H.dfree(dvj);
  H.dfree(ddj);
  H.dfree(dg);
  H.dfree(sc);
  H.device_bytes -= static_cast<int64_t>((vj.size() + dj.size()) * sizeof(TcPack) +
                                         H.plan.vgroups.size() * sizeof(VGroup) + 3 * xr * sizeof(float));
  return HMGPU_OK;
}

int HMatrix::ensure_io(size_t xbytes, size_t ybytes) {
  int rc;
  if (xbytes > io_x_bytes) {
    dfree(io_x);
    io_x = nullptr;
    io_x_bytes = 0;
    if ((rc = dalloc(&io_x, xbytes))) return rc;
    io_x_bytes = xbytes;
  }
  if (ybytes > io_y_bytes) {
    dfree(io_y);
    io_y = nullptr;
    io_y_bytes = 0;
    if ((rc = dalloc(&io_y, ybytes))) return rc;
    io_y_bytes = ybytes;
  }
  return HMGPU_OK;
}

}  // namespace hm

using hm::HMatrix;

// ---------------------------------------------------------------------------
// import of the reference's flattened HMatrix{Float64}
// ---------------------------------------------------------------------------
static int check_perm(const int64_t *map, int64_t len, const char *name) {
  if (len > 0 && !map) return hm::fail(HMGPU_ERR_INVALID, std::string(name) + " is NULL");
  std::vector<char> seen(len, 0);
  for (int64_t i = 0; i < len; i++) {
    int64_t v = map[i];
    if (v < 1 || v > len || seen[v - 1])
      return hm::fail(HMGPU_ERR_INVALID, std::string(name) + " is not a permutation of 1:" +
                                             std::to_string(len) + " (entry " +
                                             std::to_string(i + 1) + " = " + std::to_string(v) + ")");
    seen[v - 1] = 1;
  }
  return HMGPU_OK;
}

static int copy_table(const int64_t *src, int64_t count, std::vector<int64_t> &dst) {
  dst.resize(count);
  if (count == 0) return HMGPU_OK;
  cudaError_t e = cudaMemcpy(dst.data(), src, count * sizeof(int64_t), cudaMemcpyDefault);
  return e == cudaSuccess ? HMGPU_OK : hm::cuda_fail(e, "reading an index table");
}

extern "C" int hmgpu_hmatrix_import_flat(const hmgpu_options *opt, int64_t m, int64_t n,
                                         const int64_t *target_map, const int64_t *source_map,
                                         const int64_t *dense_idx, int64_t nD,
                                         const double *dense_data, int64_t dense_len,
                                         const int64_t *U_idx, int64_t nA, const double *U_data,
                                         int64_t U_len, const int64_t *V_idx, int64_t R,
                                         const double *V_data, int64_t V_len,
                                         hmgpu_hmatrix **out) {
  auto t0 = std::chrono::steady_clock::now();
  if (!out) return hm::fail(HMGPU_ERR_INVALID, "out is NULL");
  *out = nullptr;
  if (m <= 0 || n <= 0 || m >= (int64_t(1) << 31) || n >= (int64_t(1) << 31))
    return hm::fail(HMGPU_ERR_INVALID, "matrix size out of range");
  if (nD < 0 || nA < 0 || R < 0 || dense_len < 0 || U_len < 0 || V_len < 0)
    return hm::fail(HMGPU_ERR_INVALID, "negative count");
  hmgpu_options o{HMGPU_F32, 0, 0, 0, nullptr};
  if (opt) o = *opt;
  if (o.precision != HMGPU_F64 && o.precision != HMGPU_F32 && o.precision != HMGPU_MIXED)
    return hm::fail(HMGPU_ERR_INVALID, "unknown precision mode");

  std::vector<int64_t> tm, sm, di, ui, vi;
  int rc;
  if ((rc = copy_table(target_map, m, tm)) || (rc = copy_table(source_map, n, sm)) ||
      (rc = copy_table(dense_idx, 5 * nD, di)) || (rc = copy_table(U_idx, 5 * nA, ui)) ||
      (rc = copy_table(V_idx, 3 * R, vi)))
    return rc;
  if ((rc = check_perm(tm.data(), m, "target_index_map"))) return rc;
  if ((rc = check_perm(sm.data(), n, "source_index_map"))) return rc;

  auto H = std::make_unique<HMatrix>();
  H->opt = o;
  cudaGetDevice(&H->device);
  hm::BlockSet &bs = H->bs;
  bs.m = m;
  bs.n = n;
  bs.tmap = tm;
  bs.smap = sm;
  std::vector<int64_t> dsrc(nD), usrc(nA), vsrc(nA);
  for (int64_t b = 0; b < nD; b++) {
    const int64_t *d = &di[5 * b];
    if (d[0] < 1 || d[1] < d[0] || d[1] > m || d[2] < 1 || d[3] < d[2] || d[3] > n)
      return hm::fail(HMGPU_ERR_INVALID, "dense block " + std::to_string(b + 1) + " has an invalid range");
    int64_t len = (d[1] - d[0] + 1) * (d[3] - d[2] + 1);
    if (d[4] < 0 || d[4] + len > dense_len)
      return hm::fail(HMGPU_ERR_INVALID, "dense block " + std::to_string(b + 1) + " offset out of range");
    bs.d_rs.push_back(static_cast<int32_t>(d[0] - 1));
    bs.d_re.push_back(static_cast<int32_t>(d[1]));
    bs.d_cs.push_back(static_cast<int32_t>(d[2] - 1));
    bs.d_ce.push_back(static_cast<int32_t>(d[3]));
    dsrc[b] = d[4];
  }
  int64_t next_row = 1;
  for (int64_t b = 0; b < nA; b++) {
    const int64_t *u = &ui[5 * b];
    if (u[0] < 1 || u[1] < u[0] || u[1] > m)
      return hm::fail(HMGPU_ERR_INVALID, "low-rank block " + std::to_string(b + 1) + " has an invalid row range");
    int64_t r = u[3] - u[2] + 1;
    if (u[2] != next_row || r < 0 || u[3] > R)
      return hm::fail(HMGPU_ERR_INVALID, "low-rank block " + std::to_string(b + 1) +
                                              " has an invalid Vx range (rows 3-4 of U_block_indices)");
    next_row += r;
    int64_t mb = u[1] - u[0] + 1;
    if (u[4] < 0 || u[4] + mb * r > U_len)
      return hm::fail(HMGPU_ERR_INVALID, "low-rank block " + std::to_string(b + 1) + " U offset out of range");
    int64_t cs = -1, ce = -1, voff = 0;
    if (r > 0) {
      const int64_t *v = &vi[3 * (u[2] - 1)];
      cs = v[0];
      ce = v[1];
      voff = v[2];
      if (cs < 1 || ce < cs || ce > n)
        return hm::fail(HMGPU_ERR_INVALID, "V_block_indices has an invalid column range");
      int64_t nb = ce - cs + 1;
      for (int64_t k = 0; k < r; k++) {
        const int64_t *vk = &vi[3 * (u[2] - 1 + k)];
        if (vk[0] != cs || vk[1] != ce || vk[2] != voff + k * nb)
          return hm::fail(HMGPU_ERR_INVALID, "V_block_indices rows of low-rank block " +
                                                  std::to_string(b + 1) + " are inconsistent");
      }
      if (voff < 0 || voff + r * nb > V_len)
        return hm::fail(HMGPU_ERR_INVALID, "low-rank block " + std::to_string(b + 1) + " V offset out of range");
    } else {
      cs = 1;  // a rank-0 block contributes nothing; its columns are irrelevant
      ce = 1;
    }
    bs.a_rs.push_back(static_cast<int32_t>(u[0] - 1));
    bs.a_re.push_back(static_cast<int32_t>(u[1]));
    bs.a_cs.push_back(static_cast<int32_t>(cs - 1));
    bs.a_ce.push_back(static_cast<int32_t>(ce));
    bs.a_r.push_back(static_cast<int32_t>(r));
    usrc[b] = u[4];
    vsrc[b] = voff;
  }
  if (next_row - 1 != R)
    return hm::fail(HMGPU_ERR_INVALID, "sum of ranks differs from the V table length");

  // upload the FP64 factors, then re-lay them out
  double *d64 = nullptr, *u64 = nullptr, *v64 = nullptr;
  if ((rc = H->dalloc(reinterpret_cast<void **>(&d64), dense_len * 8)) ||
      (rc = H->dalloc(reinterpret_cast<void **>(&u64), U_len * 8)) ||
      (rc = H->dalloc(reinterpret_cast<void **>(&v64), V_len * 8)))
    return rc;
  cudaError_t e = cudaSuccess;
  if (dense_len) e = cudaMemcpy(d64, dense_data, dense_len * 8, cudaMemcpyDefault);
  if (e == cudaSuccess && U_len) e = cudaMemcpy(u64, U_data, U_len * 8, cudaMemcpyDefault);
  if (e == cudaSuccess && V_len) e = cudaMemcpy(v64, V_data, V_len * 8, cudaMemcpyDefault);
  if (e != cudaSuccess) return hm::cuda_fail(e, "copying factor data");
  if ((rc = hm::finalize_layout(*H, d64, dsrc, u64, usrc, v64, vsrc, nullptr))) return rc;
  H->dfree(d64);
  H->device_bytes -= dense_len * 8;
  if (o.keep_factors) {
    H->u64 = u64;
    H->v64 = v64;
    H->u_src_off = usrc;
    H->v_src_off = vsrc;
  } else {
    H->dfree(u64);
    H->dfree(v64);
    H->device_bytes -= (U_len + V_len) * 8;
  }
  H->build_seconds =
      std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  *out = reinterpret_cast<hmgpu_hmatrix *>(H.release());
  return HMGPU_OK;
}

// ---------------------------------------------------------------------------
// product
// ---------------------------------------------------------------------------
extern "C" int hmgpu_matvec(hmgpu_hmatrix *h, const void *x, void *y, int64_t nrhs, int64_t ldx,
                            int64_t ldy, void *stream) {
  if (!h) return hm::fail(HMGPU_ERR_INVALID, "H is NULL");
  HMatrix &H = *reinterpret_cast<HMatrix *>(h);
  if (H.is_shard) return hm::fail(HMGPU_ERR_INVALID, "a shard multiplies through hmgpu_matvec_shard only");
  if (nrhs < 0) return hm::fail(HMGPU_ERR_INVALID, "nrhs < 0");
  if (nrhs == 0) return HMGPU_OK;
  if (!x || !y) return hm::fail(HMGPU_ERR_INVALID, "x or y is NULL");
  if (ldx < H.bs.n || ldy < H.bs.m) return hm::fail(HMGPU_ERR_INVALID, "leading dimension too small");
  const bool f64 = H.opt.precision == HMGPU_F64;
  const bool comp = !f64 && (H.opt.compensated || H.opt.precision == HMGPU_MIXED);
  const size_t es = f64 ? 8 : 4;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  auto next_events = [&](cudaEvent_t **ev) -> int {
    *ev = nullptr;
    if (!H.profiling) return HMGPU_OK;
    if (H.prof_used == H.prof_ev.size()) {
      std::array<cudaEvent_t, 4> q;
      for (auto &e : q)
        if (cudaEventCreate(&e) != cudaSuccess) return hm::fail(HMGPU_ERR_CUDA, "cudaEventCreate failed");
      H.prof_ev.push_back(q);
    }
    *ev = H.prof_ev[H.prof_used++].data();
    return HMGPU_OK;
  };
  if (nrhs >= H.multi_from) {
    // several right-hand sides: one pass per rhs_per_pass() columns, the
    // matrix read once per pass (hm_multi.cu); for mixed precision one pass
    // per 64 columns on the tensor cores (hm_tc.cu), 32 wide when at most 32
    // columns remain
    const bool tc = H.opt.precision == HMGPU_MIXED;
    const int per = tc ? hm::kTcMaxRhs : hm::rhs_per_pass();
    int rc;
    if (tc && !H.tc.xts) {
      const int64_t xb = H.plan.xt_len * 2 * 32 * 2;
      if ((rc = H.dalloc(reinterpret_cast<void **>(&H.tc.xts), xb)) ||
          (rc = H.dalloc(reinterpret_cast<void **>(&H.tc.prow),
                         std::max<int64_t>(H.plan.p_rows, 1) * hm::kTcMaxRhs * 4)) ||
          (rc = H.dalloc(reinterpret_cast<void **>(&H.tc.xscale),
                         3 * static_cast<size_t>(H.tc.nmem) * hm::kTcMaxRhs * sizeof(float))))
        return rc;
      cudaMemsetAsync(H.tc.xts, 0, xb, s);
      if (cudaError_t e = hm::encode_xts_map(H.tc, 32)) return hm::cuda_fail(e, "tensor map of XTS");
    }
    if (tc && nrhs > 32 && !H.tc.xts64) {
      const int64_t xb = H.plan.xt_len * 2 * 64 * 2;
      if ((rc = H.dalloc(reinterpret_cast<void **>(&H.tc.xts64), xb))) return rc;
      cudaMemsetAsync(H.tc.xts64, 0, xb, s);
      if (cudaError_t e = hm::encode_xts_map(H.tc, 64)) return hm::cuda_fail(e, "tensor map of XTS");
    }
    if (!tc && !H.xt_multi) {
      if ((rc = H.dalloc(&H.xt_multi, H.plan.xt_len * per * es)) ||
          (rc = H.dalloc(&H.p_multi, std::max<int64_t>(H.plan.p_rows, 1) * per * es)))
        return rc;
      cudaMemsetAsync(H.xt_multi, 0, H.plan.xt_len * per * es, s);
      H.grid_du_multi = H.num_sms * hm::occupancy_du_multi(f64);
    }
    for (int64_t k0 = 0; k0 < nrhs; k0 += per) {
      cudaEvent_t *ev;
      if ((rc = next_events(&ev))) return rc;
      const int nr = static_cast<int>(std::min<int64_t>(per, nrhs - k0));
      int nl = 0;
      cudaError_t e;
      if (tc)  // scaled FP16 (hi, lo) splits on the tensor cores
        e = hm::launch_matvec_tc(H.dp, H.tc, reinterpret_cast<const float *>(static_cast<const char *>(x) + k0 * ldx * es),
                                 ldx, nr, reinterpret_cast<float *>(static_cast<char *>(y) + k0 * ldy * es), ldy,
                                 s, ev, &nl);
      else {
        // each pass width has its own XT (zeroed once): rows that no pass
        // writes (padding, the zero row) must read as zero in that width's layout
        const int w = hm::multi_width(nr);
        void *xt = H.xt_multi;
        if (w < per) {
          void *&xw = H.xt_multi_w[w == 8 ? 0 : 1];
          if (!xw) {
            if ((rc = H.dalloc(&xw, H.plan.xt_len * w * es))) return rc;
            cudaMemsetAsync(xw, 0, H.plan.xt_len * w * es, s);
          }
          xt = xw;
        }
        e = hm::launch_matvec_multi(f64, H.dp, H.panels, H.vdata, xt, H.p_multi,
                                    static_cast<const char *>(x) + k0 * ldx * es, ldx, nr,
                                    static_cast<char *>(y) + k0 * ldy * es, ldy, H.grid_du_multi, s, ev, &nl);
      }
      if (e != cudaSuccess) return hm::cuda_fail(e, "multi-RHS matvec launch");
      if (H.profiling) H.prof_launches += nl;
    }
    return HMGPU_OK;
  }
  for (int64_t k = 0; k < nrhs; k++) {
    cudaEvent_t *ev;
    if (int rc = next_events(&ev)) return rc;
    int nl = 0;
    cudaError_t e = hm::launch_matvec(f64, comp, H.dp, H.panels, H.vdata, H.xt,
                                      static_cast<const char *>(x) + k * ldx * es,
                                      static_cast<char *>(y) + k * ldy * es, H.grid_v, H.grid_du, s,
                                      ev, &nl);
    if (e != cudaSuccess) return hm::cuda_fail(e, "matvec launch");
    if (H.profiling) H.prof_launches += nl;
  }
  return HMGPU_OK;
}

extern "C" int hmgpu_matvec_host(hmgpu_hmatrix *h, const void *x, void *y, int64_t nrhs,
                                 int64_t ldx, int64_t ldy) {
  if (!h) return hm::fail(HMGPU_ERR_INVALID, "H is NULL");
  HMatrix &H = *reinterpret_cast<HMatrix *>(h);
  if (nrhs < 0 || ldx < H.bs.n || ldy < H.bs.m) return hm::fail(HMGPU_ERR_INVALID, "bad sizes");
  if (nrhs == 0) return HMGPU_OK;
  const size_t es = H.opt.precision == HMGPU_F64 ? 8 : 4;
  int rc = H.ensure_io(nrhs * H.bs.n * es, nrhs * H.bs.m * es);
  if (rc) return rc;
  cudaError_t e = cudaSuccess;
  // a blocking stream: ordered after work on the legacy default stream, as the
  // default stream itself would be
  if (!H.io_stream && (e = cudaStreamCreateWithFlags(&H.io_stream, cudaStreamDefault)) != cudaSuccess)
    return hm::cuda_fail(e, "creating the copy stream");
  // copy in, product, copy out on one stream, then one wait (pinned host
  // buffers make both copies asynchronous)
  e = cudaMemcpy2DAsync(H.io_x, H.bs.n * es, x, ldx * es, H.bs.n * es, nrhs, cudaMemcpyDefault, H.io_stream);
  if (e != cudaSuccess) return hm::cuda_fail(e, "copying x to the device");
  rc = hmgpu_matvec(h, H.io_x, H.io_y, nrhs, H.bs.n, H.bs.m, H.io_stream);
  if (rc) return rc;
  e = cudaMemcpy2DAsync(y, ldy * es, H.io_y, H.bs.m * es, H.bs.m * es, nrhs, cudaMemcpyDefault, H.io_stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(H.io_stream);
  if (e != cudaSuccess) return hm::cuda_fail(e, "copying y to the host");
  return HMGPU_OK;
}

// ---------------------------------------------------------------------------
// queries
// ---------------------------------------------------------------------------
extern "C" int hmgpu_hmatrix_build_profile(const hmgpu_hmatrix *h, double *seconds, int32_t n) {
  if (!h || (!seconds && n > 0)) return hm::fail(HMGPU_ERR_INVALID, "NULL argument");
  const HMatrix &H = *reinterpret_cast<const HMatrix *>(h);
  for (int32_t i = 0; i < n && i < HMGPU_BUILD_PHASES; i++) seconds[i] = H.build_phase[i];
  return HMGPU_OK;
}

extern "C" int hmgpu_hmatrix_info(const hmgpu_hmatrix *h, hmgpu_info *info) {
  if (!h || !info) return hm::fail(HMGPU_ERR_INVALID, "NULL argument");
  const HMatrix &H = *reinterpret_cast<const HMatrix *>(h);
  const hm::BlockSet &b = H.bs;
  std::memset(info, 0, sizeof *info);
  info->m = b.m;
  info->n = b.n;
  info->n_dense = static_cast<int64_t>(b.d_rs.size());
  info->n_approx = static_cast<int64_t>(b.a_rs.size());
  int64_t rmin = 0, rmax = 0, dmin = 0, dmax = 0, rt = 0;
  for (size_t a = 0; a < b.a_r.size(); a++) {
    if (a == 0 || b.a_r[a] < rmin) rmin = b.a_r[a];
    if (a == 0 || b.a_r[a] > rmax) rmax = b.a_r[a];
    rt += b.a_r[a];
  }
  for (size_t d = 0; d < b.d_rs.size(); d++) {
    int64_t s = static_cast<int64_t>(b.d_re[d] - b.d_rs[d]) * (b.d_ce[d] - b.d_cs[d]);
    if (d == 0 || s < dmin) dmin = s;
    if (d == 0 || s > dmax) dmax = s;
  }
  info->min_rank = rmin;
  info->max_rank = rmax;
  info->min_dense_size = dmin;
  info->max_dense_size = dmax;
  info->total_rank = rt;
  info->dense_entries = H.plan.dense_entries;
  info->far_entries = H.plan.far_entries;
  double comp = static_cast<double>(H.plan.dense_entries + H.plan.far_entries);
  info->compression_ratio = comp > 0 ? static_cast<double>(b.m) * b.n / comp : 0.0;
  const int64_t es = H.opt.precision == HMGPU_F64 ? 8 : 4;
  info->matrix_bytes = H.lean ? H.tc_bytes : (H.plan.panel_len + H.plan.v_len) * es;
  info->device_bytes = H.device_bytes;
  info->n_tiles = static_cast<int64_t>(H.plan.tiles.size());
  info->precision = H.opt.precision;
  info->build_seconds = H.build_seconds;
  info->aca_batches = H.aca_batches;
  info->aca_reruns = H.aca_reruns;
  info->aca_workspace_bytes = H.aca_ws_bytes;
  info->aca_continued = H.aca_continued;
  return HMGPU_OK;
}

extern "C" int hmgpu_hmatrix_set_profiling(hmgpu_hmatrix *h, int on) {
  if (!h) return hm::fail(HMGPU_ERR_INVALID, "H is NULL");
  HMatrix &H = *reinterpret_cast<HMatrix *>(h);
  H.profiling = on != 0;
  H.prof_used = 0;
  H.prof_launches = 0;
  return HMGPU_OK;
}

extern "C" int hmgpu_hmatrix_phase_times(hmgpu_hmatrix *h, double *ms3, int64_t *launches,
                                         int64_t *products) {
  if (!h) return hm::fail(HMGPU_ERR_INVALID, "H is NULL");
  HMatrix &H = *reinterpret_cast<HMatrix *>(h);
  double acc[3] = {0.0, 0.0, 0.0};
  for (size_t i = 0; i < H.prof_used; i++) {
    cudaError_t e = cudaEventSynchronize(H.prof_ev[i][3]);
    if (e != cudaSuccess) return hm::cuda_fail(e, "cudaEventSynchronize");
    for (int k = 0; k < 3; k++) {
      float t = 0.0f;
      cudaEventElapsedTime(&t, H.prof_ev[i][k], H.prof_ev[i][k + 1]);
      acc[k] += t;
    }
  }
  if (ms3)
    for (int k = 0; k < 3; k++) ms3[k] = acc[k];
  if (launches) *launches = H.prof_launches;
  if (products) *products = static_cast<int64_t>(H.prof_used);
  H.prof_used = 0;
  H.prof_launches = 0;
  return HMGPU_OK;
}

extern "C" int hmgpu_hmatrix_status(hmgpu_hmatrix *h, int *status) {
  if (!h || !status) return hm::fail(HMGPU_ERR_INVALID, "NULL argument");
  HMatrix &H = *reinterpret_cast<HMatrix *>(h);
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return hm::cuda_fail(e, "cudaDeviceSynchronize");
  int32_t v = 0;
  e = cudaMemcpy(&v, H.dp.status, sizeof v, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return hm::cuda_fail(e, "reading the device status");
  *status = v;
  if (v != 0) {
    cudaMemset(H.dp.status, 0, sizeof v);
    return hm::fail(HMGPU_ERR_TIMEOUT, "a bounded device wait expired in a product (code " +
                                           std::to_string(v) + ")");
  }
  return HMGPU_OK;
}

extern "C" int hmgpu_hmatrix_blocks(const hmgpu_hmatrix *h, int64_t *dense_idx,
                                    int64_t *approx_idx) {
  if (!h) return hm::fail(HMGPU_ERR_INVALID, "H is NULL");
  const hm::BlockSet &b = reinterpret_cast<const HMatrix *>(h)->bs;
  if (dense_idx)
    for (size_t d = 0; d < b.d_rs.size(); d++) {
      dense_idx[4 * d] = b.d_rs[d] + 1;
      dense_idx[4 * d + 1] = b.d_re[d];
      dense_idx[4 * d + 2] = b.d_cs[d] + 1;
      dense_idx[4 * d + 3] = b.d_ce[d];
    }
  if (approx_idx)
    for (size_t a = 0; a < b.a_rs.size(); a++) {
      approx_idx[5 * a] = b.a_rs[a] + 1;
      approx_idx[5 * a + 1] = b.a_re[a];
      approx_idx[5 * a + 2] = b.a_cs[a] + 1;
      approx_idx[5 * a + 3] = b.a_ce[a];
      approx_idx[5 * a + 4] = b.a_r[a];
    }
  return HMGPU_OK;
}

extern "C" int hmgpu_hmatrix_index_maps(const hmgpu_hmatrix *h, int64_t *tmap, int64_t *smap) {
  if (!h) return hm::fail(HMGPU_ERR_INVALID, "H is NULL");
  const hm::BlockSet &b = reinterpret_cast<const HMatrix *>(h)->bs;
  if (tmap) std::memcpy(tmap, b.tmap.data(), b.tmap.size() * sizeof(int64_t));
  if (smap) std::memcpy(smap, b.smap.data(), b.smap.size() * sizeof(int64_t));
  return HMGPU_OK;
}

extern "C" int hmgpu_hmatrix_block_factors(const hmgpu_hmatrix *h, int64_t blk, double *U,
                                           double *V) {
  if (!h) return hm::fail(HMGPU_ERR_INVALID, "H is NULL");
  const HMatrix &H = *reinterpret_cast<const HMatrix *>(h);
  if (!H.u64) return hm::fail(HMGPU_ERR_UNSUPPORTED, "factors were not kept (keep_factors = 0)");
  const hm::BlockSet &b = H.bs;
  if (blk < 0 || blk >= static_cast<int64_t>(b.a_r.size()))
    return hm::fail(HMGPU_ERR_INVALID, "block index out of range");
  int64_t mb = b.a_re[blk] - b.a_rs[blk], nb = b.a_ce[blk] - b.a_cs[blk], r = b.a_r[blk];
  cudaError_t e = cudaSuccess;
  if (U && mb * r > 0) e = cudaMemcpy(U, H.u64 + H.u_src_off[blk], mb * r * 8, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && V && nb * r > 0)
    e = cudaMemcpy(V, H.v64 + H.v_src_off[blk], nb * r * 8, cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? HMGPU_OK : hm::cuda_fail(e, "copying factors");
}

extern "C" int hmgpu_hmatrix_aca_ranks(const hmgpu_hmatrix *h, int64_t *aca_rank,
                                       int64_t *final_rank) {
  if (!h) return hm::fail(HMGPU_ERR_INVALID, "H is NULL");
  const hm::BlockSet &b = reinterpret_cast<const HMatrix *>(h)->bs;
  if (aca_rank && !b.aca_rank.empty())
    std::memcpy(aca_rank, b.aca_rank.data(), b.aca_rank.size() * sizeof(int64_t));
  if (final_rank && !b.final_rank.empty())
    std::memcpy(final_rank, b.final_rank.data(), b.final_rank.size() * sizeof(int64_t));
  return HMGPU_OK;
}

extern "C" int hmgpu_hmatrix_free(hmgpu_hmatrix *h) {
  delete reinterpret_cast<HMatrix *>(h);
  return HMGPU_OK;
}
