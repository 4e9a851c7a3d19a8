// On-disk form of an assembled H-matrix: save once, load without assembly.
//
// The file holds the product layout as it lives on the device (plan tables,
// index maps, tile panels and V rows in the storage precision) plus the block
// set for the queries, so a load is a few large copies and no ACA. Layout:
//   "HMGPUH01" | int32 file version, precision, compensated, multi_from,
//   V schedule (1 = tickets) | sections |
//   uint64 FNV-1a of everything before it
// where every section is int64 count + count fixed-size records. The tensor-
// core copy of a mixed-precision matrix is rebuilt on load from the FP32 data.
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "hm_api.h"

using hm::HMatrix;

namespace {

constexpr char kMagic[8] = {'H', 'M', 'G', 'P', 'U', 'H', '0', '1'};
constexpr int32_t kFileVersion = 2;  // layout of what follows the magic

struct Writer {
  FILE *f;
  uint64_t h = 1469598103934665603ull;
  bool ok = true;
  void raw(const void *p, size_t n) {
    const unsigned char *c = static_cast<const unsigned char *>(p);
    for (size_t i = 0; i < n; i++) {
      h ^= c[i];
      h *= 1099511628211ull;
    }
    if (n && std::fwrite(p, 1, n, f) != n) ok = false;
  }
  template <typename T>
  void val(const T &v) {
    raw(&v, sizeof v);
  }
  template <typename T>
  void vec(const std::vector<T> &v) {
    val(static_cast<int64_t>(v.size()));
    raw(v.data(), v.size() * sizeof(T));
  }
};

struct Reader {
  FILE *f;
  int64_t left;  // bytes not read yet
  uint64_t h = 1469598103934665603ull;
  bool ok = true;
  void raw(void *p, size_t n) {
    if (!ok) return;
    if (static_cast<int64_t>(n) > left || (n && std::fread(p, 1, n, f) != n)) {
      ok = false;
      return;
    }
    left -= static_cast<int64_t>(n);
    const unsigned char *c = static_cast<const unsigned char *>(p);
    for (size_t i = 0; i < n; i++) {
      h ^= c[i];
      h *= 1099511628211ull;
    }
  }
  template <typename T>
  void val(T &v) {
    raw(&v, sizeof v);
  }
  template <typename T>
  void vec(std::vector<T> &v) {
    int64_t n = 0;
    val(n);
    if (!ok || n < 0 || n > left / static_cast<int64_t>(sizeof(T))) {  // no larger than the file
      ok = false;
      return;
    }
    v.resize(static_cast<size_t>(n));
    raw(v.data(), v.size() * sizeof(T));
  }
};

// bytes of a device array, staged through the host in 64 MiB pieces
bool device_out(Writer &w, const void *d, int64_t bytes) {
  std::vector<unsigned char> buf(static_cast<size_t>(std::min<int64_t>(bytes, 64 << 20)));
  for (int64_t o = 0; o < bytes; o += static_cast<int64_t>(buf.size())) {
    const size_t n = static_cast<size_t>(std::min<int64_t>(buf.size(), bytes - o));
    if (cudaMemcpy(buf.data(), static_cast<const char *>(d) + o, n, cudaMemcpyDeviceToHost) != cudaSuccess)
      return false;
    w.raw(buf.data(), n);
  }
  return w.ok;
}

bool device_in(Reader &r, void *d, int64_t bytes) {
  std::vector<unsigned char> buf(static_cast<size_t>(std::min<int64_t>(bytes, 64 << 20)));
  for (int64_t o = 0; o < bytes; o += static_cast<int64_t>(buf.size())) {
    const size_t n = static_cast<size_t>(std::min<int64_t>(buf.size(), bytes - o));
    r.raw(buf.data(), n);
    if (!r.ok) return false;
    if (cudaMemcpy(static_cast<char *>(d) + o, buf.data(), n, cudaMemcpyHostToDevice) != cudaSuccess)
      return false;
  }
  return true;
}

}  // namespace

extern "C" int hmgpu_hmatrix_save(const hmgpu_hmatrix *h, const char *path) {
  if (!h || !path) return hm::fail(HMGPU_ERR_INVALID, "NULL argument");
  const HMatrix &H = *reinterpret_cast<const HMatrix *>(h);
  if (H.is_shard) return hm::fail(HMGPU_ERR_INVALID, "a shard has no file form; save the whole H-matrix");
  if (H.lean)
    return hm::fail(HMGPU_ERR_INVALID, "a lean mixed H-matrix keeps only its tensor-core copy, and a file holds the FP32 layout it is packed from");
  const hm::Plan &p = H.plan;
  const hm::BlockSet &b = H.bs;
  const int64_t es = H.opt.precision == HMGPU_F64 ? 8 : 4;
  std::vector<int32_t> tmap0(H.dp.m), smap0(H.dp.n);
  cudaError_t e = cudaMemcpy(tmap0.data(), H.dp.tmap0, tmap0.size() * 4, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(smap0.data(), H.dp.smap0, smap0.size() * 4, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return hm::cuda_fail(e, "reading the index maps");
  std::unique_ptr<FILE, int (*)(FILE *)> f(std::fopen(path, "wb"), std::fclose);
  if (!f) return hm::fail(HMGPU_ERR_INVALID, std::string("cannot open ") + path + " for writing");
  Writer w{f.get()};
  w.raw(kMagic, sizeof kMagic);
  w.val(kFileVersion);
  w.val(H.opt.precision);
  w.val(H.opt.compensated);
  w.val(static_cast<int32_t>(H.multi_from));
  w.val(static_cast<int32_t>(H.dp.v_dynamic ? 1 : 0));
  // block set
  w.val(b.m);
  w.val(b.n);
  w.vec(b.tmap);
  w.vec(b.smap);
  w.vec(b.d_rs);
  w.vec(b.d_re);
  w.vec(b.d_cs);
  w.vec(b.d_ce);
  w.vec(b.a_rs);
  w.vec(b.a_re);
  w.vec(b.a_cs);
  w.vec(b.a_ce);
  w.vec(b.a_r);
  w.vec(b.aca_rank);
  w.vec(b.final_rank);
  // plan
  w.val(static_cast<int32_t>(p.vec));
  w.val(p.x_len);
  w.val(p.R);
  w.val(p.xt_len);
  w.val(p.panel_len);
  w.val(p.v_len);
  w.val(p.p_rows);
  w.val(p.unit_rows);
  w.val(p.vunit_bytes);
  w.val(p.dense_entries);
  w.val(p.far_entries);
  w.vec(p.tiles);
  w.vec(p.segs);
  w.vec(p.tile_order);
  w.vec(p.vgroups);
  w.vec(p.mv_items);
  w.vec(p.mv_reduce);
  // device index maps and data
  w.val(H.dp.zero_row);
  w.vec(tmap0);
  w.vec(smap0);
  if (!device_out(w, H.panels, p.panel_len * es) || !device_out(w, H.vdata, p.v_len * es))
    return hm::fail(HMGPU_ERR_CUDA, "reading the device data");
  const uint64_t sum = w.h;
  w.val(sum);
  if (!w.ok) return hm::fail(HMGPU_ERR_INVALID, std::string("write error on ") + path);
  return HMGPU_OK;
}

extern "C" int hmgpu_hmatrix_load(const char *path, hmgpu_hmatrix **out) {
  if (!path || !out) return hm::fail(HMGPU_ERR_INVALID, "NULL argument");
  *out = nullptr;
  std::unique_ptr<FILE, int (*)(FILE *)> f(std::fopen(path, "rb"), std::fclose);
  if (!f) return hm::fail(HMGPU_ERR_INVALID, std::string("cannot open ") + path);
  std::fseek(f.get(), 0, SEEK_END);
  const int64_t size = std::ftell(f.get());
  std::fseek(f.get(), 0, SEEK_SET);
  Reader r{f.get(), size};
  char magic[8];
  r.raw(magic, sizeof magic);
  if (!r.ok || std::memcmp(magic, kMagic, sizeof kMagic) != 0)
    return hm::fail(HMGPU_ERR_INVALID, std::string(path) + " is not an hmgpu H-matrix file");
  int32_t abi = 0, multi_from = 0, v_dynamic = 0;
  auto H = std::make_unique<HMatrix>();
  r.val(abi);
  r.val(H->opt.precision);
  r.val(H->opt.compensated);
  r.val(multi_from);
  r.val(v_dynamic);
  if (!r.ok || abi != kFileVersion)
    return hm::fail(HMGPU_ERR_INVALID, std::string(path) + ": written in another file version");
  if (H->opt.precision != HMGPU_F64 && H->opt.precision != HMGPU_F32 && H->opt.precision != HMGPU_MIXED)
    return hm::fail(HMGPU_ERR_INVALID, std::string(path) + ": unknown precision");
  cudaGetDevice(&H->device);
  hm::BlockSet &b = H->bs;
  hm::Plan &p = H->plan;
  r.val(b.m);
  r.val(b.n);
  r.vec(b.tmap);
  r.vec(b.smap);
  r.vec(b.d_rs);
  r.vec(b.d_re);
  r.vec(b.d_cs);
  r.vec(b.d_ce);
  r.vec(b.a_rs);
  r.vec(b.a_re);
  r.vec(b.a_cs);
  r.vec(b.a_ce);
  r.vec(b.a_r);
  r.vec(b.aca_rank);
  r.vec(b.final_rank);
  int32_t vec = 0;
  r.val(vec);
  p.vec = vec;
  r.val(p.x_len);
  r.val(p.R);
  r.val(p.xt_len);
  r.val(p.panel_len);
  r.val(p.v_len);
  r.val(p.p_rows);
  r.val(p.unit_rows);
  r.val(p.vunit_bytes);
  r.val(p.dense_entries);
  r.val(p.far_entries);
  r.vec(p.tiles);
  r.vec(p.segs);
  r.vec(p.tile_order);
  r.vec(p.vgroups);
  r.vec(p.mv_items);
  r.vec(p.mv_reduce);
  int64_t zero_row = 0;
  std::vector<int32_t> tmap0, smap0;
  r.val(zero_row);
  r.vec(tmap0);
  r.vec(smap0);
  if (!r.ok) return hm::fail(HMGPU_ERR_INVALID, std::string(path) + " is truncated");
  // the tables must describe this layout: sizes and every offset checked
  const int64_t es = H->opt.precision == HMGPU_F64 ? 8 : 4;
  const bool f64 = H->opt.precision == HMGPU_F64;
  bool sane = p.vec == (f64 ? 2 : 4) && b.m > 0 && b.n > 0 && static_cast<int64_t>(tmap0.size()) == b.m &&
              static_cast<int64_t>(b.tmap.size()) == b.m && static_cast<int64_t>(b.smap.size()) == b.n &&
              static_cast<int64_t>(smap0.size()) <= p.x_len &&
              static_cast<int64_t>(smap0.size()) >= b.n && p.xt_len >= p.x_len + p.R &&
              zero_row >= 0 && zero_row < p.x_len && p.panel_len > 0 && p.v_len > 0 &&
              p.tile_order.size() == p.tiles.size() &&
              (p.unit_rows == 8 || p.unit_rows == 16 || p.unit_rows == 32 || p.unit_rows == 64) &&
              p.vunit_bytes > 0;
  for (size_t i = 0; sane && i < p.tiles.size(); i++) {
    const hm::TileDesc &d = p.tiles[i];
    sane = d.m > 0 && d.m <= 128 && d.row0 >= 0 && d.row0 + d.m <= b.m && d.ncols >= 0 && d.ld >= d.ncols &&
           d.ld % 4 == 0 && d.data_off >= 0 && d.data_off % p.vec == 0 &&
           d.data_off + static_cast<int64_t>(d.m) * d.ld <= p.panel_len && d.seg0 >= 0 && d.nseg >= 0 &&
           d.nseg <= d.ncols && static_cast<size_t>(d.seg0) + d.nseg <= p.segs.size() && (d.nseg > 0 || d.ncols == 0);
    // segments cover the columns in order, from column 0
    int64_t col = 0;
    for (int32_t q = 0; sane && q < d.nseg; q++) {
      const hm::Seg &g = p.segs[d.seg0 + q];
      sane = g.col0 == col && g.ncols > 0;
      col += g.ncols;
    }
    sane = sane && col == d.ncols;
  }
  for (size_t i = 0; sane && i < p.segs.size(); i++)
    sane = p.segs[i].vec_off >= 0 && p.segs[i].vec_off + static_cast<int64_t>(p.segs[i].ncols) <= p.xt_len;
  for (size_t i = 0; sane && i < p.tile_order.size(); i++)
    sane = p.tile_order[i] >= 0 && static_cast<size_t>(p.tile_order[i]) < p.tiles.size();
  for (size_t i = 0; sane && i < p.vgroups.size(); i++) {
    const hm::VGroup &g = p.vgroups[i];
    sane = g.stride > 0 && g.stride % 4 == 0 && g.rows > 0 && g.v_off >= 0 && g.v_off % p.vec == 0 && g.x_off % p.vec == 0 &&
           g.v_off + static_cast<int64_t>(g.rows) * g.stride <= p.v_len && g.x_off >= 0 &&
           g.x_off + static_cast<int64_t>(g.stride) <= p.x_len && g.t_off >= p.x_len &&
           g.t_off + static_cast<int64_t>(g.rows) <= p.xt_len;
  }
  for (size_t i = 0; sane && i < p.mv_items.size(); i++) {
    const hm::MVItem &it = p.mv_items[i];
    sane = it.nrows > 0 && it.nrows <= 64 && it.ncols > 0 && it.ncols % 4 == 0 && it.stride >= it.ncols &&
           it.stride % 4 == 0 && it.v_off >= 0 && it.v_off % p.vec == 0 &&
           it.v_off + static_cast<int64_t>(it.nrows - 1) * it.stride + it.ncols <= p.v_len && it.x_off >= 0 &&
           it.x_off + static_cast<int64_t>(it.ncols) <= p.x_len &&
           (it.kind == 0 ? it.out >= p.x_len && it.out + static_cast<int64_t>(it.nrows) <= p.xt_len
                         : it.kind == 1 && it.out >= 0 && it.out + static_cast<int64_t>(it.nrows) <= p.p_rows);
  }
  for (size_t i = 0; sane && i < p.mv_reduce.size(); i++) {
    const hm::MVReduce &q = p.mv_reduce[i];
    sane = q.nrows > 0 && q.npieces > 0 && q.t_row >= p.x_len && q.t_row + static_cast<int64_t>(q.nrows) <= p.xt_len &&
           q.p_row >= 0 && q.p_row + static_cast<int64_t>(q.npieces) * q.nrows <= p.p_rows;
  }
  for (size_t i = 0; sane && i < tmap0.size(); i++) sane = tmap0[i] >= 0 && tmap0[i] < b.m;
  for (size_t i = 0; sane && i < smap0.size(); i++) sane = smap0[i] >= -1 && smap0[i] < b.n;
  if (!sane) return hm::fail(HMGPU_ERR_INVALID, std::string(path) + ": inconsistent tables");
  int rc;
  if ((rc = hm::setup_grids(*H))) return rc;
  hm::make_units(p, p.unit_rows);
  hm::make_vunits(p, p.vunit_bytes, H->grid_v * (hm::kThreads / 32));
  H->multi_from = multi_from >= 2 ? multi_from : 3;
  if ((rc = H->dalloc(&H->panels, p.panel_len * es)) || (rc = H->dalloc(&H->vdata, p.v_len * es))) return rc;
  if (!device_in(r, H->panels, p.panel_len * es) || !device_in(r, H->vdata, p.v_len * es))
    return hm::fail(HMGPU_ERR_INVALID, std::string(path) + ": truncated device data");
  const uint64_t want = r.h;
  uint64_t sum = 0;
  r.val(sum);
  if (!r.ok || sum != want) return hm::fail(HMGPU_ERR_INVALID, std::string(path) + ": checksum mismatch");
  if ((rc = hm::upload_plan(*H, tmap0, smap0, zero_row))) return rc;
  H->dp.v_dynamic = v_dynamic != 0;
  if (H->opt.precision == HMGPU_MIXED && (rc = hm::build_tc(*H))) return rc;
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return hm::cuda_fail(e, "loading an H-matrix");
  *out = reinterpret_cast<hmgpu_hmatrix *>(H.release());
  return HMGPU_OK;
}
