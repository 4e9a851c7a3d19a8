// Host-side planning of the device layout used by the H-matrix product.
//
// The reference's device product (src/mult.jl:41-146) scans every block
// descriptor for every row.  Here the structure is resolved once, at build
// time, into:
//   * row tiles: maximal runs of permuted rows that every block either fully
//     covers or misses (at most kMaxTileRows rows each).  Each tile owns its
//     rows of y, which makes the product deterministic without atomics;
//   * one row-major panel per tile holding every column that touches those
//     rows (dense-block columns, then low-rank U columns), rows padded to 16
//     bytes, with a list of segments telling where each column's vector entry
//     lives in XT = [x | t];
//   * row units: runs of at most kUnitRows rows of one tile, largest first;
//   * the V factors row by row, each row phase-aligned with the permuted x so
//     that a 16-byte load of V pairs with a 16-byte load of x;
//   * a static, byte-balanced split of the V rows over the resident warps.
#include <algorithm>
#include <numeric>

#include "hm_internal.h"

namespace hm {

static constexpr int kMaxTileRows = 128;
static constexpr int64_t kVUnitBytes = 64 * 1024;
static constexpr int32_t kUnitRows = 16;  // rows per near/U unit (2 per warp of 8)
// multi-RHS V items: at most kMVRows rows (the tensor-core items' limit) and
// about kMVEntries stored entries
static constexpr int32_t kMVRows = 64;
static constexpr int64_t kMVEntries = 64 * 1024;
// Row strides are multiples of 4 elements (16 bytes in FP32, 32 in FP64): the
// multi-RHS micro-kernel reads 4 columns per step.
static constexpr int32_t kRowPad = 4;

static inline int64_t round_up(int64_t a, int64_t b) { return (a + b - 1) / b * b; }

void make_units(Plan &p, int32_t unit_rows) {
  p.units.clear();
  p.unit_rows = unit_rows;
  // units of more than 16 rows only for tiles whose entries fit one
  // shared-memory chunk of the near/U pass (16 KB: 1024 16-byte vectors)
  const int64_t chunk_cols = 1024 * static_cast<int64_t>(p.vec);
  for (int32_t ti : p.tile_order) {
    const TileDesc &d = p.tiles[ti];
    const int32_t ur = unit_rows > 16 && d.ld > chunk_cols ? 16 : unit_rows;
    const int32_t parts = (d.m + ur - 1) / ur;
    for (int32_t q = 0; q < parts; q++) {
      // near-equal row runs
      int32_t i0 = static_cast<int32_t>(static_cast<int64_t>(d.m) * q / parts);
      int32_t i1 = static_cast<int32_t>(static_cast<int64_t>(d.m) * (q + 1) / parts);
      p.units.push_back(RowUnit{ti, i0, i1, 0});
    }
  }
}

void make_vunits(Plan &p, int64_t unit_bytes, int nwarps) {
  const int esize = 16 / p.vec;
  p.vunits.clear();
  p.vunit_bytes = unit_bytes;
  std::vector<int64_t> uweight;
  for (const VGroup &g : p.vgroups) {
    // lanes per row: a power of two leaving each lane at least four 16-byte
    // vectors of the row, so that loads overlap (at most a warp per row)
    int32_t nv = g.stride / p.vec, lanes = 1;
    while (lanes * 4 < nv && lanes < 32) lanes *= 2;
    const int64_t row_bytes = static_cast<int64_t>(g.stride) * esize;
    const int32_t rows_per = static_cast<int32_t>(std::max<int64_t>(1, unit_bytes / row_bytes));
    for (int32_t k0 = 0; k0 < g.rows; k0 += rows_per) {
      VUnit u{};
      u.v_off = g.v_off + static_cast<int64_t>(k0) * g.stride;
      u.stride = g.stride;
      u.nrows = std::min(rows_per, g.rows - k0);
      u.x_off = g.x_off;
      u.t_off = g.t_off + k0;
      u.lanes = lanes;
      p.vunits.push_back(u);
      uweight.push_back(row_bytes * u.nrows + 256);
    }
  }
  // static byte-balanced split of the V units over the resident warps
  p.nwarps = std::max(1, nwarps);
  p.warp_begin.assign(p.nwarps + 1, 0);
  const int64_t total = std::accumulate(uweight.begin(), uweight.end(), int64_t(0));
  int64_t acc = 0;
  size_t u = 0;
  for (int w = 0; w < p.nwarps; w++) {
    p.warp_begin[w] = static_cast<int32_t>(u);
    const int64_t goal = total * (w + 1) / p.nwarps;
    while (u < uweight.size() && acc + uweight[u] / 2 <= goal) acc += uweight[u++];
  }
  p.warp_begin[p.nwarps] = static_cast<int32_t>(uweight.size());
}

void make_plan(const BlockSet &bs, int vec, int nwarps, const std::vector<int64_t> &dense_src_off,
               const std::vector<int64_t> &u_src_off, Plan &p) {
  p = Plan();
  p.vec = vec;
  const int64_t m = bs.m, n = bs.n;
  const size_t nd = bs.d_rs.size(), na = bs.a_rs.size();
  p.x_len = round_up(n + 4, vec);

  // ---- source groups: low-rank blocks sharing a source cluster multiply the
  // same x segment, so their V rows are stored (and their t entries numbered)
  // one after another, group by group in order of first appearance ----------
  std::vector<int32_t> gorder;  // low-rank blocks, grouped
  std::vector<int32_t> gstart;  // group boundaries in gorder
  {
    // (source range, block) pairs sorted: each range's blocks form a run in
    // increasing block order, and the run's first block is the range's first
    // appearance; the runs are then ordered by that first block
    std::vector<std::pair<int64_t, int32_t>> sorted(na);
    for (size_t b = 0; b < na; b++)
      sorted[b] = {(static_cast<int64_t>(bs.a_cs[b]) << 32) | static_cast<uint32_t>(bs.a_ce[b]),
                   static_cast<int32_t>(b)};
    std::sort(sorted.begin(), sorted.end());
    std::vector<std::pair<int32_t, int32_t>> runs;  // (first block, start in sorted)
    for (size_t i = 0; i < na; i++)
      if (i == 0 || sorted[i].first != sorted[i - 1].first)
        runs.push_back({sorted[i].second, static_cast<int32_t>(i)});
    std::sort(runs.begin(), runs.end());
    gorder.reserve(na);
    gstart.reserve(runs.size() + 1);
    for (const auto &r : runs) {
      gstart.push_back(static_cast<int32_t>(gorder.size()));
      for (size_t i = static_cast<size_t>(r.second); i < na && sorted[i].first == sorted[r.second].first; i++)
        gorder.push_back(sorted[i].second);
    }
    gstart.push_back(static_cast<int32_t>(na));
  }
  p.t_off.assign(na, 0);
  int64_t R = 0;
  for (int32_t b : gorder) {
    p.t_off[b] = p.x_len + R;
    R += bs.a_r[b];
  }
  p.R = R;
  p.xt_len = round_up(p.x_len + R, vec);

  // ---- row tiles --------------------------------------------------------------
  std::vector<int32_t> cuts;  // every block row boundary, ascending, once
  {
    std::vector<uint8_t> is_cut(static_cast<size_t>(m) + 1, 0);
    is_cut[0] = is_cut[m] = 1;
    for (size_t b = 0; b < nd; b++) is_cut[bs.d_rs[b]] = is_cut[bs.d_re[b]] = 1;
    for (size_t b = 0; b < na; b++) is_cut[bs.a_rs[b]] = is_cut[bs.a_re[b]] = 1;
    for (int64_t i = 0; i <= m; i++)
      if (is_cut[i]) cuts.push_back(static_cast<int32_t>(i));
  }
  std::vector<int32_t> trow0, trows;
  for (size_t i = 0; i + 1 < cuts.size(); i++) {
    int32_t a = cuts[i], len = cuts[i + 1] - cuts[i];
    int32_t parts = (len + kMaxTileRows - 1) / kMaxTileRows;
    for (int32_t q = 0; q < parts; q++) {
      int32_t s = a + static_cast<int32_t>((int64_t)len * q / parts);
      int32_t e = a + static_cast<int32_t>((int64_t)len * (q + 1) / parts);
      trow0.push_back(s);
      trows.push_back(e - s);
    }
  }
  const size_t nt = trow0.size();
  std::vector<int32_t> tile_at(static_cast<size_t>(m) + 1, static_cast<int32_t>(nt));
  for (size_t t = 0; t < nt; t++) tile_at[trow0[t]] = static_cast<int32_t>(t);
  auto tile_of = [&](int32_t row) {  // tile whose row0 == row (row is a cut; m: past the last tile)
    return static_cast<size_t>(tile_at[row]);
  };

  // ---- contributions per tile (CSR): dense blocks first, then low-rank -------
  std::vector<int64_t> cnt(nt + 1, 0);
  for (size_t b = 0; b < nd; b++)
    for (size_t t = tile_of(bs.d_rs[b]); t < nt && trow0[t] < bs.d_re[b]; t++) cnt[t + 1]++;
  for (size_t b = 0; b < na; b++)
    if (bs.a_r[b] > 0)
      for (size_t t = tile_of(bs.a_rs[b]); t < nt && trow0[t] < bs.a_re[b]; t++) cnt[t + 1]++;
  for (size_t t = 0; t < nt; t++) cnt[t + 1] += cnt[t];
  std::vector<int64_t> contrib(cnt[nt]);  // block id; low-rank ids offset by nd
  {
    std::vector<int64_t> fill(cnt.begin(), cnt.end() - 1);
    for (size_t b = 0; b < nd; b++)
      for (size_t t = tile_of(bs.d_rs[b]); t < nt && trow0[t] < bs.d_re[b]; t++)
        contrib[fill[t]++] = static_cast<int64_t>(b);
    for (size_t b = 0; b < na; b++)
      if (bs.a_r[b] > 0)
        for (size_t t = tile_of(bs.a_rs[b]); t < nt && trow0[t] < bs.a_re[b]; t++)
          contrib[fill[t]++] = static_cast<int64_t>(nd + b);
  }

  // ---- panels, segments, pack jobs ---------------------------------------------
  p.tiles.resize(nt);
  p.pjobs.reserve(contrib.size());
  p.segs.reserve(contrib.size());
  int64_t off = 0;
  for (size_t t = 0; t < nt; t++) {
    TileDesc &d = p.tiles[t];
    d.row0 = trow0[t];
    d.m = trows[t];
    d.data_off = off;
    d.seg0 = static_cast<int32_t>(p.segs.size());
    int32_t ncols_total = 0;
    for (int64_t q = cnt[t]; q < cnt[t + 1]; q++) {
      int64_t b = contrib[q];
      ncols_total += b < static_cast<int64_t>(nd) ? bs.d_ce[b] - bs.d_cs[b] : bs.a_r[b - nd];
    }
    d.ld = static_cast<int32_t>(round_up(ncols_total, kRowPad));
    int32_t col = 0;
    for (int64_t q = cnt[t]; q < cnt[t + 1]; q++) {
      int64_t b = contrib[q];
      int32_t ncols, vec_off;
      PackJob j{};
      j.m = d.m;
      j.dst_off = off + col;
      j.dst_ld = d.ld;
      if (b < static_cast<int64_t>(nd)) {
        ncols = bs.d_ce[b] - bs.d_cs[b];
        vec_off = bs.d_cs[b];
        if (dense_src_off[b] >= 0) {
          j.kind = 0;
          j.src_off = dense_src_off[b] + static_cast<int64_t>(d.row0 - bs.d_rs[b]) * ncols;
          j.src_ld = ncols;
        } else {
          j.kind = 2;
          j.row0 = d.row0;
          j.col0 = bs.d_cs[b];
        }
      } else {
        int64_t a = b - nd;
        ncols = bs.a_r[a];
        vec_off = static_cast<int32_t>(p.t_off[a]);
        j.kind = 1;
        j.src_off = u_src_off[a] + static_cast<int64_t>(d.row0 - bs.a_rs[a]) * ncols;
        j.src_ld = ncols;
      }
      j.ncols = ncols;
      p.pjobs.push_back(j);
      if (static_cast<int32_t>(p.segs.size()) > d.seg0 &&
          p.segs.back().vec_off + p.segs.back().ncols == vec_off) {
        p.segs.back().ncols += ncols;  // contiguous in XT: extend the segment
      } else {
        p.segs.push_back(Seg{col, ncols, vec_off, 0});
      }
      col += ncols;
    }
    d.ncols = col;
    d.nseg = static_cast<int32_t>(p.segs.size()) - d.seg0;
    off += static_cast<int64_t>(d.m) * d.ld;
  }
  p.panel_len = std::max<int64_t>(off, vec);

  // ---- near/U units: row runs, tiles with more work first ---------------------------
  std::vector<int32_t> order(nt);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) {
    return static_cast<int64_t>(p.tiles[a].ncols) > static_cast<int64_t>(p.tiles[b].ncols);
  });
  p.tile_order = order;
  make_units(p, kUnitRows);

  // ---- V pass -----------------------------------------------------------------------
  p.v_off.assign(na, 0);
  p.v_stride.assign(na, 0);
  p.v_phase.assign(na, 0);
  int64_t voff = 0;
  for (size_t gi = 0; gi + 1 < gstart.size(); gi++) {
    const int32_t a0 = gorder[gstart[gi]];
    const int32_t nb = bs.a_ce[a0] - bs.a_cs[a0];
    const int32_t ph = bs.a_cs[a0] % vec;
    const int32_t stride = static_cast<int32_t>(round_up(ph + nb, kRowPad));
    const int64_t gbase = voff;
    int32_t rows = 0;
    for (int32_t q = gstart[gi]; q < gstart[gi + 1]; q++) {  // rows of the group, block by block
      const int32_t a = gorder[q];
      p.v_off[a] = voff;
      p.v_stride[a] = stride;
      p.v_phase[a] = ph;
      voff += static_cast<int64_t>(stride) * bs.a_r[a];
      rows += bs.a_r[a];
    }
    if (rows == 0) continue;
    const int64_t t0 = p.t_off[a0];  // the group's t entries are contiguous
    p.vgroups.push_back(VGroup{gbase, stride, rows, bs.a_cs[a0] - ph, static_cast<int32_t>(t0)});
    // multi-RHS items: 128-row blocks, wide ones cut into column pieces
    for (int32_t k0 = 0; k0 < rows; k0 += kMVRows) {
      const int32_t nr = std::min(kMVRows, rows - k0);
      const int64_t pieces0 = std::max<int64_t>(1, (static_cast<int64_t>(nr) * stride + kMVEntries - 1) / kMVEntries);
      const int32_t w = static_cast<int32_t>(round_up((stride + pieces0 - 1) / pieces0, 64));
      const int32_t pieces = (stride + w - 1) / w;
      if (pieces > 1) {
        p.mv_reduce.push_back(MVReduce{static_cast<int32_t>(t0 + k0), nr, static_cast<int32_t>(p.p_rows), pieces});
      }
      for (int32_t j = 0; j < pieces; j++) {
        MVItem it{};
        it.v_off = gbase + static_cast<int64_t>(k0) * stride + static_cast<int64_t>(j) * w;
        it.stride = stride;
        it.nrows = nr;
        it.x_off = bs.a_cs[a0] - ph + j * w;
        it.ncols = std::min(w, stride - j * w);
        it.kind = pieces > 1 ? 1 : 0;
        it.out = pieces > 1 ? static_cast<int32_t>(p.p_rows + static_cast<int64_t>(j) * nr)
                            : static_cast<int32_t>(t0 + k0);
        p.mv_items.push_back(it);
      }
      if (pieces > 1) p.p_rows += static_cast<int64_t>(pieces) * nr;
    }
  }
  p.v_len = round_up(std::max<int64_t>(voff, vec), vec);
  std::stable_sort(p.mv_items.begin(), p.mv_items.end(), [](const MVItem &a, const MVItem &b) {
    return static_cast<int64_t>(a.nrows) * a.ncols > static_cast<int64_t>(b.nrows) * b.ncols;
  });
  make_vunits(p, kVUnitBytes, nwarps);

  // ---- entry counts ------------------------------------------------------------------
  p.dense_entries = 0;
  for (size_t b = 0; b < nd; b++)
    p.dense_entries += static_cast<int64_t>(bs.d_re[b] - bs.d_rs[b]) * (bs.d_ce[b] - bs.d_cs[b]);
  p.far_entries = 0;
  for (size_t a = 0; a < na; a++)
    p.far_entries += static_cast<int64_t>(bs.a_r[a]) *
                     ((bs.a_re[a] - bs.a_rs[a]) + (bs.a_ce[a] - bs.a_cs[a]));
}

void make_tc_plan(const Plan &p, TcPlan &tp) {
  constexpr int32_t kTcRows = 64;  // rows per item: hi and lo stack to the 128 UMMA rows
  tp = TcPlan();
  // bytes of an item: hi and lo, ceil(m / 8) row groups x padded columns x 16 B,
  // then the trailer (64 FP32 row factors and the item's batch member)
  auto item_bytes = [](int32_t m, int32_t ncols) {
    const int64_t npad = ncols > 0 ? round_up(ncols, 16) : 16;
    return int64_t(32) * ((m + 7) / 8) * npad + kTcTrailer;
  };
  int64_t off = 0;
  for (const MVItem &it : p.mv_items) {
    TcItem t{};
    t.a_off = off;
    t.m = it.nrows;
    t.ncols = it.ncols;
    t.map = it.x_off;
    t.out = it.out;
    t.kind = it.kind == 0 ? 1 : 2;
    const int64_t b = item_bytes(t.m, t.ncols);
    off += b;
    tp.v_items.push_back(t);
    tp.v_src.push_back(it.v_off);
  }
  int64_t ncm = 0, ndu = 0;
  for (const TileDesc &d : p.tiles) {
    ncm += d.ncols;
    ndu += (std::max(d.m, 1) + kTcRows - 1) / kTcRows;
  }
  tp.colmap.resize(static_cast<size_t>(ncm));
  tp.du_items.reserve(static_cast<size_t>(ndu));
  tp.du_src.reserve(static_cast<size_t>(ndu));
  int32_t *cm = tp.colmap.data();
  for (size_t ti = 0; ti < p.tiles.size(); ti++) {
    const TileDesc &d = p.tiles[ti];
    const int32_t map = static_cast<int32_t>(cm - tp.colmap.data());
    for (int32_t q = 0; q < d.nseg; q++) {
      const Seg &sg = p.segs[d.seg0 + q];
      for (int32_t j = 0; j < sg.ncols; j++) *cm++ = sg.vec_off + j;
    }
    for (int32_t r0 = 0; r0 < std::max(d.m, 1); r0 += kTcRows) {
      TcItem t{};
      t.a_off = off;
      t.m = std::min(kTcRows, d.m - r0);
      t.ncols = d.ncols;
      t.map = map;
      t.out = static_cast<int32_t>(ti);
      t.kind = 0;
      t.row0 = r0;
      const int64_t b = item_bytes(t.m, t.ncols);
      off += b;
      tp.du_items.push_back(t);
      tp.du_src.push_back(d.data_off + static_cast<int64_t>(r0) * d.ld);
    }
  }
  tp.bytes = std::max<int64_t>(off, 16);
}

// The plan and block set of diag(H_1, ..., H_k) from the members' (batch
// members keep their own layouts; every index is shifted): XT = [x regions of
// all members | t regions of all members], y and x concatenated in member
// order. tmap0 / smap0: the device index maps (smap0 -1 on padding entries);
// panel_base / v_base: where each member's panels and V rows go.
int combine_plans(const std::vector<const Plan *> &plans, const std::vector<const BlockSet *> &sets,
                  int nwarps, Plan &P, BlockSet &bs, std::vector<int32_t> &tmap0,
                  std::vector<int32_t> &smap0, std::vector<int64_t> &panel_base,
                  std::vector<int64_t> &v_base) {
  P = Plan();
  bs = BlockSet();
  // ---- offsets of every member ------------------------------------------------------
  const int32_t count = static_cast<int32_t>(plans.size());
  std::vector<int64_t> row_base(count), col_base(count), x_base(count), t_base(count), p_base(count);
  std::vector<int32_t> seg_base(count);
  panel_base.assign(count, 0);
  v_base.assign(count, 0);
  int64_t rows = 0, cols = 0, X = 0, R = 0, pan = 0, vl = 0, pr = 0;
  int32_t ns = 0;
  for (int32_t k = 0; k < count; k++) {
    const Plan &q = *plans[k];
    row_base[k] = rows;
    col_base[k] = cols;
    x_base[k] = X;
    t_base[k] = R;
    panel_base[k] = pan;
    v_base[k] = vl;
    p_base[k] = pr;
    seg_base[k] = ns;
    rows += sets[k]->m;
    cols += sets[k]->n;
    X += q.x_len;
    R += q.R;
    pan += q.panel_len;
    vl += q.v_len;
    pr += q.p_rows;
    ns += static_cast<int32_t>(q.segs.size());
  }
  if (rows >= (int64_t(1) << 31) || cols >= (int64_t(1) << 31) || X + R >= (int64_t(1) << 31))
    return fail(HMGPU_ERR_INVALID, "batch too large for 32-bit row indices");
  const int64_t T0 = X;

  P.vec = plans[0]->vec;
  P.x_len = X;
  P.R = R;
  P.xt_len = round_up(T0 + R, P.vec);
  P.panel_len = std::max<int64_t>(pan, P.vec);
  P.v_len = std::max<int64_t>(vl, P.vec);
  P.p_rows = pr;
  bs.m = rows;
  bs.n = cols;
  for (int32_t k = 0; k < count; k++) {
    const Plan &q = *plans[k];
    const BlockSet &mb = *sets[k];
    const int64_t xl = q.x_len;
    auto f = [&](int64_t v) { return v < xl ? x_base[k] + v : T0 + t_base[k] + (v - xl); };
    for (TileDesc d : q.tiles) {
      d.data_off += panel_base[k];
      d.row0 += static_cast<int32_t>(row_base[k]);
      d.seg0 += seg_base[k];
      P.tiles.push_back(d);
    }
    for (Seg g : q.segs) {
      g.vec_off = static_cast<int32_t>(f(g.vec_off));
      P.segs.push_back(g);
    }
    for (VGroup g : q.vgroups) {
      g.v_off += v_base[k];
      g.x_off += static_cast<int32_t>(x_base[k]);
      g.t_off = static_cast<int32_t>(f(g.t_off));
      P.vgroups.push_back(g);
    }
    for (MVItem it : q.mv_items) {
      it.v_off += v_base[k];
      it.x_off += static_cast<int32_t>(x_base[k]);
      it.out = static_cast<int32_t>(it.kind == 0 ? f(it.out) : it.out + p_base[k]);
      P.mv_items.push_back(it);
    }
    for (MVReduce r : q.mv_reduce) {
      r.t_row = static_cast<int32_t>(f(r.t_row));
      r.p_row += static_cast<int32_t>(p_base[k]);
      P.mv_reduce.push_back(r);
    }
    P.dense_entries += q.dense_entries;
    P.far_entries += q.far_entries;
    // block set (permuted index space, 1-based maps) for the queries
    for (int64_t i = 0; i < mb.m; i++) bs.tmap.push_back(mb.tmap[i] + row_base[k]);
    for (int64_t j = 0; j < mb.n; j++) bs.smap.push_back(mb.smap[j] + col_base[k]);
    const int32_t rb = static_cast<int32_t>(row_base[k]), cb = static_cast<int32_t>(col_base[k]);
    for (size_t b = 0; b < mb.d_rs.size(); b++) {
      bs.d_rs.push_back(mb.d_rs[b] + rb);
      bs.d_re.push_back(mb.d_re[b] + rb);
      bs.d_cs.push_back(mb.d_cs[b] + cb);
      bs.d_ce.push_back(mb.d_ce[b] + cb);
    }
    for (size_t b = 0; b < mb.a_rs.size(); b++) {
      bs.a_rs.push_back(mb.a_rs[b] + rb);
      bs.a_re.push_back(mb.a_re[b] + rb);
      bs.a_cs.push_back(mb.a_cs[b] + cb);
      bs.a_ce.push_back(mb.a_ce[b] + cb);
      bs.a_r.push_back(mb.a_r[b]);
    }
    bs.aca_rank.insert(bs.aca_rank.end(), mb.aca_rank.begin(), mb.aca_rank.end());
    bs.final_rank.insert(bs.final_rank.end(), mb.final_rank.begin(), mb.final_rank.end());
  }
  // work lists over the whole batch: tiles with more columns first, largest
  // multi-RHS V items first, V units split over the resident warps
  P.tile_order.resize(P.tiles.size());
  std::iota(P.tile_order.begin(), P.tile_order.end(), 0);
  std::stable_sort(P.tile_order.begin(), P.tile_order.end(),
                   [&](int32_t a, int32_t b) { return P.tiles[a].ncols > P.tiles[b].ncols; });
  make_units(P, plans[0]->unit_rows);
  make_vunits(P, plans[0]->vunit_bytes, nwarps);
  std::stable_sort(P.mv_items.begin(), P.mv_items.end(), [](const MVItem &a, const MVItem &b) {
    return static_cast<int64_t>(a.nrows) * a.ncols > static_cast<int64_t>(b.nrows) * b.ncols;
  });

  // index maps: y of member k at rows row_base[k].., x at col_base[k]..
  tmap0.assign(rows, 0);
  smap0.assign(X, -1);
  for (int32_t k = 0; k < count; k++) {
    const BlockSet &mb = *sets[k];
    for (int64_t i = 0; i < mb.m; i++)
      tmap0[row_base[k] + i] = static_cast<int32_t>(mb.tmap[i] - 1 + row_base[k]);
    for (int64_t j = 0; j < mb.n; j++)
      smap0[x_base[k] + j] = static_cast<int32_t>(mb.smap[j] - 1 + col_base[k]);
  }

  return HMGPU_OK;
}

}  // namespace hm
