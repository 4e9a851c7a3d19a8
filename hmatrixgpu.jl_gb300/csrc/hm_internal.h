// Internal declarations shared by the host (.cpp) and device (.cu) parts of libhmgpu.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/hmgpu.h"
#include "hm_packjob.h"

namespace hm {

// ---- errors -----------------------------------------------------------------
void set_error(const std::string &msg);
int fail(int code, const std::string &msg);

// ---- cluster tree (src/tree.jl) --------------------------------------------------
struct Node {
  int64_t start, end;  // 1-based start, exclusive end, scaled by dims
  int64_t left, right; // children, -1 for none
  double center[3];
  double radius;
  bool leaf;
};

struct Tree {
  int64_t npts = 0, dims = 1;
  std::vector<int64_t> index_map;  // 1-based, length dims*npts
  std::vector<Node> nodes;         // pre-order
};

int build_tree(const double *coords, int64_t npts, int64_t leaf, int64_t dims, Tree &t);
// The same tree built on the current GPU (hm_tree_dev.cu), bit-identical.
int build_tree_device(const double *coords, int64_t npts, int64_t leaf, int64_t dims, Tree &t);
// Pre-order renumbering and dims expansion shared by both builds.
void finish_tree(Tree &t, std::vector<int64_t> &perm, int64_t dims);

// ---- block tree (src/block.jl) ---------------------------------------------------
struct BNode {
  int32_t x, y;         // target node, source node
  int32_t left, right;  // children, -1 for none
  bool adm, dense;
};

struct Blocks {
  std::vector<BNode> nodes;
  std::vector<int32_t> dense;   // pairs (x, y)
  std::vector<int32_t> approx;  // pairs (x, y)
};

void build_blocks(const Tree &X, const Tree &Y, double eta, bool merge, Blocks &b);
// The same block tree built on the current GPU (hm_tree_dev.cu), bit-identical.
int build_blocks_device(const Tree &X, const Tree &Y, double eta, bool merge, Blocks &b);

// ---- the assembled block structure ------------------------------------------------
// Block ranges are 0-based and half-open in permuted index space.
struct BlockSet {
  int64_t m = 0, n = 0;
  std::vector<int64_t> tmap, smap;  // 1-based, as the reference
  // dense blocks, reference order
  std::vector<int32_t> d_rs, d_re, d_cs, d_ce;
  // low-rank blocks, reference order
  std::vector<int32_t> a_rs, a_re, a_cs, a_ce, a_r;
  // per admissible leaf of the block tree (builds only)
  std::vector<int64_t> aca_rank, final_rank;
};

// ---- matvec layout ------------------------------------------------------------------
// A row tile is a run of permuted rows that every block either covers or misses.
// Its panel stores, row-major, every column that touches those rows: the
// columns of the covering dense blocks (vector entries from the permuted x),
// then the rank columns of the covering low-rank blocks (entries from t = V x).
// Rows are padded with zeros to a 16-byte multiple, so each row is one aligned
// stream of 16-byte vectors.
struct TileDesc {
  int64_t data_off;  // element offset of the panel (multiple of the 16-byte vector)
  int32_t row0;      // first permuted row
  int32_t m;         // rows
  int32_t ncols;     // columns
  int32_t ld;        // row stride in elements (ncols rounded up to 16 bytes)
  int32_t seg0;      // first segment
  int32_t nseg;      // segment count
};
static_assert(sizeof(TileDesc) == 32, "TileDesc layout");

// A run of panel columns whose vector entries are contiguous in XT = [x_perm | t].
struct Seg {
  int32_t col0, ncols, vec_off, pad;
};

// A unit of the near/U pass: rows [i0, i1) of one tile, each row a complete
// dot product, so units never share an output.
struct RowUnit {
  int32_t tile, i0, i1, pad;
};

// A unit of the V pass: rows [0, nrows) of one low-rank block, each row a
// phase-aligned run of `stride` elements dotted with XT[x_off : x_off+stride).
struct VUnit {
  int64_t v_off;   // element offset of the first row
  int32_t stride;  // row stride in elements (multiple of the vector width)
  int32_t nrows;
  int32_t x_off;   // XT offset (aligned) matching stored position 0
  int32_t t_off;   // XT offset of the first output
  int32_t lanes;   // lanes per row (power of two <= 32)
  int32_t pad;
};
static_assert(sizeof(VUnit) == 32, "VUnit layout");

// A work item of the multi-right-hand-side V pass: at most 128 rows of one
// source group times one column piece [c, c + ncols) of the group's stored
// columns. Wide groups are cut into pieces of bounded size whose partial
// products go to rows of a scratch array P and are summed in piece order
// afterwards (MVReduce), so every CTA gets similar work and the sums stay
// deterministic.
struct MVItem {
  int64_t v_off;   // element offset of (first row, first column of the piece)
  int32_t stride;  // row stride of the group's V rows
  int32_t nrows;   // <= 128
  int32_t x_off;   // XT row of the piece's first column
  int32_t ncols;   // multiple of 4
  int32_t out;     // first output row: XT row (kind 0) or P row (kind 1)
  int32_t kind;
};
static_assert(sizeof(MVItem) == 32, "MVItem layout");

// t rows [t_row, t_row + nrows) = sum over pieces j (in order) of
// P rows [p_row + j nrows, p_row + (j + 1) nrows).
struct MVReduce {
  int32_t t_row, nrows, p_row, npieces;
};

// A work item of the tensor-core product: a panel of m <= 64 rows and
// ncols columns stored as scaled FP16 (hi, lo) pairs in the UMMA canonical
// K-major layout, 64 columns per chunk (the last chunk rounded up to 16
// columns): chunk c holds hi then lo, each ceil(m / 8) groups of 8 rows x kc
// columns (kc * 16 bytes per group); after the last chunk, 64 FP32 row
// factors that undo the rows' scales. Column j of the panel meets XT row
// map + j (V items) or colmap[map + j] (near/U items). Row tiles of more
// than 64 rows become several items.
struct TcItem {
  int64_t a_off;    // byte offset of chunk 0 in the tensor-core data
  int32_t m, ncols;
  int32_t map;      // XT row of column 0 (V) or colmap offset (near/U)
  int32_t out;      // tile index (kind 0), XT row (kind 1) or P row (kind 2)
  int32_t kind;     // 0: rows of y, 1: t rows of XT, 2: rows of P
  int32_t row0;     // kind 0: first row of the item within its tile
};
static_assert(sizeof(TcItem) == 32, "TcItem layout");
constexpr int kTcTrailer = 68 * 4;  // bytes after an item's chunks: 64 row factors, its batch member, padding

// The V rows of one source group: rows [0, rows) of `stride` stored elements
// at v_off, dotted with XT[x_off, x_off + stride), outputs at XT rows t_off...
struct VGroup {
  int64_t v_off;
  int32_t stride, rows, x_off, t_off;
};

struct Plan {
  int vec = 4;            // elements per 16-byte vector
  int64_t x_len = 0;      // XT x-region length (>= n + 4, multiple of vec)
  int64_t R = 0;          // total rank
  int64_t xt_len = 0;     // x_len + R rounded up
  std::vector<TileDesc> tiles;
  std::vector<Seg> segs;
  int64_t panel_len = 0;
  std::vector<RowUnit> units;  // near/U pass work, largest first
  int32_t unit_rows = 16;      // rows per unit (8, 16, 32 or 64; above 16 only for one-chunk tiles)
  std::vector<int32_t> tile_order;  // tiles by decreasing columns
  std::vector<PackJob> pjobs;
  // V pass
  std::vector<int64_t> v_off, t_off;  // per low-rank block
  std::vector<int32_t> v_stride, v_phase;
  std::vector<VGroup> vgroups;
  std::vector<VUnit> vunits;
  int64_t vunit_bytes = 0;
  std::vector<int32_t> warp_begin;  // nwarps + 1
  int nwarps = 0;
  int64_t v_len = 0;
  // multi-right-hand-side V pass
  std::vector<MVItem> mv_items;     // largest first
  std::vector<MVReduce> mv_reduce;
  int64_t p_rows = 0;               // rows of the partial-product scratch P
  // bytes
  int64_t dense_entries = 0, far_entries = 0;
};

// Builds the layout for a block set; `src_*_off` are per-block offsets of the
// row-major FP64 source factors (dense blocks: -1 when generated from a kernel).
void make_plan(const BlockSet &bs, int vec, int nwarps, const std::vector<int64_t> &dense_src_off,
               const std::vector<int64_t> &u_src_off, Plan &p);

// Near/U row units of `unit_rows` (<= 16) rows over p.tile_order, and the V
// units of about `unit_bytes` with their static split over `nwarps` warps: both
// only partition the stored layout, so they can be rebuilt at any time.
void make_units(Plan &p, int32_t unit_rows);
void make_vunits(Plan &p, int64_t unit_bytes, int nwarps);

// Plan and block set of the block-diagonal batch of several H-matrices (see
// hm_plan.cpp).
int combine_plans(const std::vector<const Plan *> &plans, const std::vector<const BlockSet *> &sets,
                  int nwarps, Plan &P, BlockSet &bs, std::vector<int32_t> &tmap0,
                  std::vector<int32_t> &smap0, std::vector<int64_t> &panel_base,
                  std::vector<int64_t> &v_base);

// Tensor-core layout of a FP32 plan: V items (from the multi-RHS V items),
// near/U items (row tiles, in pieces of at most 64 rows) and the column maps.
struct TcPlan {
  std::vector<TcItem> v_items, du_items;
  std::vector<int64_t> v_src, du_src;  // element offset of each item's FP32 source rows
  std::vector<int32_t> colmap;
  int64_t bytes = 0;                       // tensor-core data size
};
void make_tc_plan(const Plan &p, TcPlan &tp);

}  // namespace hm

// Definitions of the opaque handles declared in hmgpu.h.
struct hmgpu_tree {
  hm::Tree t;
};
struct hmgpu_blocks {
  hm::Blocks b;
};
