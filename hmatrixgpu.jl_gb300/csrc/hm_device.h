// Device-side launchers of libhmgpu (implemented in the .cu files).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include "hm_internal.h"

namespace hm {

// Device copies of a Plan plus the per-product scratch.
struct DevPlan {
  TileDesc *tiles = nullptr;
  Seg *segs = nullptr;
  int32_t ntiles = 0;
  RowUnit *units = nullptr;      // near/U pass work
  int32_t nunits = 0;
  int32_t *tile_order = nullptr; // tiles by decreasing work (multi-RHS pass)
  VUnit *vunits = nullptr;
  int32_t nvunits = 0;
  int32_t *warp_begin = nullptr;
  int32_t nwarps = 0;
  bool warp_begin_empty = true;  // no V units (no low-rank blocks)
  bool v_dynamic = false;        // V units from a ticket counter instead of warp ranges
  MVItem *mv_items = nullptr;  // multi-RHS V items, largest first
  int32_t nmv = 0;
  MVReduce *mv_reduce = nullptr;
  int32_t nmvr = 0;
  int64_t p_rows = 0;
  int32_t *tmap0 = nullptr;  // 0-based target map, length m
  int32_t *smap0 = nullptr;  // 0-based source map, length n (-1: a zero entry)
  int64_t zero_row = 0;      // an XT row that is always zero
  int32_t *sinv0 = nullptr;  // XT row of each 0-based source index (inverse of smap0)
  int64_t n_src = 0;
  int32_t *counter = nullptr;  // ticket counters of the passes (16 slots)
  int32_t *status = nullptr;   // device error word (0 = ok), see hmgpu_hmatrix_status
  int64_t m = 0, n = 0, x_len = 0, xt_len = 0;
};

constexpr int kThreads = 256;  // threads per CTA of the product kernels

// Resident CTAs per SM of the V pass and of the near/U pass for an element type.
int occupancy_v(bool f64);
int occupancy_du(bool f64, bool comp);

// One product y = H x (single right-hand side) on `stream`:
//   x permutation into XT, V pass (t = V x), near/U pass (y = D x + U t).
// `ev` (optional) receives 4 events recorded before, between and after the
// three phases; returns the number of kernels launched through *launches.
cudaError_t launch_matvec(bool f64, bool comp, const DevPlan &p, const void *panels,
                          const void *vdata, void *xt, const void *x, void *y, int grid_v,
                          int grid_du, cudaStream_t stream, cudaEvent_t *ev, int *launches);

// Packing of row-major block factors into the product layout: FP64 sources,
// or FP32 sources (src32) for FP32 storage.
cudaError_t launch_pack_panels(bool f64, bool src32, const PackJob *jobs, int64_t njobs, const void *dsrc,
                               const void *usrc, void *panels, cudaStream_t stream);
struct VPackJob {
  int64_t src_off, dst_off;
  int32_t n, r, stride, phase;
};
cudaError_t launch_pack_v(bool f64, bool src32, const VPackJob *jobs, int64_t njobs, const void *vsrc,
                          void *vdata, cudaStream_t stream);

}  // namespace hm

namespace hm {
// Multi-right-hand-side plain product (hm_multi.cu): up to rhs_per_pass()
// right-hand sides per call; xt holds x_len + R rows of rhs_per_pass() values.
int rhs_per_pass();
// Width (8, 16 or rhs_per_pass()) of the XT rows of a pass over nr columns.
int multi_width(int nr);
// Mixed-precision tensor-core product (hm_tc.cu), 32 or 64 right-hand sides
// per pass.
struct TcPack {  // one item's FP32 row-major source -> canonical FP16 chunks and row factors
  int64_t src_off, a_off;
  int32_t ld, m, ncols;
  int32_t kind;  // 0: near/U rows (columns scaled through colmap[map + c]), 1: V rows
  int32_t map;   // kind 0: colmap offset of column 0
  int32_t trow;  // kind 1: XT row (rank row) of row 0; rows are consecutive
  int32_t member;  // batch member of the rows (0 outside batches)
  int32_t pad;
};
struct DevTc {
  void *adata = nullptr;  // canonical FP16 (hi, lo) chunks of every item, each with its row factors
  TcItem *v_items = nullptr, *du_items = nullptr;
  int32_t *colmap = nullptr;
  MVReduce *reduce = nullptr;
  uint16_t *xts = nullptr;    // xt_len rows of 32 FP16 hi + 32 FP16 lo (passes of <= 32 columns)
  uint16_t *xts64 = nullptr;  // xt_len rows of 64 FP16 hi + 64 FP16 lo (passes of 33..64 columns)
  float *prow = nullptr;      // partial rows of split V items, 64 values per row
  float *xscale = nullptr;    // per pass and member: max |x_r| bits, sigma_r, 1 / sigma_r (64 words each)
  int64_t *mcol0 = nullptr;   // first source index of each batch member, nmem + 1 entries
  int32_t nmem = 1;           // batch members (1 outside batches)
  int32_t n_v = 0, n_du = 0, n_reduce = 0, ctas = 0;
  int64_t xt_rows = 0;  // rows of either XTS
  CUtensorMap xmap[4];  // tile-load maps of xts and xts64: 64-row boxes, then 8-row boxes (encode_xts_map)
};
constexpr int kTcMaxRhs = 64;  // right-hand sides of the widest pass
size_t tc_smem_bytes(int nr);
// The tile-load map of the XTS of width R (32: xts, 64: xts64), after the
// buffer exists.
cudaError_t encode_xts_map(DevTc &t, int R);
// Scales of the rank rows from the FP32 V rows of every source group: nu
// (max magnitude into [2^14, 2^15)), gam (2^-ceil(log2 of the row's 1-norm))
// at each row's XT row, and colsc (1 / gam on t rows, 1 on x rows; xt_rows).
cudaError_t launch_tc_scales(const VGroup *groups, int64_t ngroups, const float *vdata, int64_t xt_rows,
                             float *nu, float *gam, float *colsc, cudaStream_t s);
cudaError_t launch_pack_tc(const TcPack *jobs, int64_t njobs, const float *src, void *adata, const int32_t *colmap,
                           const float *colsc, const float *nu, const float *gam, cudaStream_t s);
// permutation + split of X, V pass, reduction of pieces, near/U pass over
// nr <= 64 columns (xts64 must exist for nr > 32); ev (optional) gets 4
// events as launch_matvec_multi.
cudaError_t launch_matvec_tc(const DevPlan &p, const DevTc &t, const float *X, int64_t ldx, int nr,
                             float *Y, int64_t ldy, cudaStream_t s, cudaEvent_t *ev, int *launches);

int occupancy_du_multi(bool f64);
// P: partial rows of cut V groups (p_rows x rhs_per_pass() values).
cudaError_t launch_matvec_multi(bool f64, const DevPlan &p, const void *panels, const void *vdata,
                                void *xt, void *P, const void *X, int64_t ldx, int nr, void *Y,
                                int64_t ldy, int grid_du, cudaStream_t s, cudaEvent_t *ev,
                                int *launches);
}  // namespace hm
