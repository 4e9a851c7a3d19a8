// Device-side launchers of libhmgpu (implemented in the .cu files).
#pragma once
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
  int32_t *tmap0 = nullptr;  // 0-based target map, length m
  int32_t *smap0 = nullptr;  // 0-based source map, length n
  int32_t *counter = nullptr;  // tile ticket of the near/U pass
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

// Packing of FP64 row-major block factors into the product layout.
cudaError_t launch_pack_panels(bool f64, const PackJob *jobs, int64_t njobs, const double *dsrc,
                               const double *usrc, void *panels, cudaStream_t stream);
struct VPackJob {
  int64_t src_off, dst_off;
  int32_t n, r, stride, phase;
};
cudaError_t launch_pack_v(bool f64, const VPackJob *jobs, int64_t njobs, const double *vsrc,
                          void *vdata, cudaStream_t stream);

}  // namespace hm

namespace hm {
// Multi-right-hand-side plain product (hm_multi.cu): up to rhs_per_pass()
// right-hand sides per call; xt holds x_len + R rows of rhs_per_pass() values.
int rhs_per_pass();
// Permutation of up to rhs_per_pass() right-hand sides into XT rows (also
// re-arms both ticket counters).
cudaError_t launch_permute_multi(bool f64, const DevPlan &p, const void *X, int64_t ldx, int nr,
                                 void *xt, cudaStream_t s);
// Mixed-precision tensor-core passes (hm_tc.cu), FP32 storage, 32 RHS per pass.
int occupancy_tc();
cudaError_t launch_matvec_tc(const DevPlan &p, const float *panels, const float *vdata, float *xt,
                             int grid, cudaStream_t s, float *Y, int64_t ldy, int nr,
                             cudaEvent_t ev_mid);

int occupancy_du_multi(bool f64);
cudaError_t launch_matvec_multi(bool f64, const DevPlan &p, const void *panels, const void *vdata,
                                void *xt, const void *X, int64_t ldx, int nr, void *Y, int64_t ldy,
                                int grid_v, int grid_du, cudaStream_t s, cudaEvent_t *ev,
                                int *launches);
}  // namespace hm
