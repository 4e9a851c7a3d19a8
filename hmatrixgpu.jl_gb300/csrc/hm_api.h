// The H-matrix object behind the opaque hmgpu_hmatrix handle.
#pragma once
#include <chrono>
#include <cuda_runtime.h>

#include <array>
#include <vector>

#include "hm_device.h"

namespace hm {

struct HMatrix;

// Fills panel columns of kind-2 pack jobs (dense blocks generated on the device).
struct DenseGenerator {
  virtual ~DenseGenerator() = default;
  virtual int generate(HMatrix &H, const PackJob *djobs, int64_t njobs) = 0;
};

struct HMatrix {
  int device = 0;
  hmgpu_options opt{HMGPU_F32, 0, 0, 0, nullptr};
  BlockSet bs;
  Plan plan;
  DevPlan dp;
  void *panels = nullptr;  // tile panels, element type of the mode
  void *vdata = nullptr;   // V rows
  void *xt = nullptr;      // XT = [x permuted | t]
  int num_sms = 0, grid_v = 0, grid_du = 0;
  // kept FP64 factors (keep_factors)
  double *u64 = nullptr, *v64 = nullptr;
  std::vector<int64_t> u_src_off, v_src_off;
  // multi-right-hand-side scratch, allocated on first use
  void *xt_multi = nullptr, *p_multi = nullptr;
  void *xt_multi_w[2] = {nullptr, nullptr};  // XT of the 8- and 16-wide passes (xt_multi: 32-wide)
  int grid_du_multi = 0;
  int multi_from = 3;  // right-hand sides from which one multi-RHS pass runs (autotuned)
  // tensor-core copy of the matrix (mixed precision)
  DevTc tc;
  int64_t tc_bytes = 0;
  // staging of hmgpu_matvec_host
  void *io_x = nullptr, *io_y = nullptr;
  size_t io_x_bytes = 0, io_y_bytes = 0;
  cudaStream_t io_stream = nullptr;  // hmgpu_matvec_host: copies and product in order, one wait
  // phase profiling (hmgpu_hmatrix_set_profiling)
  bool profiling = false;
  std::vector<std::array<cudaEvent_t, 4>> prof_ev;
  size_t prof_used = 0;
  int64_t prof_launches = 0;
  double build_seconds = 0.0;
  double build_phase[HMGPU_BUILD_PHASES] = {};  // see hmgpu_hmatrix_build_profile
  int64_t aca_batches = 0, aca_reruns = 0, aca_ws_bytes = 0, aca_continued = 0;
  int64_t device_bytes = 0;
  bool lean = false;  // HMGPU_MIXED with only the tensor-core copy (options.lean)
  std::vector<void *> dev_allocs;
  // batches: first row and first column of every member, then m and n (empty
  // outside batches)
  std::vector<int64_t> member_rows, member_cols;
  // a row shard (hmgpu_hmatrix_shard): owns permuted rows [shard_row0, shard_row1)
  bool is_shard = false;
  int32_t shard_rank = 0, shard_world = 1;
  int64_t shard_row0 = 0, shard_row1 = 0;

  ~HMatrix();
  void release();
  int dalloc(void **p, size_t bytes);
  void dfree(void *p);
  int ensure_io(size_t xbytes, size_t ybytes);
};

int cuda_fail(cudaError_t e, const char *what);

// Seconds since the previous call (the first call starts the clock).
struct PhaseClock {
  std::chrono::steady_clock::time_point t = std::chrono::steady_clock::now();
  double lap() {
    auto n = std::chrono::steady_clock::now();
    double d = std::chrono::duration<double>(n - t).count();
    t = n;
    return d;
  }
};
int setup_grids(HMatrix &H);
int upload_units(HMatrix &H);
int upload_plan(HMatrix &H, const std::vector<int32_t> &tmap0, const std::vector<int32_t> &smap0,
                int64_t zero_row);
int build_tc(HMatrix &H);
// The 8 rank-predictor features of admissible block (x, y) at tolerance eps.
void block_features(const Node &x, const Node &y, double eps, float *f);
int finalize_layout(HMatrix &H, const double *d64, const std::vector<int64_t> &dense_src_off,
                    const void *u_src, const std::vector<int64_t> &u_src_off, const void *v_src,
                    const std::vector<int64_t> &v_src_off, DenseGenerator *gen, bool src32 = false);

}  // namespace hm
