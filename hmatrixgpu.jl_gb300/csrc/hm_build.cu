// On-device assembly (placeholder until the batched ACA lands).
#include "hm_api.h"

extern "C" int hmgpu_hmatrix_build(const hmgpu_options *, const hmgpu_kernel *, const hmgpu_tree *,
                                   const hmgpu_tree *, double, double, int, hmgpu_hmatrix **) {
  return hm::fail(HMGPU_ERR_UNSUPPORTED, "not built yet");
}
extern "C" int hmgpu_aca_plus(const double *, int64_t, int64_t, int64_t, double, int64_t, int64_t,
                              double *, double *, int64_t *) {
  return hm::fail(HMGPU_ERR_UNSUPPORTED, "not built yet");
}
extern "C" int hmgpu_svd_recompress(int64_t, int64_t, int64_t, const double *, const double *,
                                    double, double *, double *, int64_t *) {
  return hm::fail(HMGPU_ERR_UNSUPPORTED, "not built yet");
}
