// Allocation-free single-right-hand-side product.
//
// hmgpu_matvec keeps its scratch (the permuted x and t = V x, and the unit
// ticket of the near/U pass) in buffers the H-matrix handle allocates.
// hmgpu_matvec_noalloc runs the same three kernels with that scratch placed
// in the array below instead, for callers that must not
// allocate device memory while they run products: code being captured into a
// CUDA graph with plain (non-async) allocation forbidden, real-time loops that
// fix their memory footprint up front, and hosts whose allocator is owned by
// another framework. The array is a module global: every GPU that loads this
// library holds it until the process exits.
#include <cuda_runtime.h>

#include <mutex>

#include "hm_api.h"

namespace hm {

constexpr size_t kNoAllocBytes = HMGPU_NOALLOC_SCRATCH_BYTES;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kMaxDevices = 64;
static void *g_scratch_addr[kMaxDevices];
static std::mutex g_scratch_mu;

static inline size_t up256(size_t b) { return (b + 255) / 256 * 256; }

// Device address of the scratch array on `dev` (which must be current),
// looked up once per device.
static int scratch_address(int dev, void **out) {
  if (dev < 0 || dev >= kMaxDevices) return fail(HMGPU_ERR_UNSUPPORTED, "device ordinal too large");
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_addr[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress of the product scratch");
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return HMGPU_OK;
}

}  // namespace hm

extern "C" int hmgpu_matvec_noalloc(hmgpu_hmatrix *h, const void *x, void *y, void *stream) {
  if (!h) return hm::fail(HMGPU_ERR_INVALID, "H is NULL");
  if (!x || !y) return hm::fail(HMGPU_ERR_INVALID, "x or y is NULL");
  hm::HMatrix &H = *reinterpret_cast<hm::HMatrix *>(h);
  if (H.is_shard) return hm::fail(HMGPU_ERR_INVALID, "a shard multiplies through hmgpu_matvec_shard only");
  if (H.lean) return hm::fail(HMGPU_ERR_INVALID, "a lean mixed H-matrix keeps only its tensor-core copy; this entry runs the FP32 single-RHS kernels");
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return hm::cuda_fail(e, "cudaGetDevice");
  if (dev != H.device)
    return hm::fail(HMGPU_ERR_INVALID, "the current device is not the device H was created on");
  const bool f64 = H.opt.precision == HMGPU_F64;
  const bool comp = !f64 && (H.opt.compensated || H.opt.precision == HMGPU_MIXED);
  const size_t es = f64 ? 8 : 4;
  // scratch layout: unit ticket (256 bytes) | XT (permuted x, then t)
  const size_t xt_bytes = hm::up256(static_cast<size_t>(H.plan.xt_len) * es);
  const size_t need = 256 + xt_bytes;
  if (need > hm::kNoAllocBytes)
    return hm::fail(HMGPU_ERR_INVALID,
                    "this H-matrix needs " + std::to_string(need) +
                        " bytes of product scratch; hmgpu_matvec_noalloc has " +
                        std::to_string(hm::kNoAllocBytes) + " (use hmgpu_matvec)");
  void *base = nullptr;
  if (int rc = hm::scratch_address(dev, &base)) return rc;
  char *b = static_cast<char *>(base);
  hm::DevPlan dp = H.dp;
  dp.counter = reinterpret_cast<int32_t *>(b);
  void *xt = b + 256;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // The array keeps whatever the previous call left. The ticket must start at
  // zero (the permutation kernel re-arms it too); the x padding is rewritten by
  // the permutation and every t entry by the V pass before it is read.
  e = cudaMemsetAsync(dp.counter, 0, 256, s);
  if (e != cudaSuccess) return hm::cuda_fail(e, "clearing the product scratch");
  int nl = 0;
  e = hm::launch_matvec(f64, comp, dp, H.panels, H.vdata, xt, x, y, H.grid_v, H.grid_du, s,
                        nullptr, &nl);
  if (e != cudaSuccess) return hm::cuda_fail(e, "matvec launch");
  return HMGPU_OK;
}
