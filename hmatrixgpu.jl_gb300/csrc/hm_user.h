// User kernels: entry functions of the caller's own, compiled at run time by
// NVRTC into the entry kernels of hm_entry.cuh (hm_user.cpp).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include "hm_internal.h"

namespace hm {

constexpr int64_t kUserMaxParams = 64;  // parameters a user kernel may take

// A user kernel's entry kernels, loaded on one device.
struct UserFns {
  CUmodule mod = nullptr;
  CUfunction aca = nullptr, gen_d = nullptr, gen_f = nullptr, sparsify = nullptr;
};

// The entry kernels of `uk` on the current device (its module is loaded on
// the first call per device and kept until hmgpu_user_kernel_free).
int user_functions(const hmgpu_user_kernel *uk, const UserFns **out);

// One launch of a user module's kernel on the legacy default stream, where the
// library's own assembly kernels run: `args` as for cuLaunchKernel.
cudaError_t launch_user(CUfunction f, int grid, int block, void **args);

}  // namespace hm
