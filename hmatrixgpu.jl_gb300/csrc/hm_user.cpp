// User kernels: the reference builds an HMatrix from any matrix K it can index
// (HMatrix(K, X, Y), src/hmatrix.jl:183,195-196 read K[i, j]). Here a caller's
// K[i, j] = f(x_i, y_j) is a CUDA C++ entry function that NVRTC compiles at
// run time into the library's own entry kernels (hm_entry.cuh, the same
// source as the built-in kernels, with HM_USER_ENTRY defined), so a user
// kernel is assembled by the same batched ACA+ on the device, bit for bit as a
// built-in kernel with the same arithmetic would be.
//
// NVRTC is opened at run time (nothing links against it), and the module is
// loaded through the driver entry points the runtime hands out.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <dlfcn.h>
#include <nvrtc.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "hm_api.h"
#include "hm_user.h"

// The entry kernels' sources, embedded by the build (hm_entry.cuh and the
// header it includes).
extern const char hm_src_entry_cuh[];
extern const char hm_src_packjob_h[];

struct hmgpu_user_kernel {
  std::vector<char> cubin;
  std::string aca, gen_d, gen_f, sparsify;  // lowered (mangled) kernel names
  std::mutex mu;
  std::map<int, hm::UserFns> loaded;  // per device
};

namespace hm {

namespace {

struct Nvrtc {
  decltype(&nvrtcCreateProgram) create = nullptr;
  decltype(&nvrtcAddNameExpression) add_name = nullptr;
  decltype(&nvrtcCompileProgram) compile = nullptr;
  decltype(&nvrtcGetProgramLogSize) log_size = nullptr;
  decltype(&nvrtcGetProgramLog) log = nullptr;
  decltype(&nvrtcGetCUBINSize) cubin_size = nullptr;
  decltype(&nvrtcGetCUBIN) cubin = nullptr;
  decltype(&nvrtcGetLoweredName) lowered = nullptr;
  decltype(&nvrtcDestroyProgram) destroy = nullptr;
  decltype(&nvrtcGetErrorString) error = nullptr;
  bool ok = false;
};

// The NVRTC library of the CUDA 13 toolkit: by its soname, else under
// $CUDA_HOME or $CUDA_PATH, else at the toolkit's usual install location.
const Nvrtc &nvrtc() {
  static const Nvrtc api = [] {
    Nvrtc a;
    std::vector<std::string> names = {"libnvrtc.so.13", "libnvrtc.so"};
    for (const char *env : {"CUDA_HOME", "CUDA_PATH"})
      if (const char *root = std::getenv(env)) names.push_back(std::string(root) + "/lib64/libnvrtc.so.13");
    names.push_back("/usr/local/cuda/lib64/libnvrtc.so.13");
    void *h = nullptr;
    for (const std::string &n : names)
      if ((h = dlopen(n.c_str(), RTLD_NOW | RTLD_LOCAL))) break;
    if (!h) return a;
    auto sym = [&](auto &fp, const char *name) { fp = reinterpret_cast<std::decay_t<decltype(fp)>>(dlsym(h, name)); };
    sym(a.create, "nvrtcCreateProgram");
    sym(a.add_name, "nvrtcAddNameExpression");
    sym(a.compile, "nvrtcCompileProgram");
    sym(a.log_size, "nvrtcGetProgramLogSize");
    sym(a.log, "nvrtcGetProgramLog");
    sym(a.cubin_size, "nvrtcGetCUBINSize");
    sym(a.cubin, "nvrtcGetCUBIN");
    sym(a.lowered, "nvrtcGetLoweredName");
    sym(a.destroy, "nvrtcDestroyProgram");
    sym(a.error, "nvrtcGetErrorString");
    a.ok = a.create && a.add_name && a.compile && a.log_size && a.log && a.cubin_size && a.cubin && a.lowered &&
           a.destroy && a.error;
    return a;
  }();
  return api;
}

struct Driver {
  PFN_cuModuleLoadData_v2000 load = nullptr;
  PFN_cuModuleGetFunction_v2000 get = nullptr;
  PFN_cuModuleUnload_v2000 unload = nullptr;
  PFN_cuLaunchKernel_v4000 launch = nullptr;
  bool ok = false;
};

const Driver &driver() {
  static const Driver d = [] {
    Driver r;
    auto get = [](const char *name, unsigned ver) -> void * {
      void *f = nullptr;
      cudaDriverEntryPointQueryResult q;
      if (cudaGetDriverEntryPointByVersion(name, &f, ver, cudaEnableDefault, &q) != cudaSuccess ||
          q != cudaDriverEntryPointSuccess)
        return nullptr;
      return f;
    };
    r.load = reinterpret_cast<PFN_cuModuleLoadData_v2000>(get("cuModuleLoadData", 2000));
    r.get = reinterpret_cast<PFN_cuModuleGetFunction_v2000>(get("cuModuleGetFunction", 2000));
    r.unload = reinterpret_cast<PFN_cuModuleUnload_v2000>(get("cuModuleUnload", 2000));
    r.launch = reinterpret_cast<PFN_cuLaunchKernel_v4000>(get("cuLaunchKernel", 4000));
    r.ok = r.load && r.get && r.unload && r.launch;
    return r;
  }();
  return d;
}

// Integer types and the kernel kinds, from the library's own definitions, for
// a compilation that sees no system header.
std::string prelude() {
  std::string s =
      "typedef long long int64_t;\ntypedef int int32_t;\ntypedef unsigned char uint8_t;\n"
      "typedef unsigned int uint32_t;\ntypedef unsigned long long uint64_t;\n";
  auto def = [&](const char *name, int v) { s += std::string("#define ") + name + " " + std::to_string(v) + "\n"; };
  def("HMGPU_KERNEL_EXPLICIT", HMGPU_KERNEL_EXPLICIT);
  def("HMGPU_KERNEL_LAPLACE3D", HMGPU_KERNEL_LAPLACE3D);
  def("HMGPU_KERNEL_YUKAWA", HMGPU_KERNEL_YUKAWA);
  def("HMGPU_KERNEL_LOG2D", HMGPU_KERNEL_LOG2D);
  def("HMGPU_KERNEL_VECTOR_R", HMGPU_KERNEL_VECTOR_R);
  def("HMGPU_KERNEL_DIPOLAR", HMGPU_KERNEL_DIPOLAR);
  def("HMGPU_KERNEL_USER", HMGPU_KERNEL_USER);
  s += "#define HM_USER_ENTRY 1\n";
  return s;
}

const char *const kNames[4] = {"hm::aca_kernel", "hm::gen_dense_kernel<double>", "hm::gen_dense_kernel<float>",
                               "hm::sparsify_kernel"};

}  // namespace

int user_functions(const hmgpu_user_kernel *ukc, const UserFns **out) {
  auto *uk = const_cast<hmgpu_user_kernel *>(ukc);
  const Driver &d = driver();
  if (!d.ok) return fail(HMGPU_ERR_UNSUPPORTED, "the CUDA driver's module entry points are not available");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaFree(nullptr);  // the device's primary context is current
  if (e != cudaSuccess) return cuda_fail(e, "user kernel: device");
  std::lock_guard<std::mutex> g(uk->mu);
  auto it = uk->loaded.find(dev);
  if (it == uk->loaded.end()) {
    UserFns f;
    if (d.load(&f.mod, uk->cubin.data()) != CUDA_SUCCESS)
      return fail(HMGPU_ERR_CUDA, "user kernel: loading its module failed");
    const std::string *names[4] = {&uk->aca, &uk->gen_d, &uk->gen_f, &uk->sparsify};
    CUfunction *fns[4] = {&f.aca, &f.gen_d, &f.gen_f, &f.sparsify};
    for (int k = 0; k < 4; k++)
      if (d.get(fns[k], f.mod, names[k]->c_str()) != CUDA_SUCCESS) {
        d.unload(f.mod);
        return fail(HMGPU_ERR_CUDA, std::string("user kernel: no function ") + kNames[k] + " in its module");
      }
    it = uk->loaded.emplace(dev, f).first;
  }
  *out = &it->second;
  return HMGPU_OK;
}

cudaError_t launch_user(CUfunction f, int grid, int block, void **args) {
  const Driver &d = driver();
  if (!d.ok || !f) return cudaErrorInvalidDeviceFunction;
  const CUresult r = d.launch(f, static_cast<unsigned>(grid), 1, 1, static_cast<unsigned>(block), 1, 1, 0, nullptr,
                              args, nullptr);
  return r == CUDA_SUCCESS ? cudaGetLastError() : cudaErrorLaunchFailure;
}

}  // namespace hm

extern "C" int hmgpu_user_kernel_compile(const char *source, hmgpu_user_kernel **out, char *log, int64_t log_len) {
  using namespace hm;
  if (!source || !out) return fail(HMGPU_ERR_INVALID, "NULL argument");
  *out = nullptr;
  if (log && log_len > 0) log[0] = '\0';
  if (!std::strstr(source, "hmgpu_entry"))
    return fail(HMGPU_ERR_INVALID, "the source must define __device__ double hmgpu_entry(const double *x, "
                                   "const double *y, const double *p, int a, int b)");
  const Nvrtc &nv = nvrtc();
  if (!nv.ok) return fail(HMGPU_ERR_UNSUPPORTED, "the NVRTC library (libnvrtc.so.13) cannot be loaded");
  // the user's lines keep their own numbers in the compiler's messages
  const std::string src = prelude() + "#line 1 \"user_kernel.cu\"\n" + source + "\n#include \"hm_entry.cuh\"\n";
  const char *hdrs[2] = {hm_src_entry_cuh, hm_src_packjob_h};
  const char *hnames[2] = {"hm_entry.cuh", "hm_packjob.h"};
  nvrtcProgram prog = nullptr;
  if (nv.create(&prog, src.c_str(), "user_kernel.cu", 2, hdrs, hnames) != NVRTC_SUCCESS)
    return fail(HMGPU_ERR_INVALID, "NVRTC could not create the program");
  std::unique_ptr<nvrtcProgram, void (*)(nvrtcProgram *)> hold(&prog, [](nvrtcProgram *p) { nvrtc().destroy(p); });
  for (const char *n : kNames)
    if (nv.add_name(prog, n) != NVRTC_SUCCESS) return fail(HMGPU_ERR_INVALID, "NVRTC name expression");
  // the entries of the built-in kernels are computed without FMA contraction
  // (explicitly rounded FP64 operations); a user kernel gets the same rule
  const char *opts[] = {"--gpu-architecture=sm_103a", "-std=c++17", "--fmad=false"};
  const nvrtcResult cr = nv.compile(prog, 3, opts);
  size_t ls = 0;
  std::string text;
  if (nv.log_size(prog, &ls) == NVRTC_SUCCESS && ls > 1) {
    text.resize(ls);
    nv.log(prog, &text[0]);
    text.resize(std::strlen(text.c_str()));
  }
  if (log && log_len > 0) {
    const size_t n = std::min<size_t>(text.size(), static_cast<size_t>(log_len - 1));
    std::memcpy(log, text.data(), n);
    log[n] = '\0';
  }
  if (cr != NVRTC_SUCCESS) {
    const size_t eol = text.find('\n');
    return fail(HMGPU_ERR_INVALID, std::string("the user kernel does not compile: ") +
                                       (text.empty() ? nv.error(cr) : text.substr(0, eol)));
  }
  auto uk = std::make_unique<hmgpu_user_kernel>();
  size_t nb = 0;
  if (nv.cubin_size(prog, &nb) != NVRTC_SUCCESS || nb == 0) return fail(HMGPU_ERR_INVALID, "NVRTC produced no CUBIN");
  uk->cubin.resize(nb);
  if (nv.cubin(prog, uk->cubin.data()) != NVRTC_SUCCESS) return fail(HMGPU_ERR_INVALID, "NVRTC CUBIN");
  std::string *dst[4] = {&uk->aca, &uk->gen_d, &uk->gen_f, &uk->sparsify};
  for (int k = 0; k < 4; k++) {
    const char *lo = nullptr;
    if (nv.lowered(prog, kNames[k], &lo) != NVRTC_SUCCESS || !lo)
      return fail(HMGPU_ERR_INVALID, std::string("NVRTC lowered name of ") + kNames[k]);
    *dst[k] = lo;
  }
  *out = uk.release();
  return HMGPU_OK;
}

extern "C" int hmgpu_user_kernel_free(hmgpu_user_kernel *uk) {
  if (!uk) return HMGPU_OK;
  const hm::Driver &d = hm::driver();
  int cur = -1;
  cudaGetDevice(&cur);
  for (auto &kv : uk->loaded) {
    if (d.ok && cudaSetDevice(kv.first) == cudaSuccess) d.unload(kv.second.mod);
  }
  if (cur >= 0) cudaSetDevice(cur);
  delete uk;
  return HMGPU_OK;
}
