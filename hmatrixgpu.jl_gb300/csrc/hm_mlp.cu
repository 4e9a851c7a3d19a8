// Learned ACA-rank predictor: an 8 -> 64 -> 64 -> 1 MLP (ReLU, FP32) mapping
// block geometry to the rank plain ACA+ reaches at a tolerance. It is trained
// on ranks the device ACA itself produced, by the kernels below, and used only
// to size the ACA workspace and to group admissible blocks of similar rank
// into the same assembly batch; a block whose ACA does not converge inside
// its predicted workspace is rerun with room for min(m, n) terms, so accuracy
// never depends on the network.
//
// Kernels: forward (one thread per sample, weights in shared memory),
// per-sample backward (activations and their gradients to global scratch),
// per-parameter gradient reduction in a fixed sample order (deterministic),
// and an Adam update.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "hm_api.h"

namespace hm {

constexpr int kIn = 8, kH = 64;
constexpr int kW1 = 0, kB1 = kW1 + kH * kIn, kW2 = kB1 + kH, kB2 = kW2 + kH * kH, kW3 = kB2 + kH,
              kB3 = kW3 + kH, kParams = kB3 + 1;
static_assert(kParams == HMGPU_RANK_MODEL_PARAMS, "parameter count");

struct Model {
  std::vector<float> params, mean, stdv;  // host copies
  float *d_params = nullptr, *d_m = nullptr, *d_v = nullptr, *d_norm = nullptr;  // norm: mean|std
  int64_t step = 0;
  ~Model() {
    cudaFree(d_params);
    cudaFree(d_m);
    cudaFree(d_v);
    cudaFree(d_norm);
  }
};

// Normalised features of sample s into z[8].
__device__ __forceinline__ void load_x(const float *X, const float *norm, int64_t s, float z[kIn]) {
#pragma unroll
  for (int k = 0; k < kIn; k++) z[k] = (X[s * kIn + k] - norm[k]) / norm[kIn + k];
}

__global__ void mlp_forward_kernel(const float *__restrict__ P, const float *__restrict__ norm,
                                   const float *__restrict__ X, int64_t n, float *__restrict__ out) {
  __shared__ float w[kParams];
  __shared__ float nm[2 * kIn];
  for (int i = threadIdx.x; i < kParams; i += blockDim.x) w[i] = P[i];
  for (int i = threadIdx.x; i < 2 * kIn; i += blockDim.x) nm[i] = norm[i];
  __syncthreads();
  for (int64_t s = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; s < n;
       s += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    float z[kIn], h1[kH];
    load_x(X, nm, s, z);
#pragma unroll
    for (int j = 0; j < kH; j++) {
      float a = w[kB1 + j];
#pragma unroll
      for (int k = 0; k < kIn; k++) a = fmaf(w[kW1 + j * kIn + k], z[k], a);
      h1[j] = fmaxf(a, 0.0f);
    }
    float o = w[kB3];
    for (int j = 0; j < kH; j++) {
      float a = w[kB2 + j];
#pragma unroll
      for (int i = 0; i < kH; i++) a = fmaf(w[kW2 + j * kH + i], h1[i], a);
      o = fmaf(w[kW3 + j], fmaxf(a, 0.0f), o);
    }
    out[s] = o;
  }
}

// Per sample: forward, then dL/dout = (out - y) / n; stores z (8), h1 (64),
// dh2 (64) and dh1 (64) for the reduction, and the sample's squared error.
__global__ void mlp_backward_sample_kernel(const float *__restrict__ P, const float *__restrict__ norm,
                                           const float *__restrict__ X, const float *__restrict__ Y,
                                           int64_t n, float *__restrict__ Z, float *__restrict__ H1,
                                           float *__restrict__ H2, float *__restrict__ D2,
                                           float *__restrict__ D1, float *__restrict__ dout,
                                           float *__restrict__ sq) {
  __shared__ float w[kParams];
  __shared__ float nm[2 * kIn];
  for (int i = threadIdx.x; i < kParams; i += blockDim.x) w[i] = P[i];
  for (int i = threadIdx.x; i < 2 * kIn; i += blockDim.x) nm[i] = norm[i];
  __syncthreads();
  const int64_t s = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (s >= n) return;
  float z[kIn], h1[kH], h2[kH];
  load_x(X, nm, s, z);
#pragma unroll
  for (int k = 0; k < kIn; k++) Z[s * kIn + k] = z[k];
  for (int j = 0; j < kH; j++) {
    float a = w[kB1 + j];
#pragma unroll
    for (int k = 0; k < kIn; k++) a = fmaf(w[kW1 + j * kIn + k], z[k], a);
    h1[j] = fmaxf(a, 0.0f);
    H1[s * kH + j] = h1[j];
  }
  float o = w[kB3];
  for (int j = 0; j < kH; j++) {
    float a = w[kB2 + j];
    for (int i = 0; i < kH; i++) a = fmaf(w[kW2 + j * kH + i], h1[i], a);
    h2[j] = fmaxf(a, 0.0f);
    H2[s * kH + j] = h2[j];
    o = fmaf(w[kW3 + j], h2[j], o);
  }
  const float e = o - Y[s];
  sq[s] = e * e;
  const float g = e / static_cast<float>(n);
  dout[s] = g;
  for (int j = 0; j < kH; j++) {
    const float d = h2[j] > 0.0f ? g * w[kW3 + j] : 0.0f;
    D2[s * kH + j] = d;
    h2[j] = d;  // reuse as dh2
  }
  for (int i = 0; i < kH; i++) {
    float a = 0.0f;
    for (int j = 0; j < kH; j++) a = fmaf(h2[j], w[kW2 + j * kH + i], a);
    D1[s * kH + i] = h1[i] > 0.0f ? a : 0.0f;
  }
}

// One thread per parameter: the gradient summed over samples in index order.
__global__ void mlp_grad_reduce_kernel(const float *__restrict__ Z, const float *__restrict__ H1,
                                       const float *__restrict__ H2, const float *__restrict__ D2,
                                       const float *__restrict__ D1, const float *__restrict__ dout,
                                       int64_t n, float *__restrict__ grad) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= kParams) return;
  float g = 0.0f;
  if (p < kB1) {  // W1[j][k]
    const int j = p / kIn, k = p % kIn;
    for (int64_t s = 0; s < n; s++) g = fmaf(D1[s * kH + j], Z[s * kIn + k], g);
  } else if (p < kW2) {
    const int j = p - kB1;
    for (int64_t s = 0; s < n; s++) g += D1[s * kH + j];
  } else if (p < kB2) {  // W2[j][i]
    const int j = (p - kW2) / kH, i = (p - kW2) % kH;
    for (int64_t s = 0; s < n; s++) g = fmaf(D2[s * kH + j], H1[s * kH + i], g);
  } else if (p < kW3) {
    const int j = p - kB2;
    for (int64_t s = 0; s < n; s++) g += D2[s * kH + j];
  } else if (p < kB3) {
    const int j = p - kW3;
    for (int64_t s = 0; s < n; s++) g = fmaf(dout[s], H2[s * kH + j], g);
  } else {
    for (int64_t s = 0; s < n; s++) g += dout[s];
  }
  grad[p] = g;
}

// Adam (Kingma & Ba, 2015) with bias correction.
__global__ void mlp_adam_kernel(float *__restrict__ P, const float *__restrict__ grad,
                                float *__restrict__ m, float *__restrict__ v, float lr, float b1,
                                float b2, float eps, float c1, float c2) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= kParams) return;
  const float g = grad[p];
  m[p] = b1 * m[p] + (1.0f - b1) * g;
  v[p] = b2 * v[p] + (1.0f - b2) * g * g;
  P[p] -= lr * (m[p] / c1) / (sqrtf(v[p] / c2) + eps);
}

// ---------------------------------------------------------------------------
struct Scratch {
  float *X = nullptr, *Y = nullptr, *Z = nullptr, *H1 = nullptr, *H2 = nullptr, *D2 = nullptr,
        *D1 = nullptr, *dout = nullptr, *sq = nullptr, *grad = nullptr;
  ~Scratch() {
    for (float *p : {X, Y, Z, H1, H2, D2, D1, dout, sq, grad}) cudaFree(p);
  }
  int alloc(int64_t n) {
    const int64_t sz[10] = {n * kIn, n, n * kIn, n * kH, n * kH, n * kH, n * kH, n, n, kParams};
    float **dst[10] = {&X, &Y, &Z, &H1, &H2, &D2, &D1, &dout, &sq, &grad};
    for (int i = 0; i < 10; i++)
      if (cudaMalloc(dst[i], std::max<int64_t>(sz[i], 1) * sizeof(float)) != cudaSuccess) {
        cudaGetLastError();
        return fail(HMGPU_ERR_NOMEM, "rank model scratch allocation failed");
      }
    return HMGPU_OK;
  }
};

static int model_upload_norm(Model &M) {
  std::vector<float> nm(2 * kIn);
  for (int k = 0; k < kIn; k++) {
    nm[k] = M.mean[k];
    nm[kIn + k] = M.stdv[k];
  }
  cudaError_t e = cudaMemcpy(M.d_norm, nm.data(), nm.size() * 4, cudaMemcpyHostToDevice);
  return e == cudaSuccess ? HMGPU_OK : cuda_fail(e, "uploading the feature scaling");
}

// Per-sample gradient pass + reduction on scratch already holding X, Y.
static int grad_pass(Model &M, Scratch &S, int64_t n, float *loss) {
  const int tb = 128;
  mlp_backward_sample_kernel<<<static_cast<int>((n + tb - 1) / tb), tb>>>(
      M.d_params, M.d_norm, S.X, S.Y, n, S.Z, S.H1, S.H2, S.D2, S.D1, S.dout, S.sq);
  mlp_grad_reduce_kernel<<<(kParams + 127) / 128, 128>>>(S.Z, S.H1, S.H2, S.D2, S.D1, S.dout, n, S.grad);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "rank model gradient kernels");
  if (loss) {
    std::vector<float> sq(n);
    e = cudaMemcpy(sq.data(), S.sq, n * 4, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "reading the loss");
    double acc = 0.0;
    for (float v : sq) acc += v;
    *loss = static_cast<float>(0.5 * acc / std::max<int64_t>(n, 1));
  }
  return HMGPU_OK;
}

int model_predict_device(const Model &M, const float *dX, int64_t n, float *dout) {
  if (n == 0) return HMGPU_OK;
  mlp_forward_kernel<<<static_cast<int>(std::min<int64_t>((n + 127) / 128, 4096)), 128>>>(
      M.d_params, M.d_norm, dX, n, dout);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? HMGPU_OK : cuda_fail(e, "rank model forward kernel");
}

// Features of admissible block (x, y) at tolerance eps (see hmgpu.h).
void block_features(const Node &x, const Node &y, double eps, float *f) {
  auto lg = [](double v) { return std::log(std::max(v, 1e-30)); };
  const double m = static_cast<double>(x.end - x.start), n = static_cast<double>(y.end - y.start);
  const double dx = x.center[0] - y.center[0], dy = x.center[1] - y.center[1],
               dz = x.center[2] - y.center[2];
  const double dist = std::sqrt(dx * dx + dy * dy + dz * dz);
  f[0] = static_cast<float>(lg(m));
  f[1] = static_cast<float>(lg(n));
  f[2] = static_cast<float>(lg(2.0 * x.radius));
  f[3] = static_cast<float>(lg(2.0 * y.radius));
  f[4] = static_cast<float>(lg(dist));
  f[5] = static_cast<float>(dist / std::max(x.radius + y.radius, 1e-30));
  f[6] = static_cast<float>(std::log10(std::max(eps, 1e-300)));
  f[7] = static_cast<float>(lg(std::min(m, n)));
}

}  // namespace hm

struct hmgpu_rank_model {
  hm::Model M;
};

using namespace hm;

extern "C" int hmgpu_rank_model_create(uint64_t seed, hmgpu_rank_model **out) {
  if (!out) return fail(HMGPU_ERR_INVALID, "out is NULL");
  auto *h = new (std::nothrow) hmgpu_rank_model;
  if (!h) return fail(HMGPU_ERR_NOMEM, "host allocation failed");
  Model &M = h->M;
  M.params.assign(kParams, 0.0f);
  std::mt19937_64 rng(seed);
  auto init = [&](int off, int fan_in, int count) {  // He initialisation for ReLU layers
    std::normal_distribution<float> nd(0.0f, std::sqrt(2.0f / fan_in));
    for (int i = 0; i < count; i++) M.params[off + i] = nd(rng);
  };
  init(kW1, kIn, kH * kIn);
  init(kW2, kH, kH * kH);
  init(kW3, kH, kH);
  M.mean.assign(kIn, 0.0f);
  M.stdv.assign(kIn, 1.0f);
  if (cudaMalloc(&M.d_params, kParams * 4) != cudaSuccess || cudaMalloc(&M.d_m, kParams * 4) != cudaSuccess ||
      cudaMalloc(&M.d_v, kParams * 4) != cudaSuccess || cudaMalloc(&M.d_norm, 2 * kIn * 4) != cudaSuccess) {
    cudaGetLastError();
    delete h;
    return fail(HMGPU_ERR_NOMEM, "rank model device allocation failed");
  }
  cudaMemcpy(M.d_params, M.params.data(), kParams * 4, cudaMemcpyHostToDevice);
  cudaMemset(M.d_m, 0, kParams * 4);
  cudaMemset(M.d_v, 0, kParams * 4);
  if (int rc = model_upload_norm(M)) {
    delete h;
    return rc;
  }
  *out = h;
  return HMGPU_OK;
}

extern "C" int hmgpu_rank_model_free(hmgpu_rank_model *h) {
  delete h;
  return HMGPU_OK;
}

extern "C" int hmgpu_rank_model_params(hmgpu_rank_model *h, float *get, const float *set,
                                       float *norm_get, const float *norm_set) {
  if (!h) return fail(HMGPU_ERR_INVALID, "model is NULL");
  Model &M = h->M;
  if (set) {
    std::memcpy(M.params.data(), set, kParams * 4);
    cudaMemcpy(M.d_params, set, kParams * 4, cudaMemcpyHostToDevice);
  }
  if (norm_set) {
    for (int k = 0; k < kIn; k++) {
      M.mean[k] = norm_set[k];
      M.stdv[k] = norm_set[kIn + k];
    }
    if (int rc = model_upload_norm(M)) return rc;
  }
  if (get) cudaMemcpy(get, M.d_params, kParams * 4, cudaMemcpyDeviceToHost);
  if (norm_get)
    for (int k = 0; k < kIn; k++) {
      norm_get[k] = M.mean[k];
      norm_get[kIn + k] = M.stdv[k];
    }
  return HMGPU_OK;
}

extern "C" int hmgpu_rank_model_gradients(hmgpu_rank_model *h, const float *X, const float *Y,
                                          int64_t n, float *grad, float *loss) {
  if (!h || !X || !Y || n <= 0) return fail(HMGPU_ERR_INVALID, "bad arguments");
  Scratch S;
  if (int rc = S.alloc(n)) return rc;
  cudaMemcpy(S.X, X, n * kIn * 4, cudaMemcpyDefault);
  cudaMemcpy(S.Y, Y, n * 4, cudaMemcpyDefault);
  if (int rc = grad_pass(h->M, S, n, loss)) return rc;
  if (grad) cudaMemcpy(grad, S.grad, kParams * 4, cudaMemcpyDeviceToHost);
  return HMGPU_OK;
}

extern "C" int hmgpu_rank_model_train(hmgpu_rank_model *h, const float *X, const float *Y,
                                      int64_t n, int64_t epochs, int64_t batch, float lr,
                                      uint64_t seed, float *final_loss) {
  if (!h || !X || !Y || n <= 0 || epochs < 0 || batch <= 0)
    return fail(HMGPU_ERR_INVALID, "bad arguments");
  Model &M = h->M;
  // feature scaling from the training set
  for (int k = 0; k < kIn; k++) {
    double s = 0.0, s2 = 0.0;
    for (int64_t i = 0; i < n; i++) {
      s += X[i * kIn + k];
      s2 += static_cast<double>(X[i * kIn + k]) * X[i * kIn + k];
    }
    const double mu = s / n, var = std::max(s2 / n - mu * mu, 0.0);
    M.mean[k] = static_cast<float>(mu);
    M.stdv[k] = static_cast<float>(var > 1e-12 ? std::sqrt(var) : 1.0);
  }
  if (int rc = model_upload_norm(M)) return rc;
  const int64_t b = std::min(batch, n);
  Scratch S;
  if (int rc = S.alloc(b)) return rc;
  std::vector<int64_t> perm(n);
  for (int64_t i = 0; i < n; i++) perm[i] = i;
  std::mt19937_64 rng(seed);
  std::vector<float> bx(b * kIn), by(b);
  for (int64_t ep = 0; ep < epochs; ep++) {
    std::shuffle(perm.begin(), perm.end(), rng);
    for (int64_t s0 = 0; s0 + b <= n; s0 += b) {
      for (int64_t q = 0; q < b; q++) {
        std::memcpy(&bx[q * kIn], &X[perm[s0 + q] * kIn], kIn * 4);
        by[q] = Y[perm[s0 + q]];
      }
      cudaMemcpy(S.X, bx.data(), b * kIn * 4, cudaMemcpyHostToDevice);
      cudaMemcpy(S.Y, by.data(), b * 4, cudaMemcpyHostToDevice);
      if (int rc = grad_pass(M, S, b, nullptr)) return rc;
      M.step++;
      const float b1 = 0.9f, b2 = 0.999f;
      const float c1 = 1.0f - std::pow(b1, static_cast<float>(M.step));
      const float c2 = 1.0f - std::pow(b2, static_cast<float>(M.step));
      mlp_adam_kernel<<<(kParams + 127) / 128, 128>>>(M.d_params, S.grad, M.d_m, M.d_v, lr, b1, b2,
                                                      1e-8f, c1, c2);
    }
  }
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return cuda_fail(e, "rank model training");
  cudaMemcpy(M.params.data(), M.d_params, kParams * 4, cudaMemcpyDeviceToHost);
  if (final_loss) {  // loss over the whole training set
    Scratch F;
    if (int rc = F.alloc(n)) return rc;
    cudaMemcpy(F.X, X, n * kIn * 4, cudaMemcpyDefault);
    cudaMemcpy(F.Y, Y, n * 4, cudaMemcpyDefault);
    if (int rc = grad_pass(M, F, n, final_loss)) return rc;
  }
  return HMGPU_OK;
}

extern "C" int hmgpu_rank_model_predict(hmgpu_rank_model *h, const float *X, int64_t n, float *out) {
  if (!h || !X || !out || n < 0) return fail(HMGPU_ERR_INVALID, "bad arguments");
  if (n == 0) return HMGPU_OK;
  float *dX = nullptr, *dO = nullptr;
  if (cudaMalloc(&dX, n * kIn * 4) != cudaSuccess || cudaMalloc(&dO, n * 4) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(dX);
    return fail(HMGPU_ERR_NOMEM, "prediction buffers");
  }
  cudaMemcpy(dX, X, n * kIn * 4, cudaMemcpyDefault);
  int rc = model_predict_device(h->M, dX, n, dO);
  if (!rc) cudaMemcpy(out, dO, n * 4, cudaMemcpyDeviceToHost);
  cudaFree(dX);
  cudaFree(dO);
  return rc;
}

extern "C" int hmgpu_block_features(const hmgpu_tree *Xh, const hmgpu_tree *Yh, double eta,
                                    double eps, float *out, int64_t *count) {
  if (!Xh || !Yh || !count) return fail(HMGPU_ERR_INVALID, "NULL argument");
  Blocks b;
  build_blocks(Xh->t, Yh->t, eta, true, b);
  const int64_t na = static_cast<int64_t>(b.approx.size() / 2);
  if (out)
    for (int64_t a = 0; a < na; a++)
      block_features(Xh->t.nodes[b.approx[2 * a]], Yh->t.nodes[b.approx[2 * a + 1]], eps, out + a * kIn);
  *count = na;
  return HMGPU_OK;
}
