// Learned ACA-rank predictor: an 8 -> 64 -> 64 -> 1 MLP (ReLU) with
// hand-written forward, backward and Adam kernels, trained on the GPU.
//
// Parameters (4801 floats): W1[8][64] b1[64] W2[64][64] b2[64] w3[64] b3.
// Inputs are normalised with per-feature mean / std fixed before training;
// the target is log(1 + ACA rank).  Every reduction over samples runs in a
// fixed order (one thread per parameter), so a training run is reproducible.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <numeric>
#include <random>
#include <vector>

#include "ahx_hmat.hpp"

namespace ahx {
namespace {

constexpr int kIn = 8, kHid = 64;
constexpr int kOffW1 = 0, kOffB1 = kOffW1 + kIn * kHid, kOffW2 = kOffB1 + kHid,
              kOffB2 = kOffW2 + kHid * kHid, kOffW3 = kOffB2 + kHid, kOffB3 = kOffW3 + kHid;
constexpr int kNParams = kOffB3 + 1;  // 4801

__device__ __forceinline__ void load_params(float* sp, const float* __restrict__ p) {
  for (int i = threadIdx.x; i < kNParams; i += blockDim.x) sp[i] = p[i];
  __syncthreads();
}

// forward; optionally keeps Z1, Z2 (pre-activations) for the backward pass
__global__ void mlp_fwd_kernel(const float* __restrict__ X, const uint32_t* __restrict__ idx,
                               uint32_t n, const float* __restrict__ params,
                               const float* __restrict__ norm, float* __restrict__ Z1,
                               float* __restrict__ Z2, float* __restrict__ out) {
  __shared__ float sp[kNParams];
  load_params(sp, params);
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const uint32_t row = idx ? idx[s] : s;
  float x[kIn];
#pragma unroll
  for (int f = 0; f < kIn; ++f) x[f] = (X[(size_t)row * kIn + f] - norm[f]) / norm[kIn + f];
  float h1[kHid];
#pragma unroll
  for (int o = 0; o < kHid; ++o) {
    float z = sp[kOffB1 + o];
#pragma unroll
    for (int f = 0; f < kIn; ++f) z = fmaf(x[f], sp[kOffW1 + f * kHid + o], z);
    if (Z1) Z1[(size_t)s * kHid + o] = z;
    h1[o] = fmaxf(z, 0.f);
  }
  float y = sp[kOffB3];
  for (int o = 0; o < kHid; ++o) {
    float z = sp[kOffB2 + o];
#pragma unroll
    for (int i = 0; i < kHid; ++i) z = fmaf(h1[i], sp[kOffW2 + i * kHid + o], z);
    if (Z2) Z2[(size_t)s * kHid + o] = z;
    y = fmaf(fmaxf(z, 0.f), sp[kOffW3 + o], y);
  }
  out[s] = y;
}

// backward per sample: dout = 2 (out - y) / n, dZ2, dZ1
__global__ void mlp_bwd_kernel(const float* __restrict__ Y, const uint32_t* __restrict__ idx,
                               uint32_t n, float inv_n, const float* __restrict__ params,
                               const float* __restrict__ Z1, const float* __restrict__ Z2,
                               const float* __restrict__ out, float* __restrict__ dout,
                               float* __restrict__ dZ1, float* __restrict__ dZ2) {
  __shared__ float sp[kNParams];
  load_params(sp, params);
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const uint32_t row = idx ? idx[s] : s;
  const float d = 2.f * (out[s] - Y[row]) * inv_n;
  dout[s] = d;
  float g2[kHid];
#pragma unroll
  for (int o = 0; o < kHid; ++o) {
    g2[o] = Z2[(size_t)s * kHid + o] > 0.f ? d * sp[kOffW3 + o] : 0.f;
    dZ2[(size_t)s * kHid + o] = g2[o];
  }
  for (int i = 0; i < kHid; ++i) {
    float g = 0.f;
#pragma unroll
    for (int o = 0; o < kHid; ++o) g = fmaf(sp[kOffW2 + i * kHid + o], g2[o], g);
    dZ1[(size_t)s * kHid + i] = Z1[(size_t)s * kHid + i] > 0.f ? g : 0.f;
  }
}

// one thread per parameter: sums over the samples in order
__global__ void mlp_wgrad_kernel(const float* __restrict__ X, const uint32_t* __restrict__ idx,
                                 uint32_t n, const float* __restrict__ norm,
                                 const float* __restrict__ Z1, const float* __restrict__ Z2,
                                 const float* __restrict__ dout, const float* __restrict__ dZ1,
                                 const float* __restrict__ dZ2, float* __restrict__ grad) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= kNParams) return;
  float g = 0.f;
  if (p < kOffB1) {  // W1[f][o]
    const int f = p / kHid, o = p % kHid;
    for (uint32_t s = 0; s < n; ++s) {
      const uint32_t row = idx ? idx[s] : s;
      const float x = (X[(size_t)row * kIn + f] - norm[f]) / norm[kIn + f];
      g = fmaf(x, dZ1[(size_t)s * kHid + o], g);
    }
  } else if (p < kOffW2) {  // b1
    const int o = p - kOffB1;
    for (uint32_t s = 0; s < n; ++s) g += dZ1[(size_t)s * kHid + o];
  } else if (p < kOffB2) {  // W2[i][o]
    const int i = (p - kOffW2) / kHid, o = (p - kOffW2) % kHid;
    for (uint32_t s = 0; s < n; ++s)
      g = fmaf(fmaxf(Z1[(size_t)s * kHid + i], 0.f), dZ2[(size_t)s * kHid + o], g);
  } else if (p < kOffW3) {  // b2
    const int o = p - kOffB2;
    for (uint32_t s = 0; s < n; ++s) g += dZ2[(size_t)s * kHid + o];
  } else if (p < kOffB3) {  // w3
    const int o = p - kOffW3;
    for (uint32_t s = 0; s < n; ++s) g = fmaf(fmaxf(Z2[(size_t)s * kHid + o], 0.f), dout[s], g);
  } else {  // b3
    for (uint32_t s = 0; s < n; ++s) g += dout[s];
  }
  grad[p] = g;
}

__global__ void mlp_adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                                float* __restrict__ v, float lr, float b1t, float b2t) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kNParams) return;
  const float b1 = 0.9f, b2 = 0.999f;
  m[i] = b1 * m[i] + (1.f - b1) * g[i];
  v[i] = b2 * v[i] + (1.f - b2) * g[i] * g[i];
  const float mh = m[i] / (1.f - b1t), vh = v[i] / (1.f - b2t);
  p[i] -= lr * mh / (sqrtf(vh) + 1e-8f);
}

__global__ void mlp_sqerr_kernel(const float* __restrict__ out, const float* __restrict__ Y,
                                 const uint32_t* __restrict__ idx, uint32_t n, float* __restrict__ acc) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  float e = 0.f;
  if (s < n) {
    const float d = out[s] - Y[idx ? idx[s] : s];
    e = d * d;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(0xffffffffu, e, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(acc, e);
}

}  // namespace
}  // namespace ahx

struct ahx_mlp {
  int device = 0;
  cudaStream_t stream = nullptr;
  ahx::DevBuf params, grad, m, v, norm;
  ahx::DevBuf z1, z2, dz1, dz2, out, dout, idx, X, Y, acc;
  uint64_t cap = 0;  // samples the work buffers hold
  uint64_t step = 0;
};

using namespace ahx;

namespace {

int mlp_reserve(ahx_mlp* M, uint64_t n) {
  if (n <= M->cap) return AHX_OK;
  int rc;
  for (DevBuf* b : {&M->z1, &M->z2, &M->dz1, &M->dz2})
    if ((rc = b->reserve(n * kHid * sizeof(float)))) return rc;
  for (DevBuf* b : {&M->out, &M->dout})
    if ((rc = b->reserve(n * sizeof(float)))) return rc;
  if ((rc = M->idx.reserve(n * sizeof(uint32_t)))) return rc;
  M->cap = n;
  return AHX_OK;
}

// forward + backward + weight gradients for the samples idx[0..n) of (X, Y)
int mlp_grad(ahx_mlp* M, const float* X, const float* Y, const uint32_t* idx, uint32_t n) {
  int rc = mlp_reserve(M, n);
  if (rc) return rc;
  const unsigned g = (n + 127) / 128;
  cudaStream_t s = M->stream;
  mlp_fwd_kernel<<<g, 128, 0, s>>>(X, idx, n, M->params.as<float>(), M->norm.as<float>(),
                                   M->z1.as<float>(), M->z2.as<float>(), M->out.as<float>());
  mlp_bwd_kernel<<<g, 128, 0, s>>>(Y, idx, n, 1.f / (float)n, M->params.as<float>(), M->z1.as<float>(),
                                   M->z2.as<float>(), M->out.as<float>(), M->dout.as<float>(),
                                   M->dz1.as<float>(), M->dz2.as<float>());
  mlp_wgrad_kernel<<<(kNParams + 127) / 128, 128, 0, s>>>(
      X, idx, n, M->norm.as<float>(), M->z1.as<float>(), M->z2.as<float>(), M->dout.as<float>(),
      M->dz1.as<float>(), M->dz2.as<float>(), M->grad.as<float>());
  AHX_CUDA(cudaGetLastError());
  return AHX_OK;
}

}  // namespace

extern "C" {

uint32_t ahx_mlp_nparams(void) { return (uint32_t)kNParams; }

int ahx_mlp_create(int device, uint64_t seed, ahx_mlp** out) {
  if (!out) return AHX_ERR_ARG;
  *out = nullptr;
  AHX_CUDA(cudaSetDevice(device));
  ahx_mlp* M = new (std::nothrow) ahx_mlp;
  if (!M) return AHX_ERR_NOMEM;
  M->device = device;
  cudaError_t e = cudaStreamCreateWithFlags(&M->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete M;
    return cuda_fail(e, "cudaStreamCreate");
  }
  // He initialisation from a fixed-seed host generator (reproducible)
  std::vector<float> p(kNParams, 0.f);
  std::mt19937_64 rng(seed);
  std::normal_distribution<double> nd(0.0, 1.0);
  for (int i = 0; i < kIn * kHid; ++i) p[kOffW1 + i] = (float)(nd(rng) * std::sqrt(2.0 / kIn));
  for (int i = 0; i < kHid * kHid; ++i) p[kOffW2 + i] = (float)(nd(rng) * std::sqrt(2.0 / kHid));
  for (int i = 0; i < kHid; ++i) p[kOffW3 + i] = (float)(nd(rng) * std::sqrt(1.0 / kHid));
  std::vector<float> nm(2 * kIn, 0.f);
  for (int f = 0; f < kIn; ++f) nm[kIn + f] = 1.f;
  int rc;
  if ((rc = M->params.reserve(kNParams * 4)) || (rc = M->grad.reserve(kNParams * 4)) ||
      (rc = M->m.reserve(kNParams * 4)) || (rc = M->v.reserve(kNParams * 4)) ||
      (rc = M->norm.reserve(2 * kIn * 4)) || (rc = M->acc.reserve(4))) {
    ahx_mlp_destroy(M);
    return rc;
  }
  cudaMemcpy(M->params.p, p.data(), kNParams * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(M->norm.p, nm.data(), 2 * kIn * 4, cudaMemcpyHostToDevice);
  cudaMemset(M->m.p, 0, kNParams * 4);
  cudaMemset(M->v.p, 0, kNParams * 4);
  *out = M;
  return AHX_OK;
}

int ahx_mlp_destroy(ahx_mlp* M) {
  if (!M) return AHX_OK;
  cudaSetDevice(M->device);
  if (M->stream) cudaStreamSynchronize(M->stream);
  for (DevBuf* b : {&M->params, &M->grad, &M->m, &M->v, &M->norm, &M->z1, &M->z2, &M->dz1, &M->dz2,
                    &M->out, &M->dout, &M->idx, &M->X, &M->Y, &M->acc})
    b->release();
  if (M->stream) cudaStreamDestroy(M->stream);
  delete M;
  return AHX_OK;
}

int ahx_mlp_get_params(const ahx_mlp* M, float* out) {
  if (!M || !out) return AHX_ERR_ARG;
  AHX_CUDA(cudaSetDevice(M->device));
  AHX_CUDA(cudaMemcpy(out, M->params.p, kNParams * 4, cudaMemcpyDeviceToHost));
  return AHX_OK;
}

int ahx_mlp_set_params(ahx_mlp* M, const float* in) {
  if (!M || !in) return AHX_ERR_ARG;
  AHX_CUDA(cudaSetDevice(M->device));
  AHX_CUDA(cudaMemcpy(M->params.p, in, kNParams * 4, cudaMemcpyHostToDevice));
  return AHX_OK;
}

// feature normalisation: mean[8], std[8]
int ahx_mlp_set_norm(ahx_mlp* M, const float* mean, const float* stdev) {
  if (!M || !mean || !stdev) return AHX_ERR_ARG;
  float nm[2 * kIn];
  for (int f = 0; f < kIn; ++f) {
    nm[f] = mean[f];
    nm[kIn + f] = stdev[f] > 0.f ? stdev[f] : 1.f;
  }
  AHX_CUDA(cudaSetDevice(M->device));
  AHX_CUDA(cudaMemcpy(M->norm.p, nm, sizeof(nm), cudaMemcpyHostToDevice));
  return AHX_OK;
}

// Gradient of the mean squared error over all n samples (host arrays), for checking.
int ahx_mlp_gradients(ahx_mlp* M, const float* X, const float* Y, uint32_t n, float* grad,
                      float* loss) {
  if (!M || !X || !Y || !grad || n == 0) return AHX_ERR_ARG;
  AHX_CUDA(cudaSetDevice(M->device));
  int rc;
  if ((rc = M->X.reserve((size_t)n * kIn * 4)) || (rc = M->Y.reserve((size_t)n * 4))) return rc;
  AHX_CUDA(cudaMemcpyAsync(M->X.p, X, (size_t)n * kIn * 4, cudaMemcpyHostToDevice, M->stream));
  AHX_CUDA(cudaMemcpyAsync(M->Y.p, Y, (size_t)n * 4, cudaMemcpyHostToDevice, M->stream));
  if ((rc = mlp_grad(M, M->X.as<float>(), M->Y.as<float>(), nullptr, n))) return rc;
  AHX_CUDA(cudaMemsetAsync(M->acc.p, 0, 4, M->stream));
  mlp_sqerr_kernel<<<(n + 127) / 128, 128, 0, M->stream>>>(M->out.as<float>(), M->Y.as<float>(), nullptr, n,
                                                            M->acc.as<float>());
  float se = 0.f;
  AHX_CUDA(cudaMemcpyAsync(grad, M->grad.p, kNParams * 4, cudaMemcpyDeviceToHost, M->stream));
  AHX_CUDA(cudaMemcpyAsync(&se, M->acc.p, 4, cudaMemcpyDeviceToHost, M->stream));
  AHX_CUDA(cudaStreamSynchronize(M->stream));
  if (loss) *loss = se / (float)n;
  return AHX_OK;
}

// Adam on mini-batches of (X, Y) (host arrays, n samples), `epochs` passes in a
// fixed-seed shuffled order; loss[e] = training MSE after epoch e (may be NULL).
int ahx_mlp_train(ahx_mlp* M, const float* X, const float* Y, uint32_t n, uint32_t epochs,
                  uint32_t batch, float lr, uint64_t seed, float* loss) {
  if (!M || !X || !Y || n == 0 || batch == 0) return AHX_ERR_ARG;
  AHX_CUDA(cudaSetDevice(M->device));
  int rc;
  if ((rc = M->X.reserve((size_t)n * kIn * 4)) || (rc = M->Y.reserve((size_t)n * 4))) return rc;
  if ((rc = mlp_reserve(M, std::max(batch, n)))) return rc;
  AHX_CUDA(cudaMemcpyAsync(M->X.p, X, (size_t)n * kIn * 4, cudaMemcpyHostToDevice, M->stream));
  AHX_CUDA(cudaMemcpyAsync(M->Y.p, Y, (size_t)n * 4, cudaMemcpyHostToDevice, M->stream));
  std::vector<uint32_t> order(n);
  std::iota(order.begin(), order.end(), 0u);
  std::mt19937_64 rng(seed);
  DevBuf dorder;
  if ((rc = dorder.reserve((size_t)n * 4))) return rc;
  for (uint32_t e = 0; e < epochs; ++e) {
    std::shuffle(order.begin(), order.end(), rng);
    AHX_CUDA(cudaMemcpyAsync(dorder.p, order.data(), (size_t)n * 4, cudaMemcpyHostToDevice, M->stream));
    AHX_CUDA(cudaStreamSynchronize(M->stream));
    for (uint32_t b0 = 0; b0 < n; b0 += batch) {
      const uint32_t nb = std::min(batch, n - b0);
      if ((rc = mlp_grad(M, M->X.as<float>(), M->Y.as<float>(), dorder.as<uint32_t>() + b0, nb))) return rc;
      ++M->step;
      const float b1t = (float)std::pow(0.9, (double)M->step), b2t = (float)std::pow(0.999, (double)M->step);
      mlp_adam_kernel<<<(kNParams + 127) / 128, 128, 0, M->stream>>>(
          M->params.as<float>(), M->grad.as<float>(), M->m.as<float>(), M->v.as<float>(), lr, b1t, b2t);
    }
    if (loss) {
      mlp_fwd_kernel<<<(n + 127) / 128, 128, 0, M->stream>>>(M->X.as<float>(), nullptr, n, M->params.as<float>(),
                                                             M->norm.as<float>(), nullptr, nullptr,
                                                             M->out.as<float>());
      AHX_CUDA(cudaMemsetAsync(M->acc.p, 0, 4, M->stream));
      mlp_sqerr_kernel<<<(n + 127) / 128, 128, 0, M->stream>>>(M->out.as<float>(), M->Y.as<float>(), nullptr, n,
                                                                M->acc.as<float>());
      float se = 0.f;
      AHX_CUDA(cudaMemcpyAsync(&se, M->acc.p, 4, cudaMemcpyDeviceToHost, M->stream));
      AHX_CUDA(cudaStreamSynchronize(M->stream));
      loss[e] = se / (float)n;
    }
  }
  AHX_CUDA(cudaGetLastError());
  AHX_CUDA(cudaStreamSynchronize(M->stream));
  dorder.release();
  return AHX_OK;
}

int ahx_mlp_predict(ahx_mlp* M, const float* X, uint32_t n, float* out) {
  if (!M || !X || !out) return AHX_ERR_ARG;
  if (n == 0) return AHX_OK;
  AHX_CUDA(cudaSetDevice(M->device));
  int rc;
  if ((rc = M->X.reserve((size_t)n * kIn * 4)) || (rc = mlp_reserve(M, n))) return rc;
  AHX_CUDA(cudaMemcpyAsync(M->X.p, X, (size_t)n * kIn * 4, cudaMemcpyHostToDevice, M->stream));
  mlp_fwd_kernel<<<(n + 127) / 128, 128, 0, M->stream>>>(M->X.as<float>(), nullptr, n, M->params.as<float>(),
                                                         M->norm.as<float>(), nullptr, nullptr, M->out.as<float>());
  AHX_CUDA(cudaGetLastError());
  AHX_CUDA(cudaMemcpyAsync(out, M->out.p, (size_t)n * 4, cudaMemcpyDeviceToHost, M->stream));
  AHX_CUDA(cudaStreamSynchronize(M->stream));
  return AHX_OK;
}

}  // extern "C"
