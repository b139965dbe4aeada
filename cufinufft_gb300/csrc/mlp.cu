// mlp.cu -- the learned layout selector's network: a 3-layer perceptron with
// hand-written CUDA forward, backward and Adam kernels (FP32).
//
// Architecture (fixed): features F=14 -> H=32 (ReLU) -> H=32 (ReLU) -> K=12.
// Output k predicts log2(time of layout class k / time of the fastest class)
// for the workload the features describe; the selector picks the argmin over
// the classes the plan can run.  Parameters are one flat FP32 array:
//   W1[H][F], b1[H], W2[H][H], b2[H], W3[K][H], b3[K]
// (kMlpParams floats).  Training minimises the masked mean squared error
//   L = sum_{b,k} m[b,k] (y[b,k] - t[b,k])^2 / sum m
// with Adam; every kernel is a plain loop over small matrices (the whole
// network is 1.9k parameters), one thread per output element.
#include <cuda_runtime.h>

#include "../../include/cufinufft.h"

namespace cfg {
namespace {

constexpr int F = CUFINUFFT_MLP_FEATURES;
constexpr int H = CUFINUFFT_MLP_HIDDEN;
constexpr int K = CUFINUFFT_MLP_CLASSES;
constexpr int OFF_W1 = 0;
constexpr int OFF_B1 = OFF_W1 + H * F;
constexpr int OFF_W2 = OFF_B1 + H;
constexpr int OFF_B2 = OFF_W2 + H * H;
constexpr int OFF_W3 = OFF_B2 + H;
constexpr int OFF_B3 = OFF_W3 + K * H;
constexpr int NPARAM = OFF_B3 + K;
static_assert(NPARAM == CUFINUFFT_MLP_PARAMS, "parameter count");

// Y[b][o] = act(sum_i W[o][i] X[b][i] + bias[o]); relu != 0 applies ReLU.
__global__ void k_dense(const float* __restrict__ W, const float* __restrict__ bias,
                        const float* __restrict__ X, float* __restrict__ Y, int B, int in, int out,
                        int relu) {
  const int n = B * out;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
    const int b = e / out, o = e - (e / out) * out;
    float s = bias[o];
    for (int i = 0; i < in; ++i) s = fmaf(W[o * in + i], X[b * in + i], s);
    Y[e] = (relu && s < 0.f) ? 0.f : s;
  }
}

// dY = 2 m (Y - T) / msum; also accumulates the loss into loss[0].
__global__ void k_loss_grad(const float* __restrict__ Y, const float* __restrict__ T,
                            const float* __restrict__ Mk, float* __restrict__ dY, int n,
                            float inv_msum, float* __restrict__ loss) {
  float part = 0.f;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
    const float d = (Y[e] - T[e]) * Mk[e];
    dY[e] = 2.f * d * inv_msum;
    part += d * d * inv_msum;
  }
  for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, part);
}

// Gradients of one dense layer: dW[o][i] = sum_b dY[b][o] X[b][i],
// db[o] = sum_b dY[b][o].
__global__ void k_dense_wgrad(const float* __restrict__ dY, const float* __restrict__ X,
                              float* __restrict__ dW, float* __restrict__ db, int B, int in,
                              int out) {
  const int n = out * (in + 1);
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
    const int o = e / (in + 1), i = e - o * (in + 1);
    float s = 0.f;
    if (i < in) {
      for (int b = 0; b < B; ++b) s = fmaf(dY[b * out + o], X[b * in + i], s);
      dW[o * in + i] = s;
    } else {
      for (int b = 0; b < B; ++b) s += dY[b * out + o];
      db[o] = s;
    }
  }
}

// dX[b][i] = (sum_o dY[b][o] W[o][i]) * [A[b][i] > 0]  (A: the ReLU output).
__global__ void k_dense_xgrad(const float* __restrict__ dY, const float* __restrict__ W,
                              const float* __restrict__ A, float* __restrict__ dX, int B, int in,
                              int out) {
  const int n = B * in;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
    const int b = e / in, i = e - (e / in) * in;
    float s = 0.f;
    for (int o = 0; o < out; ++o) s = fmaf(dY[b * out + o], W[o * in + i], s);
    dX[e] = A[e] > 0.f ? s : 0.f;
  }
}

__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, int n, float lr, float b1, float b2, float eps,
                       float c1, float c2) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
    const float gi = g[e];
    m[e] = b1 * m[e] + (1.f - b1) * gi;
    v[e] = b2 * v[e] + (1.f - b2) * gi * gi;
    p[e] -= lr * (m[e] / c1) / (sqrtf(v[e] / c2) + eps);
  }
}

inline int blocks_for(int n) {
  int b = (n + 255) / 256;
  return b < 1 ? 1 : (b > 1024 ? 1024 : b);
}

// Forward pass; A1, A2 are the hidden activations [B][H].
cudaError_t forward(const float* P, const float* X, int B, float* A1, float* A2, float* Y,
                    cudaStream_t s) {
  k_dense<<<blocks_for(B * H), 256, 0, s>>>(P + OFF_W1, P + OFF_B1, X, A1, B, F, H, 1);
  k_dense<<<blocks_for(B * H), 256, 0, s>>>(P + OFF_W2, P + OFF_B2, A1, A2, B, H, H, 1);
  k_dense<<<blocks_for(B * K), 256, 0, s>>>(P + OFF_W3, P + OFF_B3, A2, Y, B, H, K, 0);
  return cudaGetLastError();
}

// Loss and full gradient into G (NPARAM floats).  work holds
// B*(2H + K) + B*(2H) + B*K floats.
cudaError_t loss_and_grad(const float* P, const float* X, const float* T, const float* Mk, int B,
                          float msum, float* G, float* loss, float* work, cudaStream_t s) {
  float* A1 = work;
  float* A2 = A1 + B * H;
  float* Y = A2 + B * H;
  float* dY = Y + B * K;
  float* dA2 = dY + B * K;
  float* dA1 = dA2 + B * H;
  cudaError_t e = forward(P, X, B, A1, A2, Y, s);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(loss, 0, sizeof(float), s);
  if (e != cudaSuccess) return e;
  k_loss_grad<<<blocks_for(B * K), 256, 0, s>>>(Y, T, Mk, dY, B * K, 1.f / msum, loss);
  k_dense_wgrad<<<blocks_for(K * (H + 1)), 256, 0, s>>>(dY, A2, G + OFF_W3, G + OFF_B3, B, H, K);
  k_dense_xgrad<<<blocks_for(B * H), 256, 0, s>>>(dY, P + OFF_W3, A2, dA2, B, H, K);
  k_dense_wgrad<<<blocks_for(H * (H + 1)), 256, 0, s>>>(dA2, A1, G + OFF_W2, G + OFF_B2, B, H, H);
  k_dense_xgrad<<<blocks_for(B * H), 256, 0, s>>>(dA2, P + OFF_W2, A1, dA1, B, H, H);
  k_dense_wgrad<<<blocks_for(H * (F + 1)), 256, 0, s>>>(dA1, X, G + OFF_W1, G + OFF_B1, B, F, H);
  return cudaGetLastError();
}

}  // namespace
}  // namespace cfg

extern "C" {

int cufinufft_mlp_forward(const float* params, const float* X, int B, float* Y, float* work,
                          cudaStream_t stream) {
  if (!params || !X || !Y || !work || B < 0) return CUFINUFFT_ERR_ARG;
  if (B == 0) return 0;
  float* A1 = work;
  float* A2 = A1 + (size_t)B * cfg::H;
  return cfg::forward(params, X, B, A1, A2, Y, stream) == cudaSuccess ? 0 : CUFINUFFT_ERR_CUDA;
}

int cufinufft_mlp_grad(const float* params, const float* X, const float* T, const float* mask,
                       int B, float mask_sum, float* grad, float* loss, float* work,
                       cudaStream_t stream) {
  if (!params || !X || !T || !mask || !grad || !loss || !work || B <= 0 || mask_sum <= 0.f)
    return CUFINUFFT_ERR_ARG;
  return cfg::loss_and_grad(params, X, T, mask, B, mask_sum, grad, loss, work, stream) == cudaSuccess
             ? 0
             : CUFINUFFT_ERR_CUDA;
}

int cufinufft_mlp_adam(float* params, const float* grad, float* m, float* v, int step, float lr,
                       cudaStream_t stream) {
  if (!params || !grad || !m || !v || step < 1) return CUFINUFFT_ERR_ARG;
  const float b1 = 0.9f, b2 = 0.999f;
  float c1 = 1.f, c2 = 1.f;
  for (int i = 0; i < step; ++i) {
    c1 *= b1;
    c2 *= b2;
  }
  cfg::k_adam<<<cfg::blocks_for(cfg::NPARAM), 256, 0, stream>>>(params, grad, m, v, cfg::NPARAM, lr,
                                                                 b1, b2, 1e-8f, 1.f - c1, 1.f - c2);
  return cudaGetLastError() == cudaSuccess ? 0 : CUFINUFFT_ERR_CUDA;
}

}  // extern "C"
