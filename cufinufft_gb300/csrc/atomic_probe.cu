// atomic_probe.cu -- measured ceilings of the accumulation the spread kernels
// are bound by: shared-memory FP32 atomicAdd, shared-memory int32 and 64-bit
// integer atomicAdd (the candidates for fixed-point tiles) and the 8-byte
// global reduction red.global.add.v2.f32 into L2-resident addresses.  Every
// lane of a warp adds into its own address (no conflicts), as the spread
// kernels' lanes mostly do, so the rates are the throughput ceilings the
// type-1 roofline is taken against.
#include <cuda_runtime.h>

#include "cufinufft.h"
#include "device_common.cuh"

namespace {

constexpr int kThreads = 512;
constexpr int kSlots = 8;                  // addresses per thread (shared: 16 KB per block)
constexpr int kIters = 1024;               // loop trips per thread; kSlots adds each
constexpr int kGlobalElems = 1 << 22;      // float2 elements: 32 MB, resident in L2

__global__ void __launch_bounds__(kThreads) k_probe_shared_f32(float* out) {
  __shared__ float s[kThreads * kSlots];
  for (int j = 0; j < kSlots; ++j) s[threadIdx.x + kThreads * j] = 0.f;
  __syncthreads();
  for (int it = 0; it < kIters; ++it) {
#pragma unroll
    for (int j = 0; j < kSlots; ++j) atomicAdd(&s[threadIdx.x + kThreads * j], 1.0f);
  }
  __syncthreads();
  float acc = 0.f;
  for (int j = 0; j < kSlots; ++j) acc += s[threadIdx.x + kThreads * j];
  out[blockIdx.x * kThreads + threadIdx.x] = acc;
}

__global__ void __launch_bounds__(kThreads) k_probe_shared_i32(float* out) {
  __shared__ int s[kThreads * kSlots];
  for (int j = 0; j < kSlots; ++j) s[threadIdx.x + kThreads * j] = 0;
  __syncthreads();
  for (int it = 0; it < kIters; ++it) {
#pragma unroll
    for (int j = 0; j < kSlots; ++j) atomicAdd(&s[threadIdx.x + kThreads * j], 3);
  }
  __syncthreads();
  int acc = 0;
  for (int j = 0; j < kSlots; ++j) acc += s[threadIdx.x + kThreads * j];
  out[blockIdx.x * kThreads + threadIdx.x] = (float)acc;
}

__global__ void __launch_bounds__(kThreads) k_probe_shared_u64(float* out) {
  __shared__ unsigned long long s[kThreads * kSlots];
  for (int j = 0; j < kSlots; ++j) s[threadIdx.x + kThreads * j] = 0ull;
  __syncthreads();
  for (int it = 0; it < kIters; ++it) {
#pragma unroll
    for (int j = 0; j < kSlots; ++j) atomicAdd(&s[threadIdx.x + kThreads * j], 3ull);
  }
  __syncthreads();
  unsigned long long acc = 0;
  for (int j = 0; j < kSlots; ++j) acc += s[threadIdx.x + kThreads * j];
  out[blockIdx.x * kThreads + threadIdx.x] = (float)acc;
}

// Consecutive lanes add into consecutive float2 elements (a warp covers 256
// contiguous bytes), the access pattern of the warp-cooperative spread.
__global__ void __launch_bounds__(kThreads) k_probe_global_red(float2* g) {
  const unsigned t = blockIdx.x * kThreads + threadIdx.x;
  for (int it = 0; it < kIters / 8; ++it) {
#pragma unroll
    for (int j = 0; j < kSlots; ++j) {
      const unsigned e = (t + (unsigned)(it * kSlots + j) * 65536u) & (kGlobalElems - 1);
      cfg::red_add(g + e, 1.0f, 1.0f);
    }
  }
}

}  // namespace

extern "C" int cufinufft_atomic_rate(int kind, double* lane_ops_per_s) {
  if (!lane_ops_per_s || kind < 0 || kind > 3) return CUFINUFFT_ERR_ARG;
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return CUFINUFFT_ERR_CUDA;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return CUFINUFFT_ERR_CUDA;
  // four 512-thread blocks are resident per SM; eight waves of them
  const int blocks = nsm * 4 * 8;
  float* out = nullptr;
  float2* g = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaStream_t st = nullptr;
  int rc = CUFINUFFT_ERR_CUDA;
  double ops = 0;
  float ms = 0.f;
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return CUFINUFFT_ERR_CUDA;
  if (cudaMalloc(&out, sizeof(float) * (size_t)blocks * kThreads) != cudaSuccess) goto done;
  if (kind == 2 && cudaMalloc(&g, sizeof(float2) * (size_t)kGlobalElems) != cudaSuccess) goto done;
  if (g && cudaMemsetAsync(g, 0, sizeof(float2) * (size_t)kGlobalElems, st) != cudaSuccess) goto done;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) goto done;
  for (int rep = 0; rep < 2; ++rep) {  // the first launch warms up
    cudaEventRecord(e0, st);
    if (kind == 0) k_probe_shared_f32<<<blocks, kThreads, 0, st>>>(out);
    else if (kind == 1) k_probe_shared_i32<<<blocks, kThreads, 0, st>>>(out);
    else if (kind == 2) k_probe_global_red<<<blocks, kThreads, 0, st>>>(g);
    else k_probe_shared_u64<<<blocks, kThreads, 0, st>>>(out);
    cudaEventRecord(e1, st);
  }
  if (cudaGetLastError() != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess) goto done;
  if (cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess || ms <= 0.f) goto done;
  ops = (double)blocks * kThreads * (kind == 2 ? (kIters / 8) : kIters) * kSlots;
  *lane_ops_per_s = ops / (ms * 1e-3);
  rc = 0;
done:
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (out) cudaFree(out);
  if (g) cudaFree(g);
  cudaStreamDestroy(st);
  return rc;
}
