// fft_df.cu -- FFT of FP64 grids in double-float arithmetic (FP32 pairs).
//
// GB300's FP64 units are a small fraction of its FP32 rate, and cuFFT's Z2Z
// transform of an FP64 plan's fine grid is bound by them.  Here a 2D
// transform is two passes of 1D transforms along rows -- the second after a
// tiled transpose -- each row transformed in shared memory by the radix-2
// Stockham formulation (natural-order output, no bit reversal):
//   for Ns = 1, 2, 4, ..., n/2:  for j < n/2:
//     v0 = x[j], v1 = x[j + n/2] * W^((j mod Ns) n / (2 Ns)),
//     y[(j - j mod Ns) 2 + j mod Ns] = v0 + v1,  y[... + Ns] = v0 - v1
// with W = exp(sign 2 pi i / n).  Values are split on load into float
// pairs hi + lo (~2^-48 relative), twiddles come from a table computed in
// extended precision on the host, and every product and sum is a
// double-float operation (device_common.cuh); results are merged back to
// double on store.
#include <cuda_runtime.h>

#include "device_common.cuh"
#include "kernels.h"

namespace cfg {
namespace {

// 512 threads: three blocks of 64 KB (n = 2048) per SM keep 48 warps
// resident, which the double-float butterflies' latency chains need
// (radial 2D FP64, 2048^2: 384 -> 350 us with the first stage below; a
// radix-4 form of the stages measured slower, 376 us)
constexpr int kFftDfThreads = 512;

__device__ __forceinline__ float4 split_c(double2 v) {
  const DF r = df_from(v.x), i = df_from(v.y);
  return make_float4(r.h, r.l, i.h, i.l);
}
__device__ __forceinline__ double2 merge_c(float4 v) {
  return make_double2((double)v.x + (double)v.y, (double)v.z + (double)v.w);
}
__device__ __forceinline__ DF dneg(DF a) { return DF{-a.h, -a.l}; }

// One transform of length n (a power of two <= 4096) per block; rows are
// consecutive blocks of n elements.  Shared memory: two buffers of n cells.
__global__ void __launch_bounds__(kFftDfThreads)
k_fft_df_rows(const double2* __restrict__ in, double2* __restrict__ out, int n, long long rows,
              const float4* __restrict__ tw) {
  extern __shared__ float4 sm[];
  const long long row = blockIdx.x + (long long)blockIdx.y * gridDim.x;
  if (row >= rows) return;  // block-uniform
  float4* x = sm;
  float4* y = sm + n;
  const double2* src = in + row * (long long)n;
  for (int i = threadIdx.x; i < n; i += blockDim.x) x[i] = split_c(src[i]);
  __syncthreads();
  const int half = n >> 1;
  // first stage: every twiddle is 1
  for (int j = threadIdx.x; j < half; j += blockDim.x) {
    const float4 a = x[j], b = x[j + half];
    const DF ar{a.x, a.y}, ai{a.z, a.w}, br{b.x, b.y}, bi{b.z, b.w};
    const DF s0r = df_add(ar, br), s0i = df_add(ai, bi);
    const DF s1r = df_add(ar, dneg(br)), s1i = df_add(ai, dneg(bi));
    y[2 * j] = make_float4(s0r.h, s0r.l, s0i.h, s0i.l);
    y[2 * j + 1] = make_float4(s1r.h, s1r.l, s1i.h, s1i.l);
  }
  __syncthreads();
  {
    float4* t = x;
    x = y;
    y = t;
  }
  for (int Ns = 2; Ns < n; Ns <<= 1) {
    const int tstep = half / Ns;  // twiddle index = (j mod Ns) * n / (2 Ns)
    for (int j = threadIdx.x; j < half; j += blockDim.x) {
      const float4 a = x[j], b = x[j + half];
      const int jm = j & (Ns - 1);
      const float4 w = __ldg(tw + jm * tstep);
      const DF br{b.x, b.y}, bi{b.z, b.w}, wr{w.x, w.y}, wi{w.z, w.w};
      const DF tr = df_add(df_mul(br, wr), dneg(df_mul(bi, wi)));
      const DF ti = df_add(df_mul(br, wi), df_mul(bi, wr));
      const DF ar{a.x, a.y}, ai{a.z, a.w};
      const DF s0r = df_add(ar, tr), s0i = df_add(ai, ti);
      const DF s1r = df_add(ar, dneg(tr)), s1i = df_add(ai, dneg(ti));
      const int o = ((j - jm) << 1) + jm;
      y[o] = make_float4(s0r.h, s0r.l, s0i.h, s0i.l);
      y[o + Ns] = make_float4(s1r.h, s1r.l, s1i.h, s1i.l);
    }
    __syncthreads();
    float4* t = x;
    x = y;
    y = t;
  }
  double2* dst = out + row * (long long)n;
  for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = merge_c(x[i]);
}

// out[b][c][r] = in[b][r][c] for R x C planes, 32 x 32 tiles.
__global__ void __launch_bounds__(256) k_transpose_d2(const double2* __restrict__ in, double2* __restrict__ out,
                                                      int R, int C) {
  __shared__ double2 t[32][33];
  const size_t plane = (size_t)blockIdx.z * R * C;
  const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int r = r0 + k, c = c0 + threadIdx.x;
    if (r < R && c < C) t[k][threadIdx.x] = in[plane + (size_t)r * C + c];
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int c = c0 + k, r = r0 + threadIdx.x;
    if (c < C && r < R) out[plane + (size_t)c * R + r] = t[threadIdx.x][k];
  }
}

}  // namespace

bool fft_df_size_ok(int n) { return n >= 2 && n <= 4096 && (n & (n - 1)) == 0; }

size_t fft_df_smem(int n) { return (size_t)2 * n * sizeof(float4); }

cudaError_t launch_fft_df_rows(const double2* in, double2* out, int n, long long rows, const float4* tw,
                               cudaStream_t s) {
  if (rows <= 0) return cudaSuccess;
  if (!fft_df_size_ok(n)) return cudaErrorInvalidValue;
  const size_t smb = fft_df_smem(n);
  if (smb > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k_fft_df_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smb);
    if (e != cudaSuccess) return e;
  }
  const long long gx = rows < 65535 ? rows : 65535;
  const long long gy = (rows + gx - 1) / gx;
  if (gy > 65535) return cudaErrorInvalidValue;
  k_fft_df_rows<<<dim3((unsigned)gx, (unsigned)gy), kFftDfThreads, smb, s>>>(in, out, n, rows, tw);
  return cudaGetLastError();
}

cudaError_t launch_transpose_d2(const double2* in, double2* out, int R, int C, int batch, cudaStream_t s) {
  if (R <= 0 || C <= 0 || batch <= 0) return cudaSuccess;
  if (batch > 65535) return cudaErrorInvalidValue;
  dim3 grid((C + 31) / 32, (R + 31) / 32, batch);
  k_transpose_d2<<<grid, dim3(32, 8), 0, s>>>(in, out, R, C);
  return cudaGetLastError();
}

}  // namespace cfg
