// deconv.cu -- kernel Fourier series, deconvolution (type 1) and
// amplification (type 2).
//
// fseries: the reference evaluates fhat(k) = sum_n 2 f_n |a_n|^k cos(k arg a_n)
// with a_n = exp(2 pi i (nf/2 - z_n)/nf) (src/common.cu:16-45).  Because nf is
// even this equals (-1)^k sum_n 2 f_n cos(2 pi k z_n / nf); the small argument
// keeps the phase exact to ~1e-15 rad for every k.  The per-mode reciprocal
// 1/fhat_d(|k_d|) is stored once per axis in the plan precision, so the
// deconvolution is one multiply per mode per axis.
//
// deconvolve / amplify restate Deconvolve_{1,2,3}d / Amplify_{1,2,3}d
// (src/deconvolve_wrapper.cu:14-121): mode k_d in -N_d/2..(N_d-1)/2 lives at
// fine-grid index k_d mod nf_d.  Both kernels handle the whole batch in one
// launch.  Amplify writes only the mode cells: the plan zeroes the padding
// of its grid once and runs the type-2 FFT out of place, so the padding
// stays zero (the reference clears the whole grid on every execute).
#include <algorithm>

#include "device_common.cuh"
#include "kernels.h"

namespace cfg {

struct FseriesLaunch {
  FseriesNodes nodes;
  int nf[3], N[3];
  int dim;
};

template <typename T>
__global__ void k_fseries(FseriesLaunch L, T* fac0, T* fac1, T* fac2) {
  const int ax = blockIdx.y;
  if (ax >= L.dim) return;
  T* fac = ax == 0 ? fac0 : (ax == 1 ? fac1 : fac2);
  const int N = L.N[ax];
  const double nf = (double)L.nf[ax];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    const int k = abs(i - N / 2);
    double s = 0.0;
    for (int n = 0; n < L.nodes.q; ++n)
      s += 2.0 * L.nodes.f[n] * cospi(2.0 * ((double)k * L.nodes.z[n] / nf));
    if (k & 1) s = -s;
    fac[i] = (T)(1.0 / s);
  }
}

template <typename T>
cudaError_t launch_fseries(const FseriesNodes& nodes, int dim, const int nf[3], const int N[3],
                           T* fac0, T* fac1, T* fac2, cudaStream_t s) {
  FseriesLaunch L;
  L.nodes = nodes;
  L.dim = dim;
  int nmax = 1;
  for (int d = 0; d < 3; ++d) {
    L.nf[d] = nf[d];
    L.N[d] = N[d];
    if (d < dim && N[d] > nmax) nmax = N[d];
  }
  dim3 grid((nmax + 255) / 256, 3);
  k_fseries<T><<<grid, 256, 0, s>>>(L, fac0, fac1, fac2);
  return cudaGetLastError();
}

// One block row per (k2, k3) mode row; threads over k1.
// Cells per thread per pass of the row kernels below.
constexpr int kRowUnroll = 4;

template <typename T>
__global__ void __launch_bounds__(256)
k_deconvolve(int dim, int nf0, int nf1, int nf2, int N0, int N1, int N2, const cplx_t<T>* __restrict__ fw,
             cplx_t<T>* __restrict__ fk, const T* __restrict__ fac0, const T* __restrict__ fac1,
             const T* __restrict__ fac2, int ntr) {
  using C = cplx_t<T>;
  const long long Nf = (long long)nf0 * nf1 * nf2;
  const long long Nm = (long long)N0 * N1 * N2;
  const int nrows = N1 * N2;
  for (int r = blockIdx.x; r < nrows * ntr; r += gridDim.x) {
    const int t = r / nrows;
    const int rr = r - t * nrows;
    const int i2 = rr % N1, i3 = rr / N1;
    const int k2 = i2 - N1 / 2, k3 = i3 - N2 / 2;
    const int w2 = k2 >= 0 ? k2 : nf1 + k2;
    const int w3 = k3 >= 0 ? k3 : nf2 + k3;
    T f23 = T(1);
    if (dim > 1) f23 = fac1[i2];
    if (dim > 2) f23 *= fac2[i3];
    const C* src = fw + (size_t)t * Nf + ((size_t)w3 * nf1 + w2) * nf0;
    C* dst = fk + (size_t)t * Nm + ((size_t)i3 * N1 + i2) * N0;
    // kRowUnroll cells per thread with every load issued before the first
    // store: a row's reads are in flight together
    for (int b = threadIdx.x; b < N0; b += kRowUnroll * blockDim.x) {
      C v[kRowUnroll];
      T f[kRowUnroll];
#pragma unroll
      for (int u = 0; u < kRowUnroll; ++u) {
        const int i1 = b + u * blockDim.x;
        if (i1 < N0) {
          const int k1 = i1 - N0 / 2;
          v[u] = src[k1 >= 0 ? k1 : nf0 + k1];
          f[u] = fac0[i1];
        }
      }
#pragma unroll
      for (int u = 0; u < kRowUnroll; ++u) {
        const int i1 = b + u * blockDim.x;
        if (i1 < N0) {
          const T g = f[u] * f23;
          C o;
          o.x = v[u].x * g;
          o.y = v[u].y * g;
          dst[i1] = o;
        }
      }
    }
  }
}

static int row_grid(long long rows) {
  long long cap = 152LL * 16;
  return (int)(rows < cap ? (rows < 1 ? 1 : rows) : cap);
}

template <typename T>
cudaError_t launch_deconvolve(int dim, const int nf[3], const int N[3], const cplx_t<T>* fw,
                              cplx_t<T>* fk, const T* fac0, const T* fac1, const T* fac2, int ntr,
                              cudaStream_t s) {
  long long rows = (long long)N[1] * N[2] * ntr;
  k_deconvolve<T><<<row_grid(rows), 256, 0, s>>>(dim, nf[0], nf[1], nf[2], N[0], N[1], N[2], fw, fk,
                                                 fac0, fac1, fac2, ntr);
  return cudaGetLastError();
}

// Type-2 amplification into a grid whose padding is already zero (the FFT
// then runs out of place): only the mode cells are written, one block row per
// (k2, k3) mode row, threads over k1 -- the mirror of k_deconvolve.
template <typename T>
__global__ void __launch_bounds__(256)
k_amplify_modes(int dim, int nf0, int nf1, int nf2, int N0, int N1, int N2, cplx_t<T>* __restrict__ fw,
                const cplx_t<T>* __restrict__ fk, const T* __restrict__ fac0, const T* __restrict__ fac1,
                const T* __restrict__ fac2, int ntr) {
  using C = cplx_t<T>;
  const long long Nf = (long long)nf0 * nf1 * nf2;
  const long long Nm = (long long)N0 * N1 * N2;
  const int nrows = N1 * N2;
  for (int r = blockIdx.x; r < nrows * ntr; r += gridDim.x) {
    const int t = r / nrows;
    const int rr = r - t * nrows;
    const int i2 = rr % N1, i3 = rr / N1;
    const int k2 = i2 - N1 / 2, k3 = i3 - N2 / 2;
    const int w2 = k2 >= 0 ? k2 : nf1 + k2;
    const int w3 = k3 >= 0 ? k3 : nf2 + k3;
    T f23 = T(1);
    if (dim > 1) f23 = fac1[i2];
    if (dim > 2) f23 *= fac2[i3];
    C* dst = fw + (size_t)t * Nf + ((size_t)w3 * nf1 + w2) * nf0;
    const C* src = fk + (size_t)t * Nm + ((size_t)i3 * N1 + i2) * N0;
    for (int b = threadIdx.x; b < N0; b += kRowUnroll * blockDim.x) {
      C v[kRowUnroll];
      T f[kRowUnroll];
#pragma unroll
      for (int u = 0; u < kRowUnroll; ++u) {
        const int i1 = b + u * blockDim.x;
        if (i1 < N0) {
          v[u] = src[i1];
          f[u] = fac0[i1];
        }
      }
#pragma unroll
      for (int u = 0; u < kRowUnroll; ++u) {
        const int i1 = b + u * blockDim.x;
        if (i1 < N0) {
          const int k1 = i1 - N0 / 2;
          const T g = f[u] * f23;
          C o;
          o.x = v[u].x * g;
          o.y = v[u].y * g;
          dst[k1 >= 0 ? k1 : nf0 + k1] = o;
        }
      }
    }
  }
}

template <typename T>
cudaError_t launch_amplify_modes(int dim, const int nf[3], const int N[3], cplx_t<T>* fw,
                                 const cplx_t<T>* fk, const T* fac0, const T* fac1, const T* fac2,
                                 int ntr, cudaStream_t s) {
  const long long rows = (long long)N[1] * N[2] * ntr;
  const int grid = (int)std::min<long long>(std::max<long long>(rows, 1), 152LL * 32);
  k_amplify_modes<T><<<grid, 256, 0, s>>>(dim, nf[0], nf[1], nf[2], N[0], N[1], N[2], fw, fk, fac0,
                                          fac1, fac2, ntr);
  return cudaGetLastError();
}
template cudaError_t launch_amplify_modes<float>(int, const int*, const int*, cplx_t<float>*,
                                                 const cplx_t<float>*, const float*, const float*,
                                                 const float*, int, cudaStream_t);
template cudaError_t launch_amplify_modes<double>(int, const int*, const int*, cplx_t<double>*,
                                                  const cplx_t<double>*, const double*,
                                                  const double*, const double*, int, cudaStream_t);

template cudaError_t launch_fseries<float>(const FseriesNodes&, int, const int*, const int*, float*,
                                           float*, float*, cudaStream_t);
template cudaError_t launch_fseries<double>(const FseriesNodes&, int, const int*, const int*, double*,
                                            double*, double*, cudaStream_t);
template cudaError_t launch_deconvolve<float>(int, const int*, const int*, const float2*, float2*,
                                              const float*, const float*, const float*, int,
                                              cudaStream_t);
template cudaError_t launch_deconvolve<double>(int, const int*, const int*, const double2*, double2*,
                                               const double*, const double*, const double*, int,
                                               cudaStream_t);

}  // namespace cfg
