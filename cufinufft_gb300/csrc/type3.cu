// type3.cu -- device steps of the type-3 transform (nonuniform points x_j to
// nonuniform frequencies s_k), f_k = sum_j c_j exp(i sgn s_k . x_j).
//
// The reference reserves type 3 in its interface (src/cufinufft.cu:533-536,
// setpts' N, s, t, u arguments) without implementing it.  The method here is
// the standard one for the ES kernel: with x = C + gam x' and s = D + s'',
//   f_k = e^(i sgn s_k.C) sum_j [c_j e^(i sgn D.(x_j - C))] e^(i sgn (gam s''_k).x'_j),
// the inner sum is spread from x' in [-pi, pi) onto a grid of spacing
// h = 2 pi / nf, read back at tau_k = h gam s''_k by a type-2 transform of
// that grid (grid index m - nf/2 as mode m), and divided by the kernel's
// Fourier transform phihat(tau_k) = int phi(z) e^(i tau z) dz (Poisson
// summation).  This file holds the elementwise steps: extent of the points,
// rescaling, the phases and phihat.
#include <cfloat>

#include "device_common.cuh"
#include "kernels.h"

namespace cfg {
namespace {

constexpr int kT3Threads = 256;

int t3_grid(long long n) {
  long long b = (n + kT3Threads - 1) / kT3Threads;
  if (b > 152LL * 8) b = 152LL * 8;
  return b < 1 ? 1 : (int)b;
}

// Per-block minimum and maximum of a[0..n): out[2 b] = min, out[2 b + 1] = max.
template <typename T>
__global__ void __launch_bounds__(kT3Threads) k_minmax(const T* __restrict__ a, long long n, double* out) {
  double lo = DBL_MAX, hi = -DBL_MAX;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double v = (double)a[i];
    lo = fmin(lo, v);
    hi = fmax(hi, v);
  }
  __shared__ double slo[kT3Threads / 32], shi[kT3Threads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    slo[w] = lo;
    shi[w] = hi;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 1; k < kT3Threads / 32; ++k) {
      lo = fmin(lo, slo[k]);
      hi = fmax(hi, shi[k]);
    }
    out[2 * blockIdx.x] = lo;
    out[2 * blockIdx.x + 1] = hi;
  }
}

// out[i] = (a[i] - centre) * scale, computed in FP64.
template <typename T>
__global__ void k_affine(const T* __restrict__ a, long long n, double centre, double scale, T* __restrict__ out) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = (T)(((double)a[i] - centre) * scale);
}

// pre[j] = exp(i sgn sum_d D_d (x_d[j] - C_d)), FP64 phase.
template <typename T>
__global__ void k_prephase(Type3Phase<T> a, long long n, cplx_t<T>* __restrict__ pre) {
  for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (long long)gridDim.x * blockDim.x) {
    double ph = 0.0;
    for (int d = 0; d < a.dim; ++d) ph += a.D[d] * ((double)a.x[d][j] - a.C[d]);
    double sn, cs;
    sincos(a.sgn * ph, &sn, &cs);
    pre[j].x = (T)cs;
    pre[j].y = (T)sn;
  }
}

// post[k] = exp(i sgn sum_d s_d[k] C_d) / prod_d phihat(tau_d[k]), with
// phihat(tau) = sum_n 2 f_n cos(tau z_n) over the kernel's quadrature nodes
// and tau_d = h_d gam_d (s_d - D_d).
template <typename T>
__global__ void k_postfactor(Type3Phase<T> a, FseriesNodes nodes, long long n, cplx_t<T>* __restrict__ post) {
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    double ph = 0.0, den = 1.0;
    for (int d = 0; d < a.dim; ++d) {
      const double s = (double)a.x[d][k];
      ph += s * a.C[d];
      const double tau = a.hg[d] * (s - a.D[d]);
      double f = 0.0;
      for (int q = 0; q < nodes.q; ++q) f += 2.0 * nodes.f[q] * cos(tau * nodes.z[q]);
      den *= f;
    }
    double sn, cs;
    sincos(a.sgn * ph, &sn, &cs);
    post[k].x = (T)(cs / den);
    post[k].y = (T)(sn / den);
  }
}

// v[t n + i] = u[t n + i] * w[i] (complex), for t < ntr.
template <typename T>
__global__ void k_cmul_rows(const cplx_t<T>* __restrict__ u, const cplx_t<T>* __restrict__ w, long long n, int ntr,
                            cplx_t<T>* __restrict__ v) {
  const long long total = n * ntr;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
    const cplx_t<T> a = u[e], b = w[e % n];
    cplx_t<T> r;
    r.x = a.x * b.x - a.y * b.y;
    r.y = a.x * b.y + a.y * b.x;
    v[e] = r;
  }
}

}  // namespace

template <typename T>
cudaError_t launch_minmax(const T* a, long long n, double* partial, int* nblocks, cudaStream_t s) {
  const int b = t3_grid(n);
  *nblocks = b;
  k_minmax<T><<<b, kT3Threads, 0, s>>>(a, n, partial);
  return cudaGetLastError();
}
int minmax_partials() { return 152 * 8; }

template <typename T>
cudaError_t launch_affine(const T* a, long long n, double centre, double scale, T* out, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_affine<T><<<t3_grid(n), kT3Threads, 0, s>>>(a, n, centre, scale, out);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_prephase(const Type3Phase<T>& a, long long n, cplx_t<T>* pre, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_prephase<T><<<t3_grid(n), kT3Threads, 0, s>>>(a, n, pre);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_postfactor(const Type3Phase<T>& a, const FseriesNodes& nodes, long long n, cplx_t<T>* post,
                              cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_postfactor<T><<<t3_grid(n), kT3Threads, 0, s>>>(a, nodes, n, post);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_cmul_rows(const cplx_t<T>* u, const cplx_t<T>* w, long long n, int ntr, cplx_t<T>* v,
                             cudaStream_t s) {
  if (n <= 0 || ntr <= 0) return cudaSuccess;
  k_cmul_rows<T><<<t3_grid(n * ntr), kT3Threads, 0, s>>>(u, w, n, ntr, v);
  return cudaGetLastError();
}

#define CFG_T3_INST(T)                                                                                  \
  template cudaError_t launch_minmax<T>(const T*, long long, double*, int*, cudaStream_t);              \
  template cudaError_t launch_affine<T>(const T*, long long, double, double, T*, cudaStream_t);         \
  template cudaError_t launch_prephase<T>(const Type3Phase<T>&, long long, cplx_t<T>*, cudaStream_t);   \
  template cudaError_t launch_postfactor<T>(const Type3Phase<T>&, const FseriesNodes&, long long,       \
                                            cplx_t<T>*, cudaStream_t);                                  \
  template cudaError_t launch_cmul_rows<T>(const cplx_t<T>*, const cplx_t<T>*, long long, int, cplx_t<T>*, \
                                           cudaStream_t);
CFG_T3_INST(float)
CFG_T3_INST(double)

}  // namespace cfg
