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

// Deconvolution and amplification move data between the mode cube and the
// mode cells of the fine grid, one mode row (fixed k2, k3) at a time.  A
// block is tx x ty threads: ty rows, tx threads along a row, each thread
// kRowUnroll cells of its row per pass with every load issued before the
// first store; long rows are split into chunks of kRowUnroll tx cells
// (blockIdx.x = row block * nchunks + chunk), blockIdx.y = transform.
constexpr int kRowUnroll = 4;

template <typename T> struct ModeRows {
  int nf0, nf1, nf2, N0, N1, N2;
  int nrows, nchunks;
  long long Nf, Nm;
  const T *fac0, *fac1, *fac2;
};

// AMPLIFY false: fk[mode] = fw[cell] * fac (type 1); true: fw[cell] =
// fk[mode] * fac (type 2).
template <typename T, int DIM, bool AMPLIFY>
__global__ void __launch_bounds__(256)
k_mode_rows(ModeRows<T> m, const cplx_t<T>* __restrict__ in, cplx_t<T>* __restrict__ out) {
  using C = cplx_t<T>;
  const unsigned rb = blockIdx.x / (unsigned)m.nchunks;
  const int chunk = (int)(blockIdx.x - rb * (unsigned)m.nchunks);
  const int rr = (int)rb * blockDim.y + threadIdx.y;
  if (rr >= m.nrows) return;
  const int t = blockIdx.y;
  int i2 = 0, i3 = 0;
  if (DIM == 2) i2 = rr;
  if (DIM == 3) {
    i3 = rr / m.N1;
    i2 = rr - i3 * m.N1;
  }
  const int k2 = i2 - m.N1 / 2, k3 = i3 - m.N2 / 2;
  const int w2 = k2 >= 0 ? k2 : m.nf1 + k2;
  const int w3 = k3 >= 0 ? k3 : m.nf2 + k3;
  T f23 = T(1);
  if (DIM > 1) f23 = m.fac1[i2];
  if (DIM > 2) f23 *= m.fac2[i3];
  const size_t cell_row = (size_t)t * m.Nf + ((size_t)w3 * m.nf1 + w2) * m.nf0;
  const size_t mode_row = (size_t)t * m.Nm + ((size_t)i3 * m.N1 + i2) * m.N0;
  const C* src = in + (AMPLIFY ? mode_row : cell_row);
  C* dst = out + (AMPLIFY ? cell_row : mode_row);
  const int h0 = m.N0 / 2;
  const int b = chunk * kRowUnroll * blockDim.x + threadIdx.x;
  C v[kRowUnroll];
  T f[kRowUnroll];
#pragma unroll
  for (int u = 0; u < kRowUnroll; ++u) {
    const int i1 = b + u * blockDim.x;
    if (i1 < m.N0) {
      const int k1 = i1 - h0;
      v[u] = src[AMPLIFY ? i1 : (k1 >= 0 ? k1 : m.nf0 + k1)];
      f[u] = m.fac0[i1];
    }
  }
#pragma unroll
  for (int u = 0; u < kRowUnroll; ++u) {
    const int i1 = b + u * blockDim.x;
    if (i1 < m.N0) {
      const int k1 = i1 - h0;
      const T g = f[u] * f23;
      C o;
      o.x = v[u].x * g;
      o.y = v[u].y * g;
      dst[AMPLIFY ? (k1 >= 0 ? k1 : m.nf0 + k1) : i1] = o;
    }
  }
}

template <typename T, bool AMPLIFY>
static cudaError_t launch_mode_rows(int dim, const int nf[3], const int N[3], const cplx_t<T>* in,
                                    cplx_t<T>* out, const T* fac0, const T* fac1, const T* fac2, int ntr,
                                    cudaStream_t s) {
  ModeRows<T> m;
  m.nf0 = nf[0];
  m.nf1 = nf[1];
  m.nf2 = nf[2];
  m.N0 = N[0];
  m.N1 = dim > 1 ? N[1] : 1;
  m.N2 = dim > 2 ? N[2] : 1;
  m.Nf = (long long)nf[0] * nf[1] * nf[2];
  m.Nm = (long long)N[0] * N[1] * N[2];
  m.nrows = m.N1 * m.N2;
  m.fac0 = fac0;
  m.fac1 = fac1;
  m.fac2 = fac2;
  if (m.N0 <= 0 || m.nrows <= 0 || ntr <= 0) return cudaSuccess;
  // tx: enough threads for a row in one pass, a multiple of 32, at most 256
  const int per = (m.N0 + kRowUnroll - 1) / kRowUnroll;
  const int tx = std::min(256, std::max(32, (per + 31) / 32 * 32));
  const int ty = 256 / tx;
  m.nchunks = (m.N0 + kRowUnroll * tx - 1) / (kRowUnroll * tx);
  const long long blocks = (long long)((m.nrows + ty - 1) / ty) * m.nchunks;
  if (blocks > 0x7fffffffLL) return cudaErrorInvalidValue;
  for (int t0 = 0; t0 < ntr; t0 += 65535) {
    const int nt = std::min(ntr - t0, 65535);
    const size_t off = (size_t)t0 * (AMPLIFY ? m.Nm : m.Nf), offo = (size_t)t0 * (AMPLIFY ? m.Nf : m.Nm);
    dim3 grid((unsigned)blocks, nt);
    dim3 block(tx, ty);
    switch (dim) {
      case 1: k_mode_rows<T, 1, AMPLIFY><<<grid, block, 0, s>>>(m, in + off, out + offo); break;
      case 2: k_mode_rows<T, 2, AMPLIFY><<<grid, block, 0, s>>>(m, in + off, out + offo); break;
      default: k_mode_rows<T, 3, AMPLIFY><<<grid, block, 0, s>>>(m, in + off, out + offo); break;
    }
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

template <typename T>
cudaError_t launch_deconvolve(int dim, const int nf[3], const int N[3], const cplx_t<T>* fw,
                              cplx_t<T>* fk, const T* fac0, const T* fac1, const T* fac2, int ntr,
                              cudaStream_t s) {
  return launch_mode_rows<T, false>(dim, nf, N, fw, fk, fac0, fac1, fac2, ntr, s);
}

// Type-2 amplification into a grid whose padding is already zero (the FFT
// then runs out of place): only the mode cells are written.
template <typename T>
cudaError_t launch_amplify_modes(int dim, const int nf[3], const int N[3], cplx_t<T>* fw,
                                 const cplx_t<T>* fk, const T* fac0, const T* fac1, const T* fac2,
                                 int ntr, cudaStream_t s) {
  return launch_mode_rows<T, true>(dim, nf, N, fk, fw, fac0, fac1, fac2, ntr, s);
}

// FP64 <-> FP32 complex conversion (the FP32 chain of an FP64 plan): one
// 16-byte load and one 8-byte store per value, grid-stride.
__global__ void k_narrow_complex(const double2* __restrict__ in, float2* __restrict__ out, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double2 v = in[i];
    out[i] = make_float2((float)v.x, (float)v.y);
  }
}
__global__ void k_widen_complex(const float2* __restrict__ in, double2* __restrict__ out, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const float2 v = in[i];
    out[i] = make_double2((double)v.x, (double)v.y);
  }
}
static int convert_grid(long long n) {
  long long b = (n + 255) / 256;
  if (b > 152LL * 16) b = 152LL * 16;
  return b < 1 ? 1 : (int)b;
}
cudaError_t launch_narrow_complex(const double2* in, float2* out, long long n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_narrow_complex<<<convert_grid(n), 256, 0, s>>>(in, out, n);
  return cudaGetLastError();
}
cudaError_t launch_widen_complex(const float2* in, double2* out, long long n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_widen_complex<<<convert_grid(n), 256, 0, s>>>(in, out, n);
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
