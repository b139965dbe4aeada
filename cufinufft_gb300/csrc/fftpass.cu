// fftpass.cu -- pruned line FFTs with the deconvolution (type 1) and the
// amplification (type 2) fused into their first or last pass.
//
// The reference runs one cuFFT over the whole upsampled grid and separate
// Deconvolve/Amplify kernels (src/2d/cufinufft2d.cu:73,141,
// src/deconvolve_wrapper.cu:14-254).  With nf_d >= 2 N_d, at most a
// 2^-dim share of the grid holds modes, so most of that traffic moves
// zeros.  Here the d-dimensional transform is done one axis at a time, and
// each axis pass touches only the lines and positions that carry data:
//
//   type 2 (modes -> grid): the first pass reads the compact mode array
//   (CMCL order, x fastest), multiplies by the kernel's Fourier factors,
//   zero-pads in shared memory and writes full lines only for the mode
//   columns; later passes read only the mode positions of their lines.
//   type 1 (grid -> modes): the first pass reads full grid lines and writes
//   back only the mode positions; the last pass writes the compact mode
//   array with the deconvolution factors applied.
//
// Each block holds G whole lines (G a power of two) in shared memory and
// runs a Stockham autosort FFT on them (Govindaraju et al., "High performance discrete Fourier transforms
// on graphics processors", SC 2008): pass s with radix R reads R values
// j + r L/R, twiddles them by w^(r k L/(Ns R)), k = j mod Ns, does an
// R-point DFT in registers and writes them to (j/Ns) Ns R + k + r Ns of a
// second buffer; passes alternate between the two.  Radices 8, 4, 2, 5, 3 cover the 2,3,5-smooth
// lengths next235beven produces.  Twiddles exp(dir 2 pi i m / L) come from a
// per-axis table computed on the host in extended precision.
#include "device_common.cuh"
#include "kernels.h"

namespace cfg {
namespace {

constexpr int kLineThreads = 256;

// Complex helpers, generic over float2 / double2.
template <typename C>
__device__ __forceinline__ C cmul(C a, C b) {
  C r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}
template <typename C>
__device__ __forceinline__ C cadd(C a, C b) {
  C r;
  r.x = a.x + b.x;
  r.y = a.y + b.y;
  return r;
}
template <typename C>
__device__ __forceinline__ C csub(C a, C b) {
  C r;
  r.x = a.x - b.x;
  r.y = a.y - b.y;
  return r;
}
// z * (dir i)
template <typename C, typename S>
__device__ __forceinline__ C cmul_i(C z, S dir) {
  C r;
  r.x = -dir * z.y;
  r.y = dir * z.x;
  return r;
}
template <typename C, typename S>
__device__ __forceinline__ C cscale(C z, S s) {
  C r;
  r.x = z.x * s;
  r.y = z.y * s;
  return r;
}

// R-point DFTs in registers: X_m = sum_r v_r exp(dir 2 pi i r m / R).
template <typename T, int R> struct Dft;

template <typename T> struct Dft<T, 2> {
  static __device__ __forceinline__ void run(cplx_t<T>* v, T) {
    const cplx_t<T> a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  }
};

template <typename T> struct Dft<T, 4> {
  static __device__ __forceinline__ void run(cplx_t<T>* v, T dir) {
    const cplx_t<T> s02 = cadd(v[0], v[2]), d02 = csub(v[0], v[2]);
    const cplx_t<T> s13 = cadd(v[1], v[3]), d13 = cmul_i(csub(v[1], v[3]), dir);
    v[0] = cadd(s02, s13);
    v[2] = csub(s02, s13);
    v[1] = cadd(d02, d13);
    v[3] = csub(d02, d13);
  }
};

template <typename T> struct Dft<T, 8> {
  static __device__ __forceinline__ void run(cplx_t<T>* v, T dir) {
    cplx_t<T> e[4] = {v[0], v[2], v[4], v[6]};
    cplx_t<T> o[4] = {v[1], v[3], v[5], v[7]};
    Dft<T, 4>::run(e, dir);
    Dft<T, 4>::run(o, dir);
    const T h = T(0.70710678118654752440);  // 1/sqrt(2)
    // o_m *= exp(dir 2 pi i m / 8)
    cplx_t<T> w1, w3;
    w1.x = h * (o[1].x - dir * o[1].y);
    w1.y = h * (o[1].y + dir * o[1].x);
    const cplx_t<T> w2 = cmul_i(o[2], dir);
    w3.x = h * (-o[3].x - dir * o[3].y);
    w3.y = h * (-o[3].y + dir * o[3].x);
    v[0] = cadd(e[0], o[0]);
    v[4] = csub(e[0], o[0]);
    v[1] = cadd(e[1], w1);
    v[5] = csub(e[1], w1);
    v[2] = cadd(e[2], w2);
    v[6] = csub(e[2], w2);
    v[3] = cadd(e[3], w3);
    v[7] = csub(e[3], w3);
  }
};

template <typename T> struct Dft<T, 3> {
  static __device__ __forceinline__ void run(cplx_t<T>* v, T dir) {
    const T s3 = T(0.86602540378443864676);  // sin(2 pi / 3)
    const cplx_t<T> t1 = cadd(v[1], v[2]);
    const cplx_t<T> t2 = cmul_i(cscale(csub(v[1], v[2]), s3), dir);
    const cplx_t<T> m = csub(v[0], cscale(t1, T(0.5)));
    v[0] = cadd(v[0], t1);
    v[1] = cadd(m, t2);
    v[2] = csub(m, t2);
  }
};

template <typename T> struct Dft<T, 5> {
  static __device__ __forceinline__ void run(cplx_t<T>* v, T dir) {
    const T c1 = T(0.30901699437494742410);   // cos(2 pi / 5)
    const T c2 = T(-0.80901699437494742410);  // cos(4 pi / 5)
    const T s1 = T(0.95105651629515357212);   // sin(2 pi / 5)
    const T s2 = T(0.58778525229247312917);   // sin(4 pi / 5)
    const cplx_t<T> a = v[0];
    const cplx_t<T> p14 = cadd(v[1], v[4]), m14 = csub(v[1], v[4]);
    const cplx_t<T> p23 = cadd(v[2], v[3]), m23 = csub(v[2], v[3]);
    cplx_t<T> r1, r2, q1, q2;
    r1.x = a.x + c1 * p14.x + c2 * p23.x;
    r1.y = a.y + c1 * p14.y + c2 * p23.y;
    r2.x = a.x + c2 * p14.x + c1 * p23.x;
    r2.y = a.y + c2 * p14.y + c1 * p23.y;
    q1.x = s1 * m14.x + s2 * m23.x;
    q1.y = s1 * m14.y + s2 * m23.y;
    q2.x = s2 * m14.x - s1 * m23.x;
    q2.y = s2 * m14.y - s1 * m23.y;
    q1 = cmul_i(q1, dir);
    q2 = cmul_i(q2, dir);
    v[0] = cadd(a, cadd(p14, p23));
    v[1] = cadd(r1, q1);
    v[4] = csub(r1, q1);
    v[2] = cadd(r2, q2);
    v[3] = csub(r2, q2);
  }
};

// Shared-memory layout of a line: element i at i + i/16.  The extra slot
// every 16 elements (128 bytes of FP32 complex) spreads the strided Stockham
// writes (stride R Ns) over the banks instead of piling them onto one.
__device__ __forceinline__ int sidx(int i) { return i + (i >> 4); }

// One Stockham pass of radix R over G lines of length L (padded stride Lp),
// from src to dst.  POW2: L is a power of two, so the butterfly index splits
// with shifts instead of divisions.
template <typename T, int R, bool POW2>
__device__ __forceinline__ void fft_pass(const cplx_t<T>* __restrict__ src, cplx_t<T>* __restrict__ dst,
                                         int L, int Lp, int G, int Ns,
                                         const cplx_t<T>* __restrict__ tw, T dir) {
  using C = cplx_t<T>;
  const int nbf = L / R;
  const int total = G * nbf;
  const int tstep = L / (Ns * R);
  const int lnbf = POW2 ? __ffs(nbf) - 1 : 0;
  const int lNs = POW2 ? __ffs(Ns) - 1 : 0;
  for (int u = threadIdx.x; u < total; u += kLineThreads) {
    int g, j, q, k;
    if (POW2) {
      g = u >> lnbf;
      j = u & (nbf - 1);
      q = j >> lNs;
      k = j & (Ns - 1);
    } else {
      g = u / nbf;
      j = u - g * nbf;
      q = j / Ns;
      k = j - q * Ns;
    }
    const C* line = src + g * Lp;
    C v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = line[sidx(j + r * nbf)];
    if (Ns > 1) {
#pragma unroll
      for (int r = 1; r < R; ++r) v[r] = cmul(v[r], __ldg(tw + r * k * tstep));
    }
    Dft<T, R>::run(v, dir);
    C* out = dst + g * Lp;
    const int base = q * Ns * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) out[sidx(base + r * Ns)] = v[r];
  }
  __syncthreads();
}

// Asynchronous global -> shared copy of one complex value (cp.async, sm_80+):
// a thread issues all its copies back to back, so a block keeps many loads in
// flight without holding registers for them.
__device__ __forceinline__ void cp_async_c(float2* s, const float2* g) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(s);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(sa), "l"(g) : "memory");
}
__device__ __forceinline__ void cp_async_c(double2* s, const double2* g) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(s);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"(sa), "l"(g) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

// FFT index w -> mode index i in [0, Np), or -1 for a padding position.
__device__ __forceinline__ int mode_index(int w, int L, int Np) {
  if (w <= (Np - 1) / 2) return w + Np / 2;
  if (w >= L - Np / 2) return w - L + Np / 2;
  return -1;
}
// mode index i -> FFT index
__device__ __forceinline__ int mode_pos(int i, int L, int Np) {
  const int k = i - Np / 2;
  return k >= 0 ? k : L + k;
}

__device__ __forceinline__ long long side_line(const LineSide& s, int la, int lb) {
  const long long ma = s.acorner ? mode_pos(la, s.nfa, s.Na) : la;
  const long long mb = s.bcorner ? mode_pos(lb, s.nfb, s.Nb) : lb;
  return ma * s.sa + mb * s.sb;
}

template <typename T>
__device__ __forceinline__ T line_factor(const LineArgs<T>& a, int la, int lb, int i) {
  T f = T(1);
  if (a.fa) f *= a.fa[la];
  if (a.fb) f *= a.fb[lb];
  if (a.fp && i >= 0) f *= a.fp[i];
  return f;
}

template <typename T, int CAP>
__global__ void __launch_bounds__(kLineThreads)
k_line_fft(LineArgs<T> a) {
  using C = cplx_t<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int L = a.L, G = a.G;
  const int Lp = L + (L >> 4) + 1;                       // padded line stride
  C* buf0 = reinterpret_cast<C*>(smem_raw);              // two buffers of G * Lp
  C* buf1 = buf0 + G * Lp;
  const int line0 = blockIdx.x * G;
  const T dir = T(a.dir);
  const bool pow2 = (L & (L - 1)) == 0;
  const C zero = C{T(0), T(0)};
  for (int t = blockIdx.y; t < a.ntr; t += gridDim.y) {
    const C* in = a.in + (long long)t * a.si.st;
    C* out = a.out + (long long)t * a.so.st;
    // ---- load G lines into buf0: copies for data positions, zeros for
    // padding positions and for lines past the last one
    const LineSide& si = a.si;
    const bool factor_in = !a.fac_on_out && (a.fa || a.fb || a.fp);
    const bool rows_in = si.sp == 1;   // positions contiguous: lanes along the line
    const int g_fix = threadIdx.x & (G - 1);  // columns: consecutive lanes take consecutive lines
    const int w0 = rows_in ? threadIdx.x : (threadIdx.x >> a.log2G);
    const int wstep = rows_in ? kLineThreads : (kLineThreads >> a.log2G);
    for (int gg = 0; gg < (rows_in ? G : 1); ++gg) {
      const int g = rows_in ? gg : g_fix;
      const int line = line0 + g;
      C* dstl = buf0 + g * Lp;
      if (line >= a.nlines) {
        for (int w = w0; w < L; w += wstep) dstl[sidx(w)] = zero;
        continue;
      }
      const int la = line % a.A, lb = line / a.A;
      const C* src = in + side_line(si, la, lb);
      for (int w = w0; w < L; w += wstep) {
        const int i = si.pmode ? mode_index(w, L, si.Np) : -1;
        if (!si.pmode || i >= 0)
          cp_async_c(dstl + sidx(w), src + (long long)(si.pmode == 1 ? i : w) * si.sp);
        else
          dstl[sidx(w)] = zero;
      }
    }
    cp_async_wait_all();
    if (factor_in) {  // each thread scales the values it copied
      for (int gg = 0; gg < (rows_in ? G : 1); ++gg) {
        const int g = rows_in ? gg : g_fix;
        const int line = line0 + g;
        if (line >= a.nlines) continue;
        const int la = line % a.A, lb = line / a.A;
        const T f0 = line_factor(a, la, lb, -1);
        C* dstl = buf0 + g * Lp;
        for (int w = w0; w < L; w += wstep) {
          const int i = si.pmode ? mode_index(w, L, si.Np) : -1;
          if (!si.pmode || i >= 0)
            dstl[sidx(w)] = cscale(dstl[sidx(w)], (a.fp && i >= 0) ? f0 * a.fp[i] : f0);
        }
      }
    }
    __syncthreads();
    // ---- Stockham passes, alternating between the two buffers
    C* cur = buf0;
    C* nxt = buf1;
    int Ns = 1;
    for (int s = 0; s < a.nrad; ++s) {
      switch (a.rad[s]) {
        case 8:
          if (pow2) fft_pass<T, 8, true>(cur, nxt, L, Lp, G, Ns, a.tw, dir);
          else fft_pass<T, 8, false>(cur, nxt, L, Lp, G, Ns, a.tw, dir);
          break;
        case 4:
          if (pow2) fft_pass<T, 4, true>(cur, nxt, L, Lp, G, Ns, a.tw, dir);
          else fft_pass<T, 4, false>(cur, nxt, L, Lp, G, Ns, a.tw, dir);
          break;
        case 2:
          if (pow2) fft_pass<T, 2, true>(cur, nxt, L, Lp, G, Ns, a.tw, dir);
          else fft_pass<T, 2, false>(cur, nxt, L, Lp, G, Ns, a.tw, dir);
          break;
        case 5: fft_pass<T, 5, false>(cur, nxt, L, Lp, G, Ns, a.tw, dir); break;
        default: fft_pass<T, 3, false>(cur, nxt, L, Lp, G, Ns, a.tw, dir); break;
      }
      Ns *= a.rad[s];
      C* t2 = cur;
      cur = nxt;
      nxt = t2;
    }
    // ---- store the output positions of each line from cur
    const LineSide& so = a.so;
    const bool factor_out = a.fac_on_out != 0;
    const int count = so.pmode ? so.Np : L;
    const bool rows_out = so.sp == 1;
    const int q0 = rows_out ? threadIdx.x : (threadIdx.x >> a.log2G);
    const int qstep = rows_out ? kLineThreads : (kLineThreads >> a.log2G);
    for (int gg = 0; gg < (rows_out ? G : 1); ++gg) {
      const int g = rows_out ? gg : g_fix;
      const int line = line0 + g;
      if (line >= a.nlines) continue;
      const int la = line % a.A, lb = line / a.A;
      C* dst = out + side_line(so, la, lb);
      const C* srcl = cur + g * Lp;
      const T f0 = factor_out ? line_factor(a, la, lb, -1) : T(1);
      for (int q = q0; q < count; q += qstep) {
        const int w = so.pmode ? mode_pos(q, L, so.Np) : q;
        C v = srcl[sidx(w)];
        if (factor_out) v = cscale(v, (a.fp && so.pmode) ? f0 * a.fp[q] : f0);
        dst[(long long)(so.pmode == 1 ? q : w) * so.sp] = v;
      }
    }
    __syncthreads();  // the buffers are reused by the next transform
  }
}

template <typename T> constexpr int line_cap() { return sizeof(T) == 4 ? 8192 : 4096; }

}  // namespace

template <typename T> int line_fft_cap() { return line_cap<T>(); }

template <typename T>
cudaError_t line_fft_prepare() {
  return cudaFuncSetAttribute(k_line_fft<T, line_cap<T>()>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                              2 * (line_cap<T>() + line_cap<T>() / 16 + 1) * (int)sizeof(cplx_t<T>));
}

template <typename T>
cudaError_t launch_line_fft(const LineArgs<T>& a, cudaStream_t s) {
  if (a.nlines <= 0 || a.ntr <= 0) return cudaSuccess;
  const size_t smem = 2 * (size_t)a.G * (a.L + a.L / 16 + 1) * sizeof(cplx_t<T>);
  dim3 grid((a.nlines + a.G - 1) / a.G, a.ntr < 65535 ? a.ntr : 65535);
  k_line_fft<T, line_cap<T>()><<<grid, kLineThreads, smem, s>>>(a);
  return cudaGetLastError();
}

template int line_fft_cap<float>();
template int line_fft_cap<double>();
template cudaError_t line_fft_prepare<float>();
template cudaError_t line_fft_prepare<double>();
template cudaError_t launch_line_fft<float>(const LineArgs<float>&, cudaStream_t);
template cudaError_t launch_line_fft<double>(const LineArgs<double>&, cudaStream_t);

}  // namespace cfg
