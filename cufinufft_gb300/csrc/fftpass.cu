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

// 16-point DFT as 4 x 4: DFT-4 over n2 (stride 4), twiddles W16^(n1 k2),
// DFT-4 over n1; X[k2 + 4 k1].
template <typename T> struct Dft<T, 16> {
  static __device__ __forceinline__ void run(cplx_t<T>* v, T dir) {
    using C = cplx_t<T>;
    const T c1 = T(0.92387953251128675613);  // cos(pi/8)
    const T s1 = T(0.38268343236508977173);  // sin(pi/8)
    const T h = T(0.70710678118654752440);   // 1/sqrt(2)
    C y[4][4];
#pragma unroll
    for (int n1 = 0; n1 < 4; ++n1) {
      C a[4] = {v[n1], v[n1 + 4], v[n1 + 8], v[n1 + 12]};
      Dft<T, 4>::run(a, dir);
#pragma unroll
      for (int k2 = 0; k2 < 4; ++k2) y[n1][k2] = a[k2];
    }
    const C w1 = C{c1, dir * s1}, w2 = C{h, dir * h}, w3 = C{s1, dir * c1};
    const C w6 = C{-h, dir * h}, w9 = C{-c1, -dir * s1};
    y[1][1] = cmul(y[1][1], w1);
    y[1][2] = cmul(y[1][2], w2);
    y[1][3] = cmul(y[1][3], w3);
    y[2][1] = cmul(y[2][1], w2);
    y[2][2] = cmul_i(y[2][2], dir);
    y[2][3] = cmul(y[2][3], w6);
    y[3][1] = cmul(y[3][1], w3);
    y[3][2] = cmul(y[3][2], w6);
    y[3][3] = cmul(y[3][3], w9);
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) {
      C b[4] = {y[0][k2], y[1][k2], y[2][k2], y[3][k2]};
      Dft<T, 4>::run(b, dir);
#pragma unroll
      for (int k1 = 0; k1 < 4; ++k1) v[k2 + 4 * k1] = b[k1];
    }
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

// ---------------------------------------------------------------------------
// Power-of-two lines, register-resident passes.  Block = G * L / 16 threads
// (G lines of L = 2^m >= 16 points, at most 512 threads); radices 16, ...,
// 16 then one of 8/4/2.
// Every pass gives each thread exactly 16/R butterflies, so values stay in
// registers: the first pass loads its 16 inputs straight from global memory
// (the padding positions of a pruned line are not read), middle passes
// exchange through one padded shared buffer, and the last pass stores its
// outputs straight to global memory (only the mode positions of a pruned
// line), with the per-mode factors applied on the way in or out.

// v[r] *= w^(r * e), r = 1..R-1, from the table entries w^e, w^2e, w^4e,
// w^8e and products of at most three of them.
template <typename T, int R>
__device__ __forceinline__ void twiddle_p2(cplx_t<T>* v, int e, const cplx_t<T>* __restrict__ tw) {
  using C = cplx_t<T>;
  const C w1 = __ldg(tw + e);
  if (R == 2) {
    v[1] = cmul(v[1], w1);
    return;
  }
  const C w2 = __ldg(tw + 2 * e);
  const C w3 = cmul(w1, w2);
  v[1] = cmul(v[1], w1);
  v[2] = cmul(v[2], w2);
  v[3] = cmul(v[3], w3);
  if (R == 4) return;
  const C w4 = __ldg(tw + 4 * e);
  v[4] = cmul(v[4], w4);
  v[5] = cmul(v[5], cmul(w1, w4));
  v[6] = cmul(v[6], cmul(w2, w4));
  const C w7 = cmul(w3, w4);
  v[7] = cmul(v[7], w7);
  if (R == 8) return;
  const C w8 = __ldg(tw + 8 * e);
  v[8] = cmul(v[8], w8);
  v[9] = cmul(v[9], cmul(w1, w8));
  v[10] = cmul(v[10], cmul(w2, w8));
  v[11] = cmul(v[11], cmul(w3, w8));
  v[12] = cmul(v[12], cmul(w4, w8));
  v[13] = cmul(v[13], cmul(cmul(w1, w4), w8));
  v[14] = cmul(v[14], cmul(cmul(w2, w4), w8));
  v[15] = cmul(v[15], cmul(w7, w8));
}

// Per-block state of the power-of-two kernel.
template <typename T> struct P2Ctx {
  const LineArgs<T>* a;
  const cplx_t<T>* in;
  cplx_t<T>* out;
  cplx_t<T>* buf;
  int L, lgL, Lp, lgG, T_, line0;
  T dir;
};

// Line g and position j of butterfly u: lines contiguous in memory (column
// passes) take consecutive lanes; otherwise positions do.
__device__ __forceinline__ void p2_split(int u, int lg_nbf, int lgG, bool lines_fast, int& g, int& j) {
  if (lines_fast) {
    g = u & ((1 << lgG) - 1);
    j = u >> lgG;
  } else {
    g = u >> lg_nbf;
    j = u & ((1 << lg_nbf) - 1);
  }
}

// Pass 1 (radix 16, Ns = 1): global -> registers -> DFT -> shared, or
// global when it is also the last pass (L = 16).
template <typename T, bool LAST>
__device__ __forceinline__ void p2_first(const P2Ctx<T>& c) {
  using C = cplx_t<T>;
  const LineArgs<T>& a = *c.a;
  const LineSide& si = a.si;
  const int lg_nbf = c.lgL - 4;
  const int nbf = 1 << lg_nbf;
  int g, j;
  p2_split(threadIdx.x, lg_nbf, c.lgG, si.sp != 1, g, j);
  const int line = c.line0 + g;
  C v[16];
  if (line < a.nlines) {
    const int la = line % a.A, lb = line / a.A;
    const C* src = c.in + side_line(si, la, lb);
    const bool fac = !a.fac_on_out && (a.fa || a.fb || a.fp);
    const T f0 = fac ? line_factor(a, la, lb, -1) : T(1);
#pragma unroll
    for (int r = 0; r < 16; ++r) {
      const int w = j + r * nbf;
      const int i = si.pmode ? mode_index(w, c.L, si.Np) : -1;
      if (!si.pmode || i >= 0) {
        v[r] = src[(long long)(si.pmode == 1 ? i : w) * si.sp];
        if (fac) v[r] = cscale(v[r], (a.fp && i >= 0) ? f0 * a.fp[i] : f0);
      } else {
        v[r] = C{T(0), T(0)};
      }
    }
  } else {
#pragma unroll
    for (int r = 0; r < 16; ++r) v[r] = C{T(0), T(0)};
  }
  Dft<T, 16>::run(v, c.dir);
  if (LAST) {
    if (line >= a.nlines) return;
    const LineSide& so = a.so;
    const int la = line % a.A, lb = line / a.A;
    C* dst = c.out + side_line(so, la, lb);
    const bool fac = a.fac_on_out != 0;
    const T f0 = fac ? line_factor(a, la, lb, -1) : T(1);
#pragma unroll
    for (int r = 0; r < 16; ++r) {  // j = 0: output r at position r
      const int q = so.pmode ? mode_index(r, c.L, so.Np) : r;
      if (q < 0) continue;
      C o = v[r];
      if (fac) o = cscale(o, (a.fp && so.pmode) ? f0 * a.fp[q] : f0);
      dst[(long long)(so.pmode == 1 ? q : r) * so.sp] = o;
    }
  } else {
    C* l = c.buf + g * c.Lp;
    const int base = sidx(j * 16);  // j*16 + r stays inside one 16-block
#pragma unroll
    for (int r = 0; r < 16; ++r) l[base + r] = v[r];
  }
}

// A middle or last pass of radix R with Ns = 2^lgNs: shared -> registers ->
// twiddle, DFT -> shared (middle) or global (last).
template <typename T, int R, bool LAST>
__device__ __forceinline__ void p2_pass(const P2Ctx<T>& c, int lgNs) {
  using C = cplx_t<T>;
  constexpr int NB = 16 / R;
  constexpr int lgR = R == 16 ? 4 : (R == 8 ? 3 : (R == 4 ? 2 : 1));
  const int lg_nbf = c.lgL - lgR;
  const int nbf = 1 << lg_nbf;
  const int Ns = 1 << lgNs;
  const int lg_tstep = c.lgL - lgNs - lgR;
  const LineArgs<T>& a = *c.a;
  const bool lines_fast = LAST && a.so.sp != 1;
  C v[NB][R];
  int gg[NB], jj[NB];
#pragma unroll
  for (int b = 0; b < NB; ++b) {
    p2_split(threadIdx.x + b * c.T_, lg_nbf, c.lgG, lines_fast, gg[b], jj[b]);
    const C* l = c.buf + gg[b] * c.Lp;
#pragma unroll
    for (int r = 0; r < R; ++r) v[b][r] = l[sidx(jj[b] + r * nbf)];
  }
  __syncthreads();  // every read of this pass is done before any write
#pragma unroll
  for (int b = 0; b < NB; ++b) {
    const int k = jj[b] & (Ns - 1);
    twiddle_p2<T, R>(v[b], k << lg_tstep, a.tw);
    Dft<T, R>::run(v[b], c.dir);
  }
  if (!LAST) {
#pragma unroll
    for (int b = 0; b < NB; ++b) {
      const int k = jj[b] & (Ns - 1), q = jj[b] >> lgNs;
      C* l = c.buf + gg[b] * c.Lp;
      const int base = (q << (lgNs + lgR)) + k;
#pragma unroll
      for (int r = 0; r < R; ++r) l[sidx(base + r * Ns)] = v[b][r];
    }
    __syncthreads();
    return;
  }
  // last pass: nbf = Ns, so q = 0 and output r of butterfly j is at j + r Ns
  const LineSide& so = a.so;
  const bool fac = a.fac_on_out != 0;
#pragma unroll
  for (int b = 0; b < NB; ++b) {
    const int line = c.line0 + gg[b];
    if (line >= a.nlines) continue;
    const int la = line % a.A, lb = line / a.A;
    C* dst = c.out + side_line(so, la, lb);
    const T f0 = fac ? line_factor(a, la, lb, -1) : T(1);
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int w = jj[b] + r * Ns;
      const int q = so.pmode ? mode_index(w, c.L, so.Np) : w;
      if (q < 0) continue;
      C o = v[b][r];
      if (fac) o = cscale(o, (a.fp && so.pmode) ? f0 * a.fp[q] : f0);
      dst[(long long)(so.pmode == 1 ? q : w) * so.sp] = o;
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(512)
k_line_fft_p2(LineArgs<T> a) {
  using C = cplx_t<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  P2Ctx<T> c;
  c.a = &a;
  c.L = a.L;
  c.lgL = __ffs(a.L) - 1;
  c.Lp = a.L + (a.L >> 4) + 1;
  c.lgG = a.log2G;
  c.T_ = blockDim.x;
  c.line0 = blockIdx.x * a.G;
  c.dir = T(a.dir);
  c.buf = reinterpret_cast<C*>(smem_raw);
  // radices: 16 (n16 times), then rem in {1 (none), 2, 4, 8}
  const int n16 = c.lgL / 4;
  const int rem = 1 << (c.lgL - 4 * n16);
  for (int t = blockIdx.y; t < a.ntr; t += gridDim.y) {
    c.in = a.in + (long long)t * a.si.st;
    c.out = a.out + (long long)t * a.so.st;
    if (n16 == 1 && rem == 1) {
      p2_first<T, true>(c);
      continue;
    }
    p2_first<T, false>(c);
    __syncthreads();
    int lgNs = 4;
    for (int s = 1; s < n16; ++s) {
      if (s == n16 - 1 && rem == 1) p2_pass<T, 16, true>(c, lgNs);
      else p2_pass<T, 16, false>(c, lgNs);
      lgNs += 4;
    }
    if (rem == 8) p2_pass<T, 8, true>(c, lgNs);
    else if (rem == 4) p2_pass<T, 4, true>(c, lgNs);
    else if (rem == 2) p2_pass<T, 2, true>(c, lgNs);
    __syncthreads();  // the buffer is reused by the next transform
  }
}

// Longest line: 8192 points FP32, 4096 FP64 (two padded buffers of ~68 KB)
// for the generic kernel.
template <typename T> constexpr int line_cap() { return sizeof(T) == 4 ? 8192 : 4096; }
// Power-of-two kernel: G * L <= 4096 FP32 / 2048 FP64 points per block
// along x (256 / 128 threads, 16 values each), twice that along y and z.
template <typename T> constexpr int line_p2_elems() { return sizeof(T) == 4 ? 4096 : 2048; }

}  // namespace

template <typename T> int line_fft_cap() { return line_cap<T>(); }
template <typename T> int line_fft_p2_elems() { return line_p2_elems<T>(); }

template <typename T>
cudaError_t line_fft_prepare() {
  cudaError_t e = cudaFuncSetAttribute(k_line_fft<T, line_cap<T>()>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       2 * (line_cap<T>() + line_cap<T>() / 16 + 1) * (int)sizeof(cplx_t<T>));
  if (e != cudaSuccess) return e;
  // G * (L + L/16 + 1) <= E * 18/16 for E = G * L <= twice line_p2_elems, L >= 16
  return cudaFuncSetAttribute(k_line_fft_p2<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              2 * line_p2_elems<T>() * 18 / 16 * (int)sizeof(cplx_t<T>));
}

template <typename T>
cudaError_t launch_line_fft(const LineArgs<T>& a, cudaStream_t s) {
  if (a.nlines <= 0 || a.ntr <= 0) return cudaSuccess;
  if (a.p2) {
    const int threads = a.G * a.L / 16;
    const size_t smem = (size_t)a.G * (a.L + a.L / 16 + 1) * sizeof(cplx_t<T>);
    dim3 grid((a.nlines + a.G - 1) / a.G, a.ntr < 65535 ? a.ntr : 65535);
    k_line_fft_p2<T><<<grid, threads, smem, s>>>(a);
    return cudaGetLastError();
  }
  const size_t smem = 2 * (size_t)a.G * (a.L + a.L / 16 + 1) * sizeof(cplx_t<T>);
  dim3 grid((a.nlines + a.G - 1) / a.G, a.ntr < 65535 ? a.ntr : 65535);
  k_line_fft<T, line_cap<T>()><<<grid, kLineThreads, smem, s>>>(a);
  return cudaGetLastError();
}

template int line_fft_cap<float>();
template int line_fft_cap<double>();
template int line_fft_p2_elems<float>();
template int line_fft_p2_elems<double>();
template cudaError_t line_fft_prepare<float>();
template cudaError_t line_fft_prepare<double>();
template cudaError_t launch_line_fft<float>(const LineArgs<float>&, cudaStream_t);
template cudaError_t launch_line_fft<double>(const LineArgs<double>&, cudaStream_t);

}  // namespace cfg
