// halffft.cu -- pruned FFT passes for power-of-two fine grids at upsampling
// factor 2, with the amplification (type 2) or deconvolution (type 1) fused.
//
// At upsampling factor 2 at most half of each grid line holds modes.  A
// d-dimensional transform is done one axis at a time, and each pass touches
// only the lines that hold data: type 2 starts along x on the compact mode
// array (amplification fused), continues along y (and z) over the mode
// lines, and writes the grid; type 1 runs along z (and y) over the whole
// grid, then along x writing the compact mode array (deconvolution fused).
// Intermediate arrays hold only the mode lines, so the zero padding is never
// read or written.
//
// A line of L = F M' points (M' = 32 Q = 128 or 256, F classes) is handled
// as F M'-point FFTs, one warp each, so that every warp holds only Q <= 8
// values a lane and many warps are in flight:
//   type 2 (modes a_k -> grid, k in [-N/2, N/2)):
//     X[F r + q] = sum_n [sum_{k = n mod M'} a_k W_L^(k q)] W_M'^(n r),
//   the modes folded onto M' positions with the class twiddle W_L^(k q);
//   type 1 (grid x -> modes):
//     Y[k] = sum_q W_L^(k q) FFT_M'(x[F j + q])[k mod M'],
// with W_n = exp(dir 2 pi i / n).
//
// The M'-point FFT of a warp (warp_fft) is a four-step: a Q-point DFT in
// registers, twiddles, a transpose through shared memory, a second DFT in
// registers and, for Q < 32, a short DFT across lanes by shuffles.
// Results go through shared memory (XOR-swizzled or padded, the layouts
// enumerated on the CPU so that the FFT's scattered writes and the
// natural-order reads fall in distinct banks) to coalesced stores.  The
// twiddles of the in-register DFTs are constants; the others come from the
// plan's per-axis table W_L^t, t < L (extended precision on the host).
#include <algorithm>

#include "device_common.cuh"
#include "kernels.h"

namespace cfg {
namespace {

template <typename C>
__device__ __forceinline__ C hcmul(C a, C b) {
  C r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}
template <typename C>
__device__ __forceinline__ C hcadd(C a, C b) {
  C r;
  r.x = a.x + b.x;
  r.y = a.y + b.y;
  return r;
}
template <typename C>
__device__ __forceinline__ C hcsub(C a, C b) {
  C r;
  r.x = a.x - b.x;
  r.y = a.y - b.y;
  return r;
}

template <int BITS>
__host__ __device__ constexpr int brev(int x) {
  int r = 0;
  for (int b = 0; b < BITS; ++b)
    if ((x >> b) & 1) r |= 1 << (BITS - 1 - b);
  return r;
}
template <int Q> constexpr int log2i() { return Q <= 1 ? 0 : 1 + log2i<Q / 2>(); }

// cos(2 pi i / 64), i = 0..16: the twiddles of the in-register DFTs (up to
// 32 points) are compile-time constants.
__device__ constexpr double kCos64[17] = {
    1.0, 0.9951847266721969, 0.9807852804032304, 0.9569403357322088, 0.9238795325112867,
    0.881921264348355, 0.8314696123025452, 0.773010453362737, 0.7071067811865476,
    0.6343932841636455, 0.5555702330196023, 0.4713967368259978, 0.38268343236508984,
    0.29028467725446233, 0.19509032201612833, 0.09801714032956077, 0.0};
__device__ constexpr double cos64(int u) {
  u &= 63;
  return u <= 16 ? kCos64[u] : (u <= 32 ? -kCos64[32 - u] : (u <= 48 ? -kCos64[u - 32] : kCos64[64 - u]));
}
// W_N^t = exp(DIR 2 pi i t / N) for N dividing 64.
template <typename T, int DIR>
__device__ __forceinline__ cplx_t<T> wconst(int N, int t) {
  const int u = t * (64 / N);
  cplx_t<T> w;
  w.x = (T)cos64(u);
  w.y = (T)(DIR * cos64(u - 16));
  return w;
}

// In-register radix-2 DIF of Q points with constant twiddles: on exit
// v[k] = V[rev_Q(k)], V[j] = sum_m v_in[m] W_Q^(m j).
template <typename T, int Q, int DIR>
__device__ __forceinline__ void reg_dif(cplx_t<T> (&v)[Q]) {
  using C = cplx_t<T>;
#pragma unroll
  for (int h = Q / 2; h >= 1; h >>= 1) {
#pragma unroll
    for (int b = 0; b < Q; b += 2 * h) {
#pragma unroll
      for (int i = 0; i < h; ++i) {
        const C a = v[b + i], c = v[b + i + h];
        v[b + i] = hcadd(a, c);
        const C d = hcsub(a, c);
        v[b + i + h] = i == 0 ? d : hcmul(d, wconst<T, DIR>(2 * h, i));
      }
    }
  }
}

// Warp FFT of M = 32 Q points.  On entry v[m] = x[lane + 32 m].  tw[t] =
// W_L^t is the table of the line (L = F M), so W_M^t = tw[F t] and W_32^t =
// tw[F Q t].  G = 32/Q lanes share each column of the lane dimension after
// the transpose.
//   (1) Q-point DFT over m in registers;
//   (2) twiddles W_M^(lane j1) from the table;
//   (3) transpose through `scratch` (32 Q elements, an XOR layout free of
//       bank conflicts) so that lane t = G j1 + g holds D[g + G s][j1],
//       s < Q; a Q-point DFT over s in registers; for G > 1, twiddles
//       W_32^(g r) and a G-point DFT over the G lanes by shuffles.
// On exit lane t, register k holds X[j1 + Q rev_Q(k) + Q^2 rev_G(g)].
template <typename T, int Q, int DIR>
__device__ __forceinline__ void warp_fft(cplx_t<T> (&v)[Q], const cplx_t<T>* __restrict__ tw, int lane,
                                         cplx_t<T>* scratch, int F) {
  using C = cplx_t<T>;
  constexpr int QB = log2i<Q>();
  constexpr int G = 32 / Q;
  reg_dif<T, Q, DIR>(v);
#pragma unroll
  for (int k = 1; k < Q; ++k) v[k] = hcmul(v[k], __ldg(tw + F * lane * brev<QB>(k)));
#pragma unroll
  for (int k = 0; k < Q; ++k) {
    const int r = brev<QB>(k);
    scratch[r * 32 + (lane ^ (G * r))] = v[k];
  }
  __syncwarp();
  const int j1 = lane / G, g = lane % G;
#pragma unroll
  for (int s = 0; s < Q; ++s) v[s] = scratch[j1 * 32 + g + G * (s ^ j1)];
  __syncwarp();  // the caller may reuse the scratch
  reg_dif<T, Q, DIR>(v);
  if constexpr (G > 1) {
#pragma unroll
    for (int k = 1; k < Q; ++k) v[k] = hcmul(v[k], __ldg(tw + F * Q * g * brev<QB>(k)));
#pragma unroll
    for (int h = G / 2; h >= 1; h >>= 1) {
      const bool up = (g & h) != 0;
      const C w = __ldg(tw + F * Q * ((g & (h - 1)) * (16 / h)));
#pragma unroll
      for (int k = 0; k < Q; ++k) {
        C o;
        o.x = __shfl_xor_sync(0xffffffffu, v[k].x, h);
        o.y = __shfl_xor_sync(0xffffffffu, v[k].y, h);
        v[k] = up ? hcmul(hcsub(o, v[k]), w) : hcadd(v[k], o);
      }
    }
  }
}

// Output index held by lane, register k after warp_fft.
template <int Q>
__device__ __forceinline__ int fft_out_index(int k, int lane) {
  constexpr int G = 32 / Q;
  return lane / G + Q * brev<log2i<Q>()>(k) + Q * Q * brev<log2i<G>()>(lane % G);
}

// Slot of output j in a staging buffer (a permutation of [0, 32 Q)).
template <typename T, int Q>
__device__ __forceinline__ int swz(int j) {
  if constexpr (Q == 32) return j;
  constexpr int qb = log2i<Q>();
  if constexpr (sizeof(T) == 4) return j ^ ((j >> (qb + 1)) & 15);
  else return j ^ ((j >> (qb + 1)) & 7);
}

template <typename T>
__device__ __forceinline__ T line_factor(const HalfPass<T>& a, int g) {
  T f = T(1);
  if (a.fac_a) f *= __ldg(a.fac_a + g % a.Na);
  if (a.fac_b) f *= __ldg(a.fac_b + g / a.Na);
  return f;
}

// Padding of the class-major staging buffers [q][swz(r)] (pitch M' + pad)
// that keeps the reads of consecutive positions x = F r + q and the FFT's
// writes free of bank conflicts (FP32: 16 / F elements).
template <typename T>
__host__ __device__ constexpr int stage_pad(int F) {
  return sizeof(T) == 4 ? (F >= 2 ? 16 / F : 0) : (F >= 2 ? 8 / F : 0);
}

// Shared-memory pitch of a column buffer in the strided passes: at least n,
// offset 4 mod 16 elements (FP32) / 2 mod 8 (FP64) so that the 4-column
// gathers fall in distinct banks.
template <typename T>
__host__ __device__ constexpr int col_pitch(int n) {
  return sizeof(T) == 4 ? ((n + 15) / 16) * 16 + 4 : ((n + 7) / 8) * 8 + 2;
}

// Folded input of class q at cyclic position n: sum over the modes i = i0 +
// c M' (k = i - N/2 = n mod M') of ld(i) W_L^(k q).
template <typename T, typename LD>
__device__ __forceinline__ cplx_t<T> fold_modes(int n, int q, int N, int Mp, int L, const cplx_t<T>* tw, LD ld) {
  cplx_t<T> acc;
  acc.x = acc.y = T(0);
  const int i0 = (n + N / 2) % Mp;
  for (int i = i0; i < N; i += Mp) {
    cplx_t<T> x = ld(i);
    if (q) {
      int e = ((i - N / 2) * q) % L;
      if (e < 0) e += L;
      x = hcmul(x, __ldg(tw + e));
    }
    acc = hcadd(acc, x);
  }
  return acc;
}

// Type 2, first pass (along x, contiguous lines of the compact mode array):
// block = LB lines x F classes, warp (line, class); output lines of L.
template <typename T, int Q, int DIR>
__global__ void __launch_bounds__(256) k_half_t2_rows(HalfPass<T> a) {
  using C = cplx_t<T>;
  constexpr int Mp = 32 * Q;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* st = reinterpret_cast<C*>(smem_raw);  // [LB][F][Mp + pad]
  const int F = a.F, L = F * Mp;
  const int Pq = Mp + stage_pad<T>(F);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int gl = warp / F, q = warp % F;
  const int LB = (blockDim.x >> 5) / F;
  const long long gline = (long long)blockIdx.x * LB + gl;
  const bool live = gline < (long long)a.nlines * a.ntr;
  const int t = live ? (int)(gline / a.nlines) : 0;
  const int g = live ? (int)(gline % a.nlines) : 0;
  const C* in = a.in + (long long)t * a.in_tr + (long long)g * a.in_row;
  const T lf = live ? line_factor(a, g) : T(0);
  C v[Q];
#pragma unroll
  for (int m = 0; m < Q; ++m) {
    if (live) {
      v[m] = fold_modes<T>(lane + 32 * m, q, a.N, Mp, L, a.tw, [&](int i) {
        C x = __ldg(in + i);
        const T f = a.fac ? lf * __ldg(a.fac + i) : lf;
        x.x *= f;
        x.y *= f;
        return x;
      });
    } else {
      v[m].x = v[m].y = T(0);
    }
  }
  C* mine = st + (gl * F + q) * Pq;
  warp_fft<T, Q, DIR>(v, a.tw, lane, mine, F);
#pragma unroll
  for (int k = 0; k < Q; ++k) mine[swz<T, Q>(fft_out_index<Q>(k, lane))] = v[k];
  __syncthreads();
  if (!live) return;
  const C* lst = st + gl * F * Pq;
  C* out = a.out + (long long)t * a.out_tr + (long long)g * a.out_row;
  for (int x = q * 32 + lane; x < L; x += 32 * F) out[x] = lst[(x % F) * Pq + swz<T, Q>(x / F)];
}

// Type 2, later passes (strided lines): 4 adjacent columns of one outer
// index, classes qg Fb .. qg Fb + Fb - 1 (warp (column, class)).  Input: N
// values per column at stride in_row (mode order), gathered into [4][P];
// output: rows y = F r + q at stride out_row, staged in the same buffer.
template <typename T, int Q, int DIR>
__global__ void __launch_bounds__(512) k_half_t2_cols(HalfPass<T> a) {
  using C = cplx_t<T>;
  constexpr int Mp = 32 * Q;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* sm = reinterpret_cast<C*>(smem_raw);
  const int F = a.F, L = F * Mp, Fb = a.Fb;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int w = warp & 3, qq = warp >> 2;
  long long u = blockIdx.x;
  const int qg = (int)(u % (F / Fb));
  u /= (F / Fb);
  const int cg = (int)(u % (a.ncols / 4));
  u /= (a.ncols / 4);
  const int o = (int)(u % a.nouter);
  const int t = (int)(u / a.nouter);
  const int q = qg * Fb + qq;
  const int c0 = cg * 4;
  const int P = a.pitch;
  const C* in = a.in + (long long)t * a.in_tr + (long long)o * a.in_plane + c0;
  for (int idx = threadIdx.x; idx < 4 * a.N; idx += blockDim.x) {
    const int cw = idx & 3, i = idx >> 2;
    if constexpr (sizeof(T) == 4) cp_async8(sm + cw * P + i, in + (long long)i * a.in_row + cw);
    else cp_async16(sm + cw * P + i, in + (long long)i * a.in_row + cw);
  }
  cp_async_wait();
  __syncthreads();
  C v[Q];
  const C* col = sm + w * P;
#pragma unroll
  for (int m = 0; m < Q; ++m)
    v[m] = fold_modes<T>(lane + 32 * m, q, a.N, Mp, L, a.tw, [&](int i) { return col[i]; });
  __syncthreads();  // every warp has its input: the buffer becomes scratch and staging
  const int Pq = Mp + stage_pad<T>(4 * Fb);
  C* mine = sm + (qq * 4 + w) * Pq;
  warp_fft<T, Q, DIR>(v, a.tw, lane, mine, F);
#pragma unroll
  for (int k = 0; k < Q; ++k) mine[swz<T, Q>(fft_out_index<Q>(k, lane))] = v[k];
  __syncthreads();
  C* out = a.out + (long long)t * a.out_tr + (long long)o * a.out_plane + c0;
  for (int idx = threadIdx.x; idx < 4 * Fb * Mp; idx += blockDim.x) {
    const int cw = idx & 3, e = idx >> 2;  // e = r Fb + qi
    const int qi = e % Fb, r = e / Fb;
    out[(long long)(F * r + qg * Fb + qi) * a.out_row + cw] = sm[(qi * 4 + cw) * Pq + swz<T, Q>(r)];
  }
}

// Type 1, strided passes (whole lines of L values): 4 adjacent columns of one
// outer index, all F classes (warp (column, class)); the rows y = F j + q
// are gathered class-major into [F][4][P]; outputs the N mode rows,
// Y[k] = sum_q W_L^(k q) F_q[k mod M'].
template <typename T, int Q, int DIR>
__global__ void __launch_bounds__(1024) k_half_t1_cols(HalfPass<T> a) {
  using C = cplx_t<T>;
  constexpr int Mp = 32 * Q;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* sm = reinterpret_cast<C*>(smem_raw);
  const int F = a.F, L = F * Mp;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int w = warp & 3, q = warp >> 2;
  long long u = blockIdx.x;
  const int cg = (int)(u % (a.ncols / 4));
  u /= (a.ncols / 4);
  const int o = (int)(u % a.nouter);
  const int t = (int)(u / a.nouter);
  const int c0 = cg * 4;
  const int P = a.pitch;
  const C* in = a.in + (long long)t * a.in_tr + (long long)o * a.in_plane + c0;
  for (int idx = threadIdx.x; idx < 4 * L; idx += blockDim.x) {
    const int cw = idx & 3, y = idx >> 2;
    C* dst = sm + ((y % F) * 4 + cw) * P + y / F;
    if constexpr (sizeof(T) == 4) cp_async8(dst, in + (long long)y * a.in_row + cw);
    else cp_async16(dst, in + (long long)y * a.in_row + cw);
  }
  cp_async_wait();
  __syncthreads();
  C v[Q];
  C* col = sm + (q * 4 + w) * P;
#pragma unroll
  for (int m = 0; m < Q; ++m) v[m] = col[lane + 32 * m];
  __syncwarp();  // the buffer is this warp's own: it becomes the scratch
  warp_fft<T, Q, DIR>(v, a.tw, lane, col, F);
#pragma unroll
  for (int k = 0; k < Q; ++k) col[swz<T, Q>(fft_out_index<Q>(k, lane))] = v[k];
  __syncthreads();
  C* out = a.out + (long long)t * a.out_tr + (long long)o * a.out_plane + c0;
  for (int idx = threadIdx.x; idx < 4 * a.N; idx += blockDim.x) {
    const int cw = idx & 3, i = idx >> 2;
    const int k = i - a.N / 2;
    int r = k % Mp;
    if (r < 0) r += Mp;
    const int s = swz<T, Q>(r);
    C y = sm[cw * P + s];
    for (int qi = 1; qi < F; ++qi) {
      int e = (k * qi) % L;
      if (e < 0) e += L;
      y = hcadd(y, hcmul(__ldg(a.tw + e), sm[(qi * 4 + cw) * P + s]));
    }
    out[(long long)i * a.out_row + cw] = y;
  }
}

// Type 1, last pass (along x, contiguous lines of length L): block = LB
// lines x F classes; the line is gathered class-major ([F][M' + pad]), warp
// (line, class) transforms its class; writes the N modes of the line with
// the deconvolution factors.
template <typename T, int Q, int DIR>
__global__ void __launch_bounds__(256) k_half_t1_rows(HalfPass<T> a) {
  using C = cplx_t<T>;
  constexpr int Mp = 32 * Q;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* st = reinterpret_cast<C*>(smem_raw);  // [LB][F][Mp + pad]
  const int F = a.F, L = F * Mp;
  const int Pq = Mp + stage_pad<T>(F);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int gl = warp / F, q = warp % F;
  const int LB = (blockDim.x >> 5) / F;
  const long long gline = (long long)blockIdx.x * LB + gl;
  const bool live = gline < (long long)a.nlines * a.ntr;
  const int t = live ? (int)(gline / a.nlines) : 0;
  const int g = live ? (int)(gline % a.nlines) : 0;
  const C* in = a.in + (long long)t * a.in_tr + (long long)g * a.in_row;
  C* lst = st + gl * F * Pq;
  if (live) {
    for (int x = q * 32 + lane; x < L; x += 32 * F) {
      C* dst = lst + (x % F) * Pq + swz<T, Q>(x / F);
      if constexpr (sizeof(T) == 4) cp_async8(dst, in + x);
      else cp_async16(dst, in + x);
    }
  }
  cp_async_wait();
  __syncthreads();
  C v[Q];
  C* mine = lst + q * Pq;
#pragma unroll
  for (int m = 0; m < Q; ++m) {
    if (live) v[m] = mine[swz<T, Q>(lane + 32 * m)];
    else v[m].x = v[m].y = T(0);
  }
  __syncwarp();
  warp_fft<T, Q, DIR>(v, a.tw, lane, mine, F);
#pragma unroll
  for (int k = 0; k < Q; ++k) mine[swz<T, Q>(fft_out_index<Q>(k, lane))] = v[k];
  __syncthreads();
  if (!live) return;
  C* out = a.out + (long long)t * a.out_tr + (long long)g * a.out_row;
  const T lf = line_factor(a, g);
  for (int i = q * 32 + lane; i < a.N; i += 32 * F) {
    const int k = i - a.N / 2;
    int r = k % Mp;
    if (r < 0) r += Mp;
    const int s = swz<T, Q>(r);
    C y = lst[s];
    for (int qi = 1; qi < F; ++qi) {
      int e = (k * qi) % L;
      if (e < 0) e += L;
      y = hcadd(y, hcmul(__ldg(a.tw + e), lst[qi * Pq + s]));
    }
    T f = lf;
    if (a.fac) f *= __ldg(a.fac + i);
    y.x *= f;
    y.y *= f;
    out[i] = y;
  }
}

template <typename T, int Q, int DIR>
cudaError_t launch_qd(const HalfPass<T>& a, cudaStream_t s) {
  using C = cplx_t<T>;
  constexpr int Mp = 32 * Q;
  const int F = a.F;
  size_t smem = 0;
  int blocks = 0, threads = 0;
  cudaError_t e = cudaSuccess;
  switch (a.kind) {
    case kHalfT2Rows:
    case kHalfT1Rows: {
      threads = 256;  // F <= 8 classes
      const int LB = 8 / F;
      smem = sizeof(C) * (size_t)LB * F * (Mp + stage_pad<T>(F));
      blocks = (int)(((long long)a.nlines * a.ntr + LB - 1) / LB);
      break;
    }
    case kHalfT2Cols:
      threads = 32 * 4 * a.Fb;
      smem = sizeof(C) * std::max((size_t)4 * a.pitch, (size_t)4 * a.Fb * (Mp + stage_pad<T>(4 * a.Fb)));
      blocks = (int)((long long)(a.ncols / 4) * a.nouter * a.ntr * (F / a.Fb));
      break;
    default:
      threads = 32 * 4 * F;
      smem = sizeof(C) * (size_t)4 * F * a.pitch;
      blocks = (int)((long long)(a.ncols / 4) * a.nouter * a.ntr);
      break;
  }
  if (blocks <= 0) return cudaSuccess;
  auto prep = [&](auto kern) {
    return smem > 48 * 1024 ? cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)
                            : cudaSuccess;
  };
  switch (a.kind) {
    case kHalfT2Rows:
      e = prep(k_half_t2_rows<T, Q, DIR>);
      if (e == cudaSuccess) k_half_t2_rows<T, Q, DIR><<<blocks, threads, smem, s>>>(a);
      break;
    case kHalfT2Cols:
      e = prep(k_half_t2_cols<T, Q, DIR>);
      if (e == cudaSuccess) k_half_t2_cols<T, Q, DIR><<<blocks, threads, smem, s>>>(a);
      break;
    case kHalfT1Cols:
      e = prep(k_half_t1_cols<T, Q, DIR>);
      if (e == cudaSuccess) k_half_t1_cols<T, Q, DIR><<<blocks, threads, smem, s>>>(a);
      break;
    default:
      e = prep(k_half_t1_rows<T, Q, DIR>);
      if (e == cudaSuccess) k_half_t1_rows<T, Q, DIR><<<blocks, threads, smem, s>>>(a);
      break;
  }
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

template <typename T, int Q>
cudaError_t launch_q(const HalfPass<T>& a, cudaStream_t s) {
  return a.dir > 0 ? launch_qd<T, Q, 1>(a, s) : launch_qd<T, Q, -1>(a, s);
}

}  // namespace

template <typename T>
cudaError_t launch_half_pass(const HalfPass<T>& a, cudaStream_t s) {
  if (a.F < 1 || a.F > 8 || a.Fb < 1 || a.F % a.Fb != 0) return cudaErrorInvalidValue;
  switch (a.Mp) {
    case 128: return launch_q<T, 4>(a, s);
    case 256: return launch_q<T, 8>(a, s);
    default: return cudaErrorInvalidValue;
  }
}

bool half_fft_size_ok(int nf) { return nf >= 256 && nf <= 2048 && (nf & (nf - 1)) == 0; }

// Per-warp FFT size on an axis of nf points: 256, or 128 for nf = 256 (at
// least two classes either way).
int half_fft_mp(int nf) { return nf >= 512 ? 256 : 128; }

template <typename T>
int half_col_pitch(int n, int M) {
  return col_pitch<T>(n > M ? n : M);
}
template int half_col_pitch<float>(int, int);
template int half_col_pitch<double>(int, int);

template cudaError_t launch_half_pass<float>(const HalfPass<float>&, cudaStream_t);
template cudaError_t launch_half_pass<double>(const HalfPass<double>&, cudaStream_t);

}  // namespace cfg
