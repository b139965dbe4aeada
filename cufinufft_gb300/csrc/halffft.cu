// halffft.cu -- pruned FFT passes for power-of-two fine grids at upsampling
// factor 2, with the amplification (type 2) or deconvolution (type 1) fused.
//
// With nf = 2 M (M a power of two) and at most M modes per axis, every
// transform along an axis is two M-point FFTs instead of one 2M-point FFT:
//   type 2 (modes a_k -> grid, k in [-N/2, N/2)):
//     X[2j + p] = sum_k (a_k W^(k p)) W_M^(k j),   p = 0, 1, W = e^(dir 2 pi i / 2M),
//   so each parity p is an M-point FFT of the modes placed cyclically
//   (mode k at k mod M), the odd one twiddled by W^k first;
//   type 1 (grid x_n -> modes):
//     Y[k] = F_0[k mod M] + W^k F_1[k mod M],  F_p = FFT_M(x[2j + p]),
//   so the two parities' M-point FFTs are combined only at the N mode
//   positions.
// A d-dimensional transform is one such pass per axis: type 2 starts along
// x on the compact mode array (amplification fused), continues along y (and
// z) over the lines that hold data, and writes the grid; type 1 runs along z
// (and y) over the whole grid, then along x writing the compact mode array
// (deconvolution fused).  Intermediate arrays hold only the mode lines
// (half of the grid per axis), so each pass moves about half the bytes of a
// full-grid FFT pass and the zero padding is never read.
//
// The M-point FFT runs in one warp, M = 32 Q: lane l holds x[l + 32 m],
// m < Q, so global loads of a line are coalesced.  Four-step:
//   (1) Q-point FFT over m in registers (radix-2 decimation in frequency),
//   (2) twiddle W_M^(l j1),
//   (3) 32-point FFT over the lanes (radix-2 butterflies by shuffles),
// after which lane l, register k holds X[rev_Q(k) + Q rev_32(l)].  Results
// go through shared memory (XOR-swizzled so both the scattered writes and
// the natural-order reads are free of bank conflicts) to coalesced stores.
// Twiddles come from the plan's per-axis table W^t, t < 2M (extended
// precision on the host).
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

// Shared-memory slot of output j of a warp FFT (a permutation of [0, 32 Q)):
// flips the low bits by the lane part of j, so that both the lanes' writes
// (fixed register, j = r + Q rev_32(l)) and natural-order reads touch
// distinct banks in every phase (16 lanes x 8 bytes FP32, 8 x 16 FP64).
template <typename T, int Q>
__device__ __forceinline__ int swz(int j) {
  constexpr int qb = log2i<Q>();
  if constexpr (sizeof(T) == 4) return j ^ ((j >> (qb + 1)) & 15);
  else return j ^ ((j >> (qb + 2)) & 7);
}

// Warp FFT of M = 32 Q points: on entry v[m] = x[lane + 32 m]; on exit
// v[k] = X[rev_Q(k) + Q rev_32(lane)], X[j] = sum_n x[n] W_M^(n j).  tw[t] =
// W_L^t with L = 2 M, so W_M^t = tw[2t], W_Q^t = tw[64 t], W_32^t = tw[2 Q t].
template <typename T, int Q>
__device__ __forceinline__ void warp_fft(cplx_t<T> (&v)[Q], const cplx_t<T>* __restrict__ tw, int lane) {
  using C = cplx_t<T>;
  constexpr int QB = log2i<Q>();
  // (1) Q-point DIF over the registers
#pragma unroll
  for (int h = Q / 2; h >= 1; h >>= 1) {
#pragma unroll
    for (int b = 0; b < Q; b += 2 * h) {
#pragma unroll
      for (int i = 0; i < h; ++i) {
        const C a = v[b + i], c = v[b + i + h];
        v[b + i] = hcadd(a, c);
        const C d = hcsub(a, c);
        v[b + i + h] = i == 0 ? d : hcmul(d, __ldg(tw + 64 * i * (Q / (2 * h))));
      }
    }
  }
  // (2) twiddles W_M^(lane rev_Q(k))
#pragma unroll
  for (int k = 1; k < Q; ++k) v[k] = hcmul(v[k], __ldg(tw + 2 * lane * brev<QB>(k)));
  // (3) 32-point DIF over the lanes
#pragma unroll
  for (int h = 16; h >= 1; h >>= 1) {
    const bool up = (lane & h) != 0;
    const C w = __ldg(tw + 2 * Q * ((lane & (h - 1)) * (16 / h)));
#pragma unroll
    for (int k = 0; k < Q; ++k) {
      C o;
      o.x = __shfl_xor_sync(0xffffffffu, v[k].x, h);
      o.y = __shfl_xor_sync(0xffffffffu, v[k].y, h);
      v[k] = up ? hcmul(hcsub(o, v[k]), w) : hcadd(v[k], o);
    }
  }
}

// Output index held by lane, register k after warp_fft.
template <int Q>
__device__ __forceinline__ int fft_out_index(int k, int lane) {
  return brev<log2i<Q>()>(k) + Q * brev<5>(lane);
}

// Mode index i in [0, N) of cyclic position n in [0, M) (mode k = i - N/2 at
// k mod M), or -1 for the positions between the modes.
__device__ __forceinline__ int cyc_mode(int n, int N, int M) {
  const int pos = N - N / 2;  // modes k = 0 .. pos - 1 at n = k
  if (n < pos) return n + N / 2;
  if (n >= M - N / 2) return n - M + N / 2;
  return -1;
}

// W^k for a signed mode k from the table of length L.
template <typename C>
__device__ __forceinline__ C tw_signed(const C* tw, int k, int L) {
  return __ldg(tw + (k < 0 ? k + L : k));
}

template <typename T>
__device__ __forceinline__ T line_factor(const HalfPass<T>& a, int g) {
  T f = T(1);
  if (a.fac_a) f *= __ldg(a.fac_a + g % a.Na);
  if (a.fac_b) f *= __ldg(a.fac_b + g / a.Na);
  return f;
}

constexpr int kRowLines = 4;  // lines per block of the contiguous passes (2 warps each)

// Type 2, first pass (along x, contiguous lines of the compact mode array):
// line g of transform t, parity p = warp & 1.  Output line of length 2M.
template <typename T, int Q>
__global__ void __launch_bounds__(256) k_half_t2_rows(HalfPass<T> a) {
  using C = cplx_t<T>;
  constexpr int M = 32 * Q;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* st = reinterpret_cast<C*>(smem_raw);  // [kRowLines][2][M]
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int gl = warp >> 1, p = warp & 1;
  const long long gline = (long long)blockIdx.x * kRowLines + gl;  // over transforms x lines
  const bool live = gline < (long long)a.nlines * a.ntr;
  const int t = live ? (int)(gline / a.nlines) : 0;
  const int g = live ? (int)(gline % a.nlines) : 0;
  C v[Q];
  if (live) {
    const C* in = a.in + (long long)t * a.in_tr + (long long)g * a.in_row;
    const T lf = line_factor(a, g);
#pragma unroll
    for (int m = 0; m < Q; ++m) {
      const int i = cyc_mode(lane + 32 * m, a.N, M);
      C x;
      x.x = x.y = T(0);
      if (i >= 0) {
        x = __ldg(in + i);
        T f = lf;
        if (a.fac) f *= __ldg(a.fac + i);
        x.x *= f;
        x.y *= f;
        if (p) x = hcmul(x, tw_signed(a.tw, i - a.N / 2, 2 * M));
      }
      v[m] = x;
    }
  } else {
#pragma unroll
    for (int m = 0; m < Q; ++m) v[m].x = v[m].y = T(0);
  }
  warp_fft<T, Q>(v, a.tw, lane);
  C* mine = st + (gl * 2 + p) * M;
#pragma unroll
  for (int k = 0; k < Q; ++k) mine[swz<T, Q>(fft_out_index<Q>(k, lane))] = v[k];
  __syncthreads();
  if (!live) return;
  // both parities of line gl: grid positions 2j, 2j+1 as one 2-element store
  const C* e = st + (gl * 2) * M;
  const C* o = e + M;
  C* out = a.out + (long long)t * a.out_tr + (long long)g * a.out_row;
  for (int j = (p << 5) | lane; j < M; j += 64) {
    const int s = swz<T, Q>(j);
    if constexpr (sizeof(T) == 4) {
      // rows start 16-byte aligned (even length): one 16-byte store
      const C ev = e[s], od = o[s];
      *reinterpret_cast<float4*>(out + 2 * j) = make_float4(ev.x, ev.y, od.x, od.y);
    } else {
      out[2 * j] = e[s];
      out[2 * j + 1] = o[s];
    }
  }
}

// Type 2, later passes (strided lines): 4 adjacent columns of one outer
// index, one parity; warp w takes column c0 + w.  Input: N values per column
// at stride in_row (mode order); output: rows y = 2j + p at stride out_row.
template <typename T, int Q>
__global__ void __launch_bounds__(128) k_half_t2_cols(HalfPass<T> a) {
  using C = cplx_t<T>;
  constexpr int M = 32 * Q;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* sm = reinterpret_cast<C*>(smem_raw);  // [4][P] columns, reused as [4][M] output
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  long long u = blockIdx.x;
  const int p = (int)(u & 1);
  u >>= 1;
  const int cg = (int)(u % (a.ncols / 4));
  u /= (a.ncols / 4);
  const int o = (int)(u % a.nouter);
  const int t = (int)(u / a.nouter);
  const int c0 = cg * 4;
  const int P = a.pitch;
  const C* in = a.in + (long long)t * a.in_tr + (long long)o * a.in_plane + c0;
  // gather the 4 x N block (columns transposed into rows of the buffer)
  for (int idx = threadIdx.x; idx < 4 * a.N; idx += 128) {
    const int cw = idx & 3, i = idx >> 2;
    if constexpr (sizeof(T) == 4) cp_async8(sm + cw * P + i, in + (long long)i * a.in_row + cw);
    else cp_async16(sm + cw * P + i, in + (long long)i * a.in_row + cw);
  }
  cp_async_wait();
  __syncthreads();
  C v[Q];
  const C* col = sm + w * P;
#pragma unroll
  for (int m = 0; m < Q; ++m) {
    const int i = cyc_mode(lane + 32 * m, a.N, M);
    C x;
    x.x = x.y = T(0);
    if (i >= 0) {
      x = col[i];
      if (p) x = hcmul(x, tw_signed(a.tw, i - a.N / 2, 2 * M));
    }
    v[m] = x;
  }
  warp_fft<T, Q>(v, a.tw, lane);
  __syncthreads();  // every warp has read its column: reuse the buffer
  C* st = sm + w * M;
#pragma unroll
  for (int k = 0; k < Q; ++k) st[swz<T, Q>(fft_out_index<Q>(k, lane))] = v[k];
  __syncthreads();
  C* out = a.out + (long long)t * a.out_tr + (long long)o * a.out_plane + c0;
  for (int idx = threadIdx.x; idx < 4 * M; idx += 128) {
    const int cw = idx & 3, j = idx >> 2;
    out[(long long)(2 * j + p) * a.out_row + cw] = sm[cw * M + swz<T, Q>(j)];
  }
}

// Type 1, strided passes (whole lines of 2M values): 4 adjacent columns of
// one outer index; warp (w, p) = (warp & 3, warp >> 2) transforms the parity
// p rows of column c0 + w; outputs the N mode rows, F_0 + W^k F_1.
template <typename T, int Q>
__global__ void __launch_bounds__(256) k_half_t1_cols(HalfPass<T> a) {
  using C = cplx_t<T>;
  constexpr int M = 32 * Q;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* sm = reinterpret_cast<C*>(smem_raw);  // [2][4][P]: parity, column, j
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int w = warp & 3, p = warp >> 2;
  long long u = blockIdx.x;
  const int cg = (int)(u % (a.ncols / 4));
  u /= (a.ncols / 4);
  const int o = (int)(u % a.nouter);
  const int t = (int)(u / a.nouter);
  const int c0 = cg * 4;
  const int P = a.pitch;
  const C* in = a.in + (long long)t * a.in_tr + (long long)o * a.in_plane + c0;
  for (int idx = threadIdx.x; idx < 4 * 2 * M; idx += 256) {
    const int cw = idx & 3, y = idx >> 2;
    C* dst = sm + ((y & 1) * 4 + cw) * P + (y >> 1);
    if constexpr (sizeof(T) == 4) cp_async8(dst, in + (long long)y * a.in_row + cw);
    else cp_async16(dst, in + (long long)y * a.in_row + cw);
  }
  cp_async_wait();
  __syncthreads();
  C v[Q];
  C* col = sm + (p * 4 + w) * P;
#pragma unroll
  for (int m = 0; m < Q; ++m) v[m] = col[lane + 32 * m];
  warp_fft<T, Q>(v, a.tw, lane);
  __syncwarp();  // the column is this warp's own: overwrite it in place
#pragma unroll
  for (int k = 0; k < Q; ++k) col[swz<T, Q>(fft_out_index<Q>(k, lane))] = v[k];
  __syncthreads();
  C* out = a.out + (long long)t * a.out_tr + (long long)o * a.out_plane + c0;
  for (int idx = threadIdx.x; idx < 4 * a.N; idx += 256) {
    const int cw = idx & 3, i = idx >> 2;
    const int k = i - a.N / 2;
    const int s = swz<T, Q>(k < 0 ? k + M : k);
    const C f0 = sm[cw * P + s], f1 = sm[(4 + cw) * P + s];
    out[(long long)i * a.out_row + cw] = hcadd(f0, hcmul(tw_signed(a.tw, k, 2 * M), f1));
  }
}

// Type 1, last pass (along x, contiguous lines of length 2M): line g of
// transform t, parity p = warp & 1 reads x[2j + p]; writes the N modes of the
// line with the deconvolution factors.
template <typename T, int Q>
__global__ void __launch_bounds__(256) k_half_t1_rows(HalfPass<T> a) {
  using C = cplx_t<T>;
  constexpr int M = 32 * Q;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* st = reinterpret_cast<C*>(smem_raw);  // [kRowLines][2][M]
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int gl = warp >> 1, p = warp & 1;
  const long long gline = (long long)blockIdx.x * kRowLines + gl;
  const bool live = gline < (long long)a.nlines * a.ntr;
  const int t = live ? (int)(gline / a.nlines) : 0;
  const int g = live ? (int)(gline % a.nlines) : 0;
  C v[Q];
  const C* in = a.in + (long long)t * a.in_tr + (long long)g * a.in_row;
#pragma unroll
  for (int m = 0; m < Q; ++m) {
    if (live) v[m] = __ldg(in + 2 * (lane + 32 * m) + p);
    else v[m].x = v[m].y = T(0);
  }
  warp_fft<T, Q>(v, a.tw, lane);
  C* mine = st + (gl * 2 + p) * M;
#pragma unroll
  for (int k = 0; k < Q; ++k) mine[swz<T, Q>(fft_out_index<Q>(k, lane))] = v[k];
  __syncthreads();
  if (!live) return;
  const C* f0 = st + (gl * 2) * M;
  const C* f1 = f0 + M;
  C* out = a.out + (long long)t * a.out_tr + (long long)g * a.out_row;
  const T lf = line_factor(a, g);
  for (int i = (p << 5) | lane; i < a.N; i += 64) {
    const int k = i - a.N / 2;
    const int s = swz<T, Q>(k < 0 ? k + M : k);
    C y = hcadd(f0[s], hcmul(tw_signed(a.tw, k, 2 * M), f1[s]));
    T f = lf;
    if (a.fac) f *= __ldg(a.fac + i);
    y.x *= f;
    y.y *= f;
    out[i] = y;
  }
}

template <typename T, int Q>
cudaError_t launch_q(const HalfPass<T>& a, cudaStream_t s) {
  using C = cplx_t<T>;
  constexpr int M = 32 * Q;
  size_t smem = 0;
  int blocks = 0, threads = 0;
  cudaError_t e = cudaSuccess;
  switch (a.kind) {
    case kHalfT2Rows:
    case kHalfT1Rows:
      smem = sizeof(C) * kRowLines * 2 * M;
      blocks = (int)(((long long)a.nlines * a.ntr + kRowLines - 1) / kRowLines);
      threads = 256;
      break;
    case kHalfT2Cols:
      smem = sizeof(C) * 4 * (size_t)std::max(a.pitch, M);
      blocks = (int)((long long)(a.ncols / 4) * a.nouter * a.ntr * 2);
      threads = 128;
      break;
    default:
      smem = sizeof(C) * 8 * (size_t)a.pitch;
      blocks = (int)((long long)(a.ncols / 4) * a.nouter * a.ntr);
      threads = 256;
      break;
  }
  if (blocks <= 0) return cudaSuccess;
  auto prep = [&](auto kern) {
    return smem > 48 * 1024 ? cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)
                            : cudaSuccess;
  };
  switch (a.kind) {
    case kHalfT2Rows:
      e = prep(k_half_t2_rows<T, Q>);
      if (e == cudaSuccess) k_half_t2_rows<T, Q><<<blocks, threads, smem, s>>>(a);
      break;
    case kHalfT2Cols:
      e = prep(k_half_t2_cols<T, Q>);
      if (e == cudaSuccess) k_half_t2_cols<T, Q><<<blocks, threads, smem, s>>>(a);
      break;
    case kHalfT1Cols:
      e = prep(k_half_t1_cols<T, Q>);
      if (e == cudaSuccess) k_half_t1_cols<T, Q><<<blocks, threads, smem, s>>>(a);
      break;
    default:
      e = prep(k_half_t1_rows<T, Q>);
      if (e == cudaSuccess) k_half_t1_rows<T, Q><<<blocks, threads, smem, s>>>(a);
      break;
  }
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

}  // namespace

template <typename T>
cudaError_t launch_half_pass(const HalfPass<T>& a, cudaStream_t s) {
  switch (a.M) {
    case 64: return launch_q<T, 2>(a, s);
    case 128: return launch_q<T, 4>(a, s);
    case 256: return launch_q<T, 8>(a, s);
    case 512: return launch_q<T, 16>(a, s);
    case 1024: return launch_q<T, 32>(a, s);
    default: return cudaErrorInvalidValue;
  }
}

bool half_fft_size_ok(int nf) { return nf >= 128 && nf <= 2048 && (nf & (nf - 1)) == 0; }

template cudaError_t launch_half_pass<float>(const HalfPass<float>&, cudaStream_t);
template cudaError_t launch_half_pass<double>(const HalfPass<double>&, cudaStream_t);

}  // namespace cfg
