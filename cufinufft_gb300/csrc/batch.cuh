// batch.cuh -- many plans run as one captured CUDA graph with multi-plan kernels.
//
// A batch groups plans of one type, dimension and precision whose points are
// already set.  Each batch execute runs, for all member plans together:
//   type 1: clear the grids, ONE multi-plan spreading kernel, one cuFFT call
//           per plan (its whole ntransf in one batched FFT), ONE multi-plan
//           deconvolution kernel;
//   type 2: ONE multi-plan amplify kernel, cuFFT per plan, ONE multi-plan
//           interpolation kernel.
// The whole sequence is captured once into a CUDA graph and replayed; the
// per-plan data pointers travel in a small descriptor table that the graph
// copies from pinned host memory at the start of every replay.  The
// multi-plan kernels walk a global list of work items (a warp of points, or
// a grid row) and find their plan by binary search over the per-plan
// starts, so small plans share the GPU instead of each leaving most SMs idle.
// The reference runs plans one after another with several launches per
// transform (src/2d/cufinufft2d.cu:15-165).
#pragma once

#include <algorithm>
#include <vector>

#include "plan.h"
#include "spreadinterp.cuh"

namespace cfg {

template <typename T> struct BatchDesc {
  int M, ntr;
  int nf[3];
  int N[3];
  long long Nf, Nm;
  const int* idx;
  const int* i0[3];
  const T* d[3];
  T beta, c;
  T e_beta, bl2e;  // e^beta and beta log2(e) (FP32 kernel evaluation)
  cplx_t<T>* fw;
  const cplx_t<T>* c_in;    // type 1 strengths
  cplx_t<T>* c_out;         // type 2 values
  cplx_t<T>* fk;            // type 1 output / type 2 input
  const T* fac[3];
  long long task0;          // first point-chunk task of this plan (method 1 plans)
  long long row0;           // first grid-row task of this plan
  long long blk0;           // first subproblem-block task of this plan (method 2 plans)
  BinTables bins;           // bin tables (method 2 plans)
  int method;
  const unsigned char* sub_dense;  // cell-run layout: subproblems for k_batch_spread_run
};

// Largest plan index p whose first task of the given kind is <= task
// (kind 0: point chunks, 1: grid rows, 2: subproblem blocks).
template <typename T>
__device__ __forceinline__ int find_plan(const BatchDesc<T>* D, int nplans, long long task,
                                         int kind) {
  int lo = 0, hi = nplans;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    const long long s = kind == 1 ? D[mid].row0 : (kind == 0 ? D[mid].task0 : D[mid].blk0);
    if (s <= task) lo = mid;
    else hi = mid;
  }
  return lo;
}

template <typename T, int NS>
__device__ __forceinline__ T batch_tap(T d, int j, const BatchDesc<T>& P) {
  const T x = d - T(0.5) * T(NS) + T(j);
  const T z = P.c * x * x;
  if constexpr (sizeof(T) == 4) return es_value_fast(z, P.e_beta, P.bl2e);
  else return es_value(z, P.beta);
}

// Spreading, warp-cooperative, NU-point driven (as k_spread_gm_wc), over the
// point chunks of every plan.
template <typename T, int DIM, int NS>
__global__ void __launch_bounds__(kSpreadThreads)
k_batch_spread(const BatchDesc<T>* D, int nplans, long long task_begin, long long task_end) {
  using C = cplx_t<T>;
  constexpr int L = spread_lanes<NS>();
  constexpr int PPW = 32 / L;
  constexpr int NY = DIM > 1 ? NS : 1;
  constexpr int NZ = DIM > 2 ? NS : 1;
  const int lane = threadIdx.x & 31, g = lane / L, j = lane % L;
  const bool tap = j < NS;
  const int jj = tap ? j : 0;
  const long long wid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long task = task_begin + wid; task < task_end; task += nw) {
    const BatchDesc<T>& P = D[find_plan(D, nplans, task, 0)];
    const long long pl = (task - P.task0) * PPW + g;
    const bool valid = g < PPW && pl < P.M;
    const int p = valid ? (int)pl : P.M - 1;
    const int xj = wrap_idx(P.i0[0][p] + jj, P.nf[0]);
    const T kx = batch_tap<T, NS>(P.d[0][p], jj, P);
    T ky = T(1), kz = T(1);
    int i2 = 0, i3 = 0;
    if (DIM > 1) { i2 = P.i0[1][p]; ky = batch_tap<T, NS>(P.d[1][p], jj, P); }
    if (DIM > 2) { i3 = P.i0[2][p]; kz = batch_tap<T, NS>(P.d[2][p], jj, P); }
    const int src = P.idx[p];
    for (int t = 0; t < P.ntr; ++t) {
      const C v = P.c_in[(size_t)t * P.M + src];
      const T vr = v.x * kx, vi = v.y * kx;
      C* gt = P.fw + (size_t)t * P.Nf + xj;
#pragma unroll 1
      for (int dz = 0; dz < NZ; ++dz) {
        const T kzv = DIM > 2 ? __shfl_sync(0xffffffffu, kz, g * L + dz) : T(1);
        const int iz = DIM > 2 ? wrap_idx(i3 + dz, P.nf[2]) : 0;
#pragma unroll
        for (int dy = 0; dy < NY; ++dy) {
          const T kyv = DIM > 1 ? __shfl_sync(0xffffffffu, ky, g * L + dy) : T(1);
          const int iy = DIM > 1 ? wrap_idx(i2 + dy, P.nf[1]) : 0;
          const T w = kyv * kzv;
          if (tap && valid) red_add(gt + ((size_t)iz * P.nf[1] + iy) * P.nf[0], vr * w, vi * w);
        }
      }
    }
  }
}

// Interpolation, warp-cooperative (as k_interp_gm_wc), over every plan.
template <typename T, int DIM, int NS>
__global__ void __launch_bounds__(kSpreadThreads)
k_batch_interp(const BatchDesc<T>* D, int nplans, long long task_begin, long long task_end) {
  using C = cplx_t<T>;
  constexpr int L = lanes_per_point<NS>();
  constexpr int PPW = 32 / L;
  constexpr int NY = DIM > 1 ? NS : 1;
  constexpr int NZ = DIM > 2 ? NS : 1;
  const int lane = threadIdx.x & 31, g = lane / L, j = lane % L;
  const bool tap = j < NS;
  const int jj = tap ? j : 0;
  const long long wid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long task = task_begin + wid; task < task_end; task += nw) {
    const BatchDesc<T>& P = D[find_plan(D, nplans, task, 0)];
    const long long pl = (task - P.task0) * PPW + g;
    const bool valid = pl < P.M;
    const int p = valid ? (int)pl : P.M - 1;
    const int xj = wrap_idx(P.i0[0][p] + jj, P.nf[0]);
    const T kx = batch_tap<T, NS>(P.d[0][p], jj, P);
    T ky = T(1), kz = T(1);
    int i2 = 0, i3 = 0;
    if (DIM > 1) { i2 = P.i0[1][p]; ky = batch_tap<T, NS>(P.d[1][p], jj, P); }
    if (DIM > 2) { i3 = P.i0[2][p]; kz = batch_tap<T, NS>(P.d[2][p], jj, P); }
    const int dst = P.idx[p];
    for (int t = 0; t < P.ntr; ++t) {
      const C* gt = P.fw + (size_t)t * P.Nf + xj;
      T ar = T(0), ai = T(0);
#pragma unroll 1
      for (int dz = 0; dz < NZ; ++dz) {
        const T kzv = DIM > 2 ? __shfl_sync(0xffffffffu, kz, g * L + dz) : T(1);
        const int iz = DIM > 2 ? wrap_idx(i3 + dz, P.nf[2]) : 0;
#pragma unroll
        for (int dy = 0; dy < NY; ++dy) {
          const T kyv = DIM > 1 ? __shfl_sync(0xffffffffu, ky, g * L + dy) : T(1);
          const int iy = DIM > 1 ? wrap_idx(i2 + dy, P.nf[1]) : 0;
          if (tap) {
            const C v = __ldg(gt + ((size_t)iz * P.nf[1] + iy) * P.nf[0]);
            const T w = kyv * kzv;
            ar = fma_rn(v.x, w, ar);
            ai = fma_rn(v.y, w, ai);
          }
        }
      }
      ar *= kx;
      ai *= kx;
#pragma unroll
      for (int off = L / 2; off > 0; off >>= 1) {
        ar += __shfl_xor_sync(0xffffffffu, ar, off);
        ai += __shfl_xor_sync(0xffffffffu, ai, off);
      }
      if (j == 0 && valid) {
        C o;
        o.x = ar;
        o.y = ai;
        P.c_out[(size_t)t * P.M + dst] = o;
      }
    }
  }
}

// Deconvolution over the mode rows of every plan and transform (as
// k_deconvolve): row task r of plan P is (t, i2, i3).
template <typename T>
__global__ void __launch_bounds__(256)
k_batch_deconvolve(const BatchDesc<T>* D, int nplans, long long row_begin, long long row_end, int dim) {
  using C = cplx_t<T>;
  for (long long r = row_begin + blockIdx.x; r < row_end; r += gridDim.x) {
    const BatchDesc<T>& P = D[find_plan(D, nplans, r, 1)];
    const long long rr0 = r - P.row0;
    const long long per = (long long)P.N[1] * P.N[2];
    const int t = (int)(rr0 / per);
    const int rr = (int)(rr0 - (long long)t * per);
    const int i2 = rr % P.N[1], i3 = rr / P.N[1];
    const int k2 = i2 - P.N[1] / 2, k3 = i3 - P.N[2] / 2;
    const int w2 = k2 >= 0 ? k2 : P.nf[1] + k2;
    const int w3 = k3 >= 0 ? k3 : P.nf[2] + k3;
    T f23 = T(1);
    if (dim > 1) f23 = P.fac[1][i2];
    if (dim > 2) f23 *= P.fac[2][i3];
    const C* src = P.fw + (size_t)t * P.Nf + ((size_t)w3 * P.nf[1] + w2) * P.nf[0];
    C* dst = P.fk + (size_t)t * P.Nm + ((size_t)i3 * P.N[1] + i2) * P.N[0];
    for (int i1 = threadIdx.x; i1 < P.N[0]; i1 += blockDim.x) {
      const int k1 = i1 - P.N[0] / 2;
      const int w1 = k1 >= 0 ? k1 : P.nf[0] + k1;
      const T f = P.fac[0][i1] * f23;
      const C v = src[w1];
      C o;
      o.x = v.x * f;
      o.y = v.y * f;
      dst[i1] = o;
    }
  }
}

// Amplification over the fine-grid rows of every plan and transform (as
// k_amplify), writing every cell.
template <typename T>
__global__ void __launch_bounds__(256)
k_batch_amplify(const BatchDesc<T>* D, int nplans, long long row_begin, long long row_end, int dim) {
  using C = cplx_t<T>;
  for (long long r = row_begin + blockIdx.x; r < row_end; r += gridDim.x) {
    const BatchDesc<T>& P = D[find_plan(D, nplans, r, 1)];
    const long long rr0 = r - P.row0;
    const long long per = (long long)P.nf[1] * P.nf[2];
    const int t = (int)(rr0 / per);
    const int rr = (int)(rr0 - (long long)t * per);
    const int w2 = rr % P.nf[1], w3 = rr / P.nf[1];
    int i2 = 0, i3 = 0;
    bool live = true;
    if (dim > 1) {
      const int k2 = w2 <= (P.N[1] - 1) / 2 ? w2 : (w2 >= P.nf[1] - P.N[1] / 2 ? w2 - P.nf[1] : P.nf[1]);
      live = live && k2 != P.nf[1];
      i2 = k2 + P.N[1] / 2;
    }
    if (dim > 2) {
      const int k3 = w3 <= (P.N[2] - 1) / 2 ? w3 : (w3 >= P.nf[2] - P.N[2] / 2 ? w3 - P.nf[2] : P.nf[2]);
      live = live && k3 != P.nf[2];
      i3 = k3 + P.N[2] / 2;
    }
    C* dst = P.fw + (size_t)t * P.Nf + ((size_t)w3 * P.nf[1] + w2) * P.nf[0];
    T f23 = T(1);
    if (live && dim > 1) f23 = P.fac[1][i2];
    if (live && dim > 2) f23 *= P.fac[2][i3];
    const C* src = P.fk + (size_t)t * P.Nm + ((size_t)i3 * P.N[1] + i2) * P.N[0];
    for (int w1 = threadIdx.x; w1 < P.nf[0]; w1 += blockDim.x) {
      C o;
      o.x = T(0);
      o.y = T(0);
      if (live) {
        const int k1 = w1 <= (P.N[0] - 1) / 2 ? w1 : (w1 >= P.nf[0] - P.N[0] / 2 ? w1 - P.nf[0] : P.nf[0]);
        if (k1 != P.nf[0]) {
          const int i1 = k1 + P.N[0] / 2;
          const T f = P.fac[0][i1] * f23;
          const C v = src[i1];
          o.x = v.x * f;
          o.y = v.y * f;
        }
      }
      dst[w1] = o;
    }
  }
}

// Shared-memory subproblem spreading (as k_spread_sm_wc) over the subproblems
// of every method-2 plan; one block per (subproblem, transform).
template <typename T, int DIM, int NS>
__global__ void __launch_bounds__(kSpreadThreads)
k_batch_spread_sm(const BatchDesc<T>* D, int nplans, long long blk_begin, long long blk_end) {
  using C = cplx_t<T>;
  constexpr int L = spread_lanes<NS>();
  constexpr int PPW = 32 / L;
  constexpr int NY = DIM > 1 ? NS : 1;
  constexpr int NZ = DIM > 2 ? NS : 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  for (long long task = blk_begin + blockIdx.x; task < blk_end; task += gridDim.x) {
    const BatchDesc<T>& P = D[find_plan(D, nplans, task, 2)];
    const long long local = task - P.blk0;
    const int t = (int)(local / P.bins.nsub);
    const int sub = (int)(local - (long long)t * P.bins.nsub);
    if (P.sub_dense && P.sub_dense[sub]) continue;  // cell-run layout: k_batch_spread_run
    const SubTile st = sub_tile_block<DIM, NS, true>(P.bins, sub);
    T* re = reinterpret_cast<T*>(smem_raw);  // real plane, then imaginary plane
    T* im = re + st.ntile;
    __syncthreads();  // the previous task's flush is done with the tile
    for (int i = threadIdx.x; i < 2 * st.ntile; i += blockDim.x) re[i] = T(0);
    __syncthreads();
    const int lane = threadIdx.x & 31, g = lane / L, j = lane % L;
    const bool tap = j < NS;
    const int jj = tap ? j : 0;
    const int warp = threadIdx.x >> 5, nwb = blockDim.x >> 5;
    const C* cin = P.c_in + (size_t)t * P.M;
    for (int base = warp * PPW; base < st.np; base += nwb * PPW) {
      const int pl = base + g;
      const bool valid = g < PPW && pl < st.np;
      const int p = st.p0 + (valid ? pl : st.np - 1);
      const int lx = P.i0[0][p] - st.ox;
      const T kx = batch_tap<T, NS>(P.d[0][p], jj, P);
      T ky = T(1), kz = T(1);
      int ly = 0, lz = 0;
      if (DIM > 1) { ly = P.i0[1][p] - st.oy; ky = batch_tap<T, NS>(P.d[1][p], jj, P); }
      if (DIM > 2) { lz = P.i0[2][p] - st.oz; kz = batch_tap<T, NS>(P.d[2][p], jj, P); }
      const C v = cin[P.idx[p]];
      const T vr = v.x * kx, vi = v.y * kx;
      const int off0 = (lz * st.TY + ly) * st.TX + lx + jj;
#pragma unroll 1
      for (int dz = 0; dz < NZ; ++dz) {
        const T kzv = DIM > 2 ? __shfl_sync(0xffffffffu, kz, g * L + dz) : T(1);
#pragma unroll
        for (int dy = 0; dy < NY; ++dy) {
          const T kyv = DIM > 1 ? __shfl_sync(0xffffffffu, ky, g * L + dy) : T(1);
          const T w = kyv * kzv;
          if (tap && valid) {
            const int off = off0 + (dz * st.TY + dy) * st.TX;
            atomicAdd(re + off, vr * w);
            atomicAdd(im + off, vi * w);
          }
        }
      }
    }
    __syncthreads();
    GridGeom gg;
    gg.nf[0] = P.nf[0];
    gg.nf[1] = P.nf[1];
    gg.nf[2] = P.nf[2];
    gg.Nf = P.Nf;
    plane_flush<T>(re, im, P.fw + (size_t)t * P.Nf, st, gg);
  }
}

// Cell-run spreading (as k_spread_sm_run) over the dense subproblems of the
// plans in the cell-run layout; their other subproblems go through
// k_batch_spread_sm.
template <typename T, int DIM, int NS>
__global__ void __launch_bounds__(kSpreadThreads)
k_batch_spread_run(const BatchDesc<T>* D, int nplans, long long blk_begin, long long blk_end) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  for (long long task = blk_begin + blockIdx.x; task < blk_end; task += gridDim.x) {
    const BatchDesc<T>& P = D[find_plan(D, nplans, task, 2)];
    const long long local = task - P.blk0;
    const int t = (int)(local / P.bins.nsub);
    const int sub = (int)(local - (long long)t * P.bins.nsub);
    if (!(P.sub_dense && P.sub_dense[sub])) continue;
    const SubTile st = sub_tile_block<DIM, NS, true>(P.bins, sub);
    T* re = reinterpret_cast<T*>(smem_raw);
    T* im = re + st.ntile;
    __syncthreads();  // the previous task's flush is done with the tile
    for (int i = threadIdx.x; i < 2 * st.ntile; i += blockDim.x) re[i] = T(0);
    __syncthreads();
    SortedPts<T> pts;
    pts.idx = P.idx;
    for (int k = 0; k < 3; ++k) {
      pts.i0[k] = P.i0[k];
      pts.d[k] = P.d[k];
    }
    pts.M = P.M;
    run_subproblem<T, DIM, NS>(
        st, re, im, pts, P.c_in + (size_t)t * P.M,
        [&](T dv, T* out) {
#pragma unroll
          for (int j = 0; j < NS; ++j) out[j] = batch_tap<T, NS>(dv, j, P);
        },
        [&](T dv, int j) { return batch_tap<T, NS>(dv, j, P); });
    __syncthreads();
    GridGeom gg;
    gg.nf[0] = P.nf[0];
    gg.nf[1] = P.nf[1];
    gg.nf[2] = P.nf[2];
    gg.Nf = P.Nf;
    plane_flush<T>(re, im, P.fw + (size_t)t * P.Nf, st, gg);
  }
}

// Shared-memory subproblem interpolation (as k_interp_sm) over every method-2
// plan.
template <typename T, int DIM, int NS>
__global__ void __launch_bounds__(kSpreadThreads)
k_batch_interp_sm(const BatchDesc<T>* D, int nplans, long long blk_begin, long long blk_end) {
  using C = cplx_t<T>;
  constexpr int NY = DIM > 1 ? NS : 1;
  constexpr int NZ = DIM > 2 ? NS : 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* tile = reinterpret_cast<C*>(smem_raw);
  for (long long task = blk_begin + blockIdx.x; task < blk_end; task += gridDim.x) {
    const BatchDesc<T>& P = D[find_plan(D, nplans, task, 2)];
    const long long local = task - P.blk0;
    const int t = (int)(local / P.bins.nsub);
    const int sub = (int)(local - (long long)t * P.bins.nsub);
    const SubTile st = sub_tile_block<DIM, NS, true>(P.bins, sub);
    GridGeom gg;
    gg.nf[0] = P.nf[0];
    gg.nf[1] = P.nf[1];
    gg.nf[2] = P.nf[2];
    gg.Nf = P.Nf;
    __syncthreads();  // the previous task is done reading the tile
    tile_load<T>(tile, P.fw + (size_t)t * P.Nf, st, gg);
    __syncthreads();
    for (int p = st.p0 + threadIdx.x; p < st.p0 + st.np; p += blockDim.x) {
      T k1[NS], k2[NS];
      const int lx = P.i0[0][p] - st.ox;
#pragma unroll
      for (int j = 0; j < NS; ++j) k1[j] = batch_tap<T, NS>(P.d[0][p], j, P);
      int ly = 0, lz = 0;
      if (DIM > 1) {
        ly = P.i0[1][p] - st.oy;
#pragma unroll
        for (int j = 0; j < NS; ++j) k2[j] = batch_tap<T, NS>(P.d[1][p], j, P);
      }
      T d3 = T(0);
      if (DIM > 2) { lz = P.i0[2][p] - st.oz; d3 = P.d[2][p]; }
      T ar = T(0), ai = T(0);
#pragma unroll 1
      for (int dz = 0; dz < NZ; ++dz) {
        const T kz = DIM > 2 ? batch_tap<T, NS>(d3, dz, P) : T(1);
        const C* plane = tile + ((lz + dz) * st.TY + ly) * st.TX + lx;
#pragma unroll
        for (int dy = 0; dy < NY; ++dy) {
          const C* row = plane + dy * st.TX;
          T rr = T(0), ri = T(0);
#pragma unroll
          for (int dx = 0; dx < NS; ++dx) {
            const C g = row[dx];
            rr = fma_rn(g.x, k1[dx], rr);
            ri = fma_rn(g.y, k1[dx], ri);
          }
          T kyz = T(1);
          if (DIM > 1) kyz = k2[dy];
          if (DIM > 2) kyz *= kz;
          ar = fma_rn(rr, kyz, ar);
          ai = fma_rn(ri, kyz, ai);
        }
      }
      C o;
      o.x = ar;
      o.y = ai;
      P.c_out[(size_t)t * P.M + P.idx[p]] = o;
    }
  }
}

// A run of consecutive plans [p0, p1) of a batch with its ranges of
// point-chunk tasks [t0, t1), subproblem blocks [b0, b1) and mode/grid rows
// [r0, r1) (the plans' task0/blk0/row0 prefix sums are monotone).
struct BatchGroup {
  int p0, p1;
  long long t0, t1, b0, b1, r0, r1;
};

template <typename T> struct Batch {
  std::vector<Plan<T>*> plans;
  std::vector<BatchGroup> groups;   // type 1: spread groups pipelined against FFTs
  std::vector<cudaEvent_t> evpool;  // events of the recorded sequence
  size_t evnext = 0;
  unsigned fft_used = 0;            // FFT streams the recorded sequence used (bit k: side[2 + k])
  // by_plans: the graph holds every plan's own execute (its tuned kernels) on
  // parallel branches instead of multi-plan kernels; it bakes in the
  // caller's arrays, so it is captured again when they change
  bool by_plans = false;
  std::vector<const void*> cap_c, cap_fk;
  int type = 0, dim = 0, ns = 0, device = 0;
  std::vector<cplx_t<T>*> fw;
  std::vector<cufftHandle> fft;
  BatchDesc<T>* h_desc = nullptr;   // pinned
  BatchDesc<T>* d_desc = nullptr;
  long long ntasks = 0, nrows = 0, nblocks = 0;
  size_t smem = 0;  // largest method-2 tile
  size_t smem_run = 0;  // largest cell-run footprint (0: no plan in that layout)
  cudaStream_t stream = nullptr;
  // side streams: the method-2 spread/interp kernels (0, 1) and the per-plan
  // FFTs (2..7) run on parallel branches of the captured graph
  static constexpr int kSide = 8;
  static constexpr int kFftSide = kSide - 2;
  cudaStream_t side[kSide] = {};
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  cudaEvent_t done = nullptr;
  bool launched = false;
};

template <typename T>
inline void batch_release(Batch<T>* b) {
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  if (b->graph) cudaGraphDestroy(b->graph);
  for (cufftHandle h : b->fft) cufftDestroy(h);
  for (auto* p : b->fw) cudaFree(p);
  for (cudaEvent_t e : b->evpool) cudaEventDestroy(e);
  b->evpool.clear();
  b->groups.clear();
  cudaFree(b->d_desc);
  if (b->h_desc) cudaFreeHost(b->h_desc);
  if (b->done) cudaEventDestroy(b->done);
  for (int k = 0; k < Batch<T>::kSide; ++k) {
    if (b->side[k]) cudaStreamDestroy(b->side[k]);
    b->side[k] = nullptr;
  }
  if (b->stream) cudaStreamDestroy(b->stream);
  b->gexec = nullptr;
  b->graph = nullptr;
  b->fft.clear();
  b->fw.clear();
  b->d_desc = nullptr;
  b->h_desc = nullptr;
  b->done = nullptr;
  b->stream = nullptr;
}

// The multi-plan spread/interp kernels over one group's task ranges:
// method-1 chunks on b->stream, method-2 (and cell-run) blocks on side[0] and
// side[1].
template <typename T, int DIM>
inline cudaError_t batch_spreadinterp_dim(Batch<T>* b, int n, const BatchGroup& gr) {
  constexpr int kMaxGrid = 152 * 32;
  const long long ntasks = gr.t1 - gr.t0, nblk = gr.b1 - gr.b0;
  long long blocks = (ntasks * 32 + kSpreadThreads - 1) / kSpreadThreads;
  if (blocks > kMaxGrid) blocks = kMaxGrid;
  if (blocks < 1) blocks = 1;
  const int g = (int)blocks;
  const int gb = (int)std::min<long long>(std::max<long long>(nblk, 1), 152LL * 8);
  cudaError_t fe = cudaSuccess;
#define CFG_BATCH_CASE(NSV)                                                                       \
  case NSV:                                                                                       \
    if (b->type == 1) {                                                                           \
      if (ntasks > 0)                                                                             \
        k_batch_spread<T, DIM, NSV><<<g, kSpreadThreads, 0, b->stream>>>(b->d_desc, n, gr.t0,    \
                                                                         gr.t1);                  \
      if (nblk > 0) {                                                                             \
        fe = prepare_smem(k_batch_spread_sm<T, DIM, NSV>, b->smem);                               \
        if (fe != cudaSuccess) return fe;                                                         \
        k_batch_spread_sm<T, DIM, NSV><<<gb, kSpreadThreads, b->smem, b->side[0]>>>(b->d_desc, n, \
                                                                                  gr.b0, gr.b1); \
        if constexpr (run_ok<DIM, NSV>()) {                                                       \
          if (b->smem_run > 0) {                                                                  \
            fe = prepare_smem(k_batch_spread_run<T, DIM, NSV>, b->smem_run);                      \
            if (fe != cudaSuccess) return fe;                                                     \
            k_batch_spread_run<T, DIM, NSV><<<gb, kSpreadThreads, b->smem_run, b->side[1]>>>(     \
                b->d_desc, n, gr.b0, gr.b1);                                                      \
          }                                                                                       \
        }                                                                                         \
      }                                                                                           \
    } else {                                                                                      \
      if (ntasks > 0)                                                                             \
        k_batch_interp<T, DIM, NSV><<<g, kSpreadThreads, 0, b->stream>>>(b->d_desc, n, gr.t0,    \
                                                                         gr.t1);                  \
      if (nblk > 0) {                                                                             \
        fe = prepare_smem(k_batch_interp_sm<T, DIM, NSV>, b->smem);                               \
        if (fe != cudaSuccess) return fe;                                                         \
        k_batch_interp_sm<T, DIM, NSV><<<gb, kSpreadThreads, b->smem, b->side[0]>>>(b->d_desc, n, \
                                                                                  gr.b0, gr.b1); \
      }                                                                                           \
    }                                                                                             \
    break;
  switch (b->ns) {
    CFG_BATCH_CASE(2) CFG_BATCH_CASE(3) CFG_BATCH_CASE(4) CFG_BATCH_CASE(5) CFG_BATCH_CASE(6)
    CFG_BATCH_CASE(7) CFG_BATCH_CASE(8) CFG_BATCH_CASE(9) CFG_BATCH_CASE(10) CFG_BATCH_CASE(11)
    CFG_BATCH_CASE(12) CFG_BATCH_CASE(13) CFG_BATCH_CASE(14) CFG_BATCH_CASE(15) CFG_BATCH_CASE(16)
    default: return cudaErrorInvalidValue;
  }
#undef CFG_BATCH_CASE
  return cudaGetLastError();
}

// Multi-plan spread/interp launch over one group for one precision;
// instantiated in batch_f.cu and batch_d.cu.
template <typename T>
cudaError_t batch_spreadinterp(Batch<T>* b, const BatchGroup& g);

}  // namespace cfg
