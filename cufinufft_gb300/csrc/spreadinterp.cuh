// spreadinterp.cuh -- spreading (type 1) and interpolation (type 2) kernels.
//
// Method 1 ("NU-point driven", src/2d/spreadinterp2d.cu:16-98 and :516-593
// of the reference): one thread per (bin-sorted) point; spreading adds its
// ns^d taps straight into the fine grid with vector reductions, interpolation
// gathers them.  Method 2 ("subproblem", src/2d/spreadinterp2d.cu:152-312 and
// :596-745): one block per subproblem (<= maxsub points of one bin) works in a
// shared-memory tile that covers the bin plus the ns-1 cells its points reach
// beyond it; spreading accumulates with shared atomics and flushes the tile
// once, interpolation loads the tile once and gathers from it.
//
// Differences from the reference kernels, all result-preserving:
//   * points are read from the plan's sorted SoA copy (first tap + offset in
//     [0,1), see place_coord), not re-rescaled from the caller's arrays;
//   * each thread evaluates its kernel rows once and reuses them for every
//     transform of the batch (the reference launches once per transform);
//   * FP32 plans evaluate the kernel in FP32 (the reference promotes the
//     FP32 build's kernel to FP64, src/cuspreadinterp.h:15);
//   * the tile is bs + ns - 1 wide (the reference pads 2*ceil(ns/2)), and the
//     flush skips cells no point touched;
//   * interpolation tiles that do not wrap the periodic edge arrive by one
//     tiled bulk copy (TMA, cp.async.bulk.tensor) instead of per-cell loads.
#pragma once

#include <cuda.h>  // CUtensorMap and its encoder's types (the encoder is fetched at run time)

#include <cstdlib>
#include <cstring>

#include "device_common.cuh"
#include "kernels.h"
#include "tc_common.cuh"

namespace cfg {

constexpr int kSpreadThreads = 256;
// Threads of a k_interp_sm block, and the blocks per SM its register bound
// is set for.  FP32: 256 threads, 6 blocks (40 registers a thread for
// ns <= 9; 4 blocks above).  FP64 plans' subproblem interpolation (FP64 or
// double-float), 128 registers a thread (two 256-thread blocks ran radial 2D
// FP64 at ns 13 4% faster than one block of 188 registers, despite 52 bytes
// of spill): 2D in one 512-thread block -- the double-float kernel on radial
// 2D at ns 14 1.11 -> 1.01 ms -- and 3D in two 256-thread blocks, whose
// sparse subproblems (tens of points per 8^3 bin) leave most of a 512-thread
// block idle (clustered 3D at ns 11: 74.3 ms against 79.4 ms).  FP32 plans
// keep 256-thread blocks (34.2 vs 35.1 us at ns 8).
constexpr int kInterpThreads = 256;
constexpr int kInterpBlocksF32 = 6 * 256 / kInterpThreads;
template <int DIM> constexpr int interp_threads_f64() { return DIM == 2 ? 512 : 256; }
template <int DIM> constexpr int interp_blocks_f64() { return DIM == 2 ? 1 : 2; }
template <typename T, int DIM> constexpr int interp_threads() {
  return sizeof(T) == 4 ? kInterpThreads : interp_threads_f64<DIM>();
}

// Subproblem header shared by the shared-memory kernels.
struct SubTile {
  int p0, np, ox, oy, oz, TX, TY, TZ, ntile;
};

template <int DIM, int NS>
__device__ __forceinline__ SubTile sub_tile(const BinTables& bt, int sub) {
  SubTile s;
  const int b = bt.sub_to_bin[sub];
  const int js = sub - bt.sub_start[b];
  s.p0 = bt.start[b] + js * bt.maxsub;
  s.np = min(bt.maxsub, bt.count[b] - js * bt.maxsub);
  const int bx = b % bt.nb[0];
  const int by = (b / bt.nb[0]) % bt.nb[1];
  const int bz = b / (bt.nb[0] * bt.nb[1]);
  s.ox = bx * bt.bs[0];
  s.oy = by * bt.bs[1];
  s.oz = bz * bt.bs[2];
  s.TX = bt.bs[0] + NS - 1;
  s.TY = DIM > 1 ? bt.bs[1] + NS - 1 : 1;
  s.TZ = DIM > 2 ? bt.bs[2] + NS - 1 : 1;
  s.ntile = s.TX * s.TY * s.TZ;
  return s;
}

// sub_tile from the subproblem's precomputed header: every thread reads the
// same 16 (3D: 32) bytes, no block barrier.
template <int DIM, int NS>
__device__ __forceinline__ SubTile sub_tile_hdr(const BinTables& bt, int sub) {
  const int4 h = __ldg(reinterpret_cast<const int4*>(bt.hdr + sub));
  SubTile s;
  s.p0 = h.x;
  s.np = h.y;
  s.ox = h.z;
  s.oy = h.w;
  s.oz = DIM > 2 ? __ldg(&bt.hdr[sub].oz) : 0;
  s.TX = bt.bs[0] + NS - 1;
  s.TY = DIM > 1 ? bt.bs[1] + NS - 1 : 1;
  s.TZ = DIM > 2 ? bt.bs[2] + NS - 1 : 1;
  s.ntile = s.TX * s.TY * s.TZ;
  return s;
}

// sub_tile computed once per block (three integer divisions) and shared
// through shared memory; PERSISTENT blocks (several subproblems each) first
// wait until every thread is done with the previous one.
template <int DIM, int NS, bool PERSISTENT = false>
__device__ __forceinline__ SubTile sub_tile_block(const BinTables& bt, int sub) {
  __shared__ SubTile s_tile;
  if (PERSISTENT) __syncthreads();
  if (threadIdx.x == 0) s_tile = sub_tile<DIM, NS>(bt, sub);
  __syncthreads();
  return s_tile;
}

// v wrapped into [0, n) for 0 <= v < 3n: two conditional subtractions.
__device__ __forceinline__ int wrap3(int v, int n) {
  v -= v >= n ? n : 0;
  v -= v >= n ? n : 0;
  return v;
}

// Tile rows (iy, iz) visited by one warp: rows warp, warp + nwarps, ...,
// advanced without divisions.
struct TileRows {
  int iy, iz;
  __device__ __forceinline__ TileRows(int r, int TY) : iy(r % TY), iz(r / TY) {}
  __device__ __forceinline__ void next(int step, int TY) {
    iy += step;
    while (iy >= TY) {
      iy -= TY;
      ++iz;
    }
  }
};

// True when the tile lies inside the grid (no periodic wrap on any axis;
// the unused axes have nf = 1, origin 0 and extent 1).
__device__ __forceinline__ bool tile_in_grid(const SubTile& st, const GridGeom& g) {
  return st.ox + st.TX <= g.nf[0] && st.oy + st.TY <= g.nf[1] && st.oz + st.TZ <= g.nf[2];
}

// Copy the subproblem's padded tile from the fine grid (periodic wrap) into
// shared memory: one warp per tile row, lanes along x.  Tile coordinates
// stay below 3 nf (bins within the grid, halo ns - 1 <= nf / 2), so two
// conditional subtractions wrap them.
template <typename T>
__device__ __forceinline__ void tile_load_periodic(cplx_t<T>* tile, const cplx_t<T>* grid, const SubTile& st,
                                                   const GridGeom& g) {
  const int lane = threadIdx.x & 31, nwb = blockDim.x >> 5;
  const int rows = st.TY * st.TZ;
  TileRows rw(threadIdx.x >> 5, st.TY);
  for (int r = threadIdx.x >> 5; r < rows; r += nwb, rw.next(nwb, st.TY)) {
    const int gy = wrap3(st.oy + rw.iy, g.nf[1]), gz = wrap3(st.oz + rw.iz, g.nf[2]);
    const cplx_t<T>* src = grid + ((size_t)gz * g.nf[1] + gy) * g.nf[0];
    cplx_t<T>* dst = tile + r * st.TX;
    for (int ix = lane; ix < st.TX; ix += 32) {
      const int gx = wrap3(st.ox + ix, g.nf[0]);
      // asynchronous copy: no register round trip, many cells in flight
      if constexpr (sizeof(T) == 4) cp_async8(dst + ix, src + gx);
      else cp_async16(dst + ix, src + gx);
    }
  }
  cp_async_wait();  // this thread's copies have landed; the caller syncs the block
}

// Same, without the per-cell wrap where the tile lies inside the grid.
template <typename T>
__device__ __forceinline__ void tile_load(cplx_t<T>* tile, const cplx_t<T>* grid, const SubTile& st,
                                          const GridGeom& g) {
  if (!tile_in_grid(st, g)) {
    tile_load_periodic<T>(tile, grid, st, g);
    return;
  }
  const int lane = threadIdx.x & 31, nwb = blockDim.x >> 5;
  const int rows = st.TY * st.TZ;
  TileRows rw(threadIdx.x >> 5, st.TY);
  for (int r = threadIdx.x >> 5; r < rows; r += nwb, rw.next(nwb, st.TY)) {
    const cplx_t<T>* src = grid + ((size_t)(st.oz + rw.iz) * g.nf[1] + st.oy + rw.iy) * g.nf[0] + st.ox;
    cplx_t<T>* dst = tile + r * st.TX;
    for (int ix = lane; ix < st.TX; ix += 32) {
      if constexpr (sizeof(T) == 4) cp_async8(dst + ix, src + ix);
      else cp_async16(dst + ix, src + ix);
    }
  }
  cp_async_wait();
}

// Add the tile back into the fine grid with vector reductions, skipping the
// cells no point touched.
template <typename T>
__device__ __forceinline__ void tile_flush(const cplx_t<T>* tile, cplx_t<T>* grid, const SubTile& st,
                                           const GridGeom& g) {
  const int lane = threadIdx.x & 31, nwb = blockDim.x >> 5;
  const int rows = st.TY * st.TZ;
  TileRows rw(threadIdx.x >> 5, st.TY);
  if (tile_in_grid(st, g)) {  // no wrap
    for (int r = threadIdx.x >> 5; r < rows; r += nwb, rw.next(nwb, st.TY)) {
      cplx_t<T>* dst = grid + ((size_t)(st.oz + rw.iz) * g.nf[1] + st.oy + rw.iy) * g.nf[0] + st.ox;
      const cplx_t<T>* src = tile + r * st.TX;
      for (int ix = lane; ix < st.TX; ix += 32) {
        const cplx_t<T> v = src[ix];
        if (v.x == T(0) && v.y == T(0)) continue;
        red_add(dst + ix, v.x, v.y);
      }
    }
    return;
  }
  for (int r = threadIdx.x >> 5; r < rows; r += nwb, rw.next(nwb, st.TY)) {
    const int gy = wrap3(st.oy + rw.iy, g.nf[1]), gz = wrap3(st.oz + rw.iz, g.nf[2]);
    cplx_t<T>* dst = grid + ((size_t)gz * g.nf[1] + gy) * g.nf[0];
    const cplx_t<T>* src = tile + r * st.TX;
    for (int ix = lane; ix < st.TX; ix += 32) {
      const cplx_t<T> v = src[ix];
      if (v.x == T(0) && v.y == T(0)) continue;
      red_add(dst + wrap3(st.ox + ix, g.nf[0]), v.x, v.y);
    }
  }
}

// ---- TMA tile loads (interpolation) ---------------------------------------
// The fine grids are described to the copy engine as a (DIM+1)-rank tensor
// of real components: x runs over 2 nf0 reals, then y, z and the transform
// index.  A subproblem tile that does not wrap the periodic edge is one box
// of that tensor ({2 TX, TY, TZ, 1} at (2 ox, oy, oz, t)), moved into shared
// memory by one tiled bulk copy that one thread issues; the block waits on
// an mbarrier.  Tiles that wrap keep the per-cell cp.async path.

// Polls of the tile barrier before a thread gives up on the bulk copy and
// loads its share of the tile itself (the data is the same either way).
// Each poll may itself wait a short, hardware-chosen time.
constexpr int kTmaWaitPolls = 1 << 20;

// Tile row length (cells) of a bulk-copied tile: a box row must be a
// multiple of 16 bytes, so FP32 rows of an odd number of cells take one
// more cell (its value is loaded and never used).
template <typename T>
__host__ __device__ __forceinline__ int bulk_tile_x(int TX) {
  return sizeof(T) == 4 ? (TX + 1) & ~1 : TX;
}

// Shared-memory start of the tile rounded up to 128 bytes (bulk tensor
// copies want an aligned destination; the launch adds 128 bytes).
__device__ __forceinline__ unsigned char* smem_align128(unsigned char* p) {
  return p + ((128u - (smem_u32(p) & 127u)) & 127u);
}

// Thread 0: start the tile's bulk copy.
template <typename T, int DIM>
__device__ __forceinline__ void tile_copy_start(cplx_t<T>* tile, const CUtensorMap* map, const SubTile& st,
                                                int t, unsigned long long* bar) {
  mbar_expect_tx(bar, (unsigned)(st.ntile * sizeof(cplx_t<T>)));
  if constexpr (DIM == 1) tma_load2(tile, map, 2 * st.ox, t, bar);
  else if constexpr (DIM == 2) tma_load3(tile, map, 2 * st.ox, st.oy, t, bar);
  else tma_load4(tile, map, 2 * st.ox, st.oy, st.oz, t, bar);
}

// Every thread: wait for the bulk copy.  A thread whose wait runs out
// records it in status[0] (the next call on the plan returns an error) and
// loads its share of the tile cell by cell, which writes the values the copy
// writes; it then waits for the copy once more, so that the block does not
// retire -- and its shared memory go to another block -- while the copy may
// still write into it.  A copy still missing after that second wait is
// recorded in status[1].  `test` makes the first wait give up at once.
__device__ __forceinline__ void status_set(int* status, int k) {
  if (status) *reinterpret_cast<volatile int*>(status + k) = 1;
}
template <typename T>
__device__ __forceinline__ void tile_copy_wait(cplx_t<T>* tile, unsigned long long* bar, const cplx_t<T>* grid,
                                               const SubTile& st, const GridGeom& g, int* status, int test) {
  if (mbar_wait(bar, 0, test ? 0 : kTmaWaitPolls)) return;
  status_set(status, 0);
  tile_load_periodic<T>(tile, grid, st, g);
  if (!mbar_wait(bar, 0, kTmaWaitPolls)) status_set(status, 1);
}

// Host: encode the tensor map of `ntr` fine grids at `grid` for tiles of a
// bulk_tile_x(bs0 + ns - 1) x (bs1 + ns - 1) x (bs2 + ns - 1) box.  Returns
// false (the kernel then loads every tile cell by cell) where a rule of
// tiled bulk copies would be broken: a start address or row pitch off 16
// bytes, an odd FP32 bin width (tile x origins must sit on 16 bytes), a box
// side above 256, or no encoder in the driver.  CUFINUFFT_TMA=0 turns the
// bulk copies off.
template <typename T, int DIM>
bool grid_tensor_map(CUtensorMap* map, const cplx_t<T>* grid, const GridGeom& g, int ntr, const int bs[3],
                     int ns) {
  using Encode = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                              const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                              CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
  const Encode encode = reinterpret_cast<Encode>(tma_encoder());
  if (const char* v = std::getenv("CUFINUFFT_TMA"))
    if (v[0] == '0') return false;
  if (!encode || grid == nullptr || ntr < 1) return false;
  const int TX = bulk_tile_x<T>(bs[0] + ns - 1), TY = DIM > 1 ? bs[1] + ns - 1 : 1,
            TZ = DIM > 2 ? bs[2] + ns - 1 : 1;
  constexpr size_t C = sizeof(cplx_t<T>);
  if ((reinterpret_cast<uintptr_t>(grid) & 15) != 0) return false;
  if (sizeof(T) == 4 && (bs[0] & 1)) return false;
  if (2 * TX > 256 || TY > 256 || TZ > 256) return false;
  if (TX > g.nf[0] || TY > g.nf[1] || TZ > g.nf[2]) return false;
  cuuint64_t dims[4], strides[3];
  cuuint32_t box[4], estr[4] = {1, 1, 1, 1};
  int r = 0;
  dims[r] = 2ull * g.nf[0];
  box[r++] = 2u * TX;
  size_t pitch = (size_t)g.nf[0] * C;
  if (DIM > 1) { strides[r - 1] = pitch; dims[r] = g.nf[1]; box[r++] = TY; pitch *= g.nf[1]; }
  if (DIM > 2) { strides[r - 1] = pitch; dims[r] = g.nf[2]; box[r++] = TZ; }
  strides[r - 1] = (size_t)g.Nf * C;
  dims[r] = ntr;
  box[r++] = 1;
  for (int i = 0; i < r - 1; ++i)
    if (strides[i] % 16 != 0 || strides[i] >= (1ull << 40)) return false;
  std::memset(map, 0, sizeof(*map));
  const CUresult e = encode(map, sizeof(T) == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64,
                            (cuuint32_t)r, const_cast<cplx_t<T>*>(grid), dims, strides, box, estr,
                            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return e == CUDA_SUCCESS;
}

template <typename T>
__device__ __forceinline__ void tile_zero(cplx_t<T>* tile, int ntile) {
  for (int i = threadIdx.x; i < ntile; i += blockDim.x) {
    tile[i].x = T(0);
    tile[i].y = T(0);
  }
}

// ---------------------------------------------------------------------------
// Method 1: NU-point driven spread.
template <typename T, int DIM, int NS>
__global__ void __launch_bounds__(kSpreadThreads)
k_spread_gm(SpreadArgs<T> a) {
  using C = cplx_t<T>;
  constexpr int HD = horner_degree<T>(NS);
  constexpr int NY = DIM > 1 ? NS : 1;
  constexpr int NZ = DIM > 2 ? NS : 1;
  const int nf0 = a.g.nf[0], nf1 = a.g.nf[1], nf2 = a.g.nf[2];
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < a.M; p += gridDim.x * blockDim.x) {
    T k1[NS], k2[NS];
    int xs[NS];
    const int i1 = a.pts.i0[0][p];
    kernel_row<T, NS, HD>(a.pts.d[0][p], a.kc, k1);
#pragma unroll
    for (int j = 0; j < NS; ++j) xs[j] = wrap_idx(i1 + j, nf0);
    int i2 = 0, i3 = 0;
    if (DIM > 1) { i2 = a.pts.i0[1][p]; kernel_row<T, NS, HD>(a.pts.d[1][p], a.kc, k2); }
    T d3 = T(0);
    if (DIM > 2) { i3 = a.pts.i0[2][p]; d3 = a.pts.d[2][p]; }
    const int src = a.pts.idx[p];
    for (int t = 0; t < a.ntr; ++t) {
      const C v = a.c_in[(size_t)t * a.M + src];
      C* base = a.fw + (size_t)t * a.g.Nf;
#pragma unroll 1
      for (int dz = 0; dz < NZ; ++dz) {
        const int iz = DIM > 2 ? wrap_idx(i3 + dz, nf2) : 0;
        const T kz = DIM > 2 ? kernel_tap<T, NS, HD>(d3, dz, a.kc) : T(1);
#pragma unroll
        for (int dy = 0; dy < NY; ++dy) {
          const int iy = DIM > 1 ? wrap_idx(i2 + dy, nf1) : 0;
          T kyz = T(1);
          if (DIM > 1) kyz = k2[dy];
          if (DIM > 2) kyz *= kz;
          const T vr = v.x * kyz, vi = v.y * kyz;
          C* row = base + ((size_t)iz * nf1 + iy) * nf0;
#pragma unroll
          for (int dx = 0; dx < NS; ++dx) red_add(row + xs[dx], vr * k1[dx], vi * k1[dx]);
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Method 2: shared-memory subproblem spread.  grid = (nsub, ntr).
template <typename T, int DIM, int NS>
__global__ void __launch_bounds__(kSpreadThreads)
k_spread_sm(SpreadArgs<T> a) {
  using C = cplx_t<T>;
  constexpr int HD = horner_degree<T>(NS);
  constexpr int NY = DIM > 1 ? NS : 1;
  constexpr int NZ = DIM > 2 ? NS : 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* tile = reinterpret_cast<C*>(smem_raw);
  const SubTile st = sub_tile_block<DIM, NS>(a.bins, blockIdx.x);
  const int t = blockIdx.y;
  tile_zero<T>(tile, st.ntile);
  __syncthreads();
  const C* cin = a.c_in + (size_t)t * a.M;
  for (int p = st.p0 + threadIdx.x; p < st.p0 + st.np; p += blockDim.x) {
    T k1[NS], k2[NS];
    const int lx = a.pts.i0[0][p] - st.ox;
    kernel_row<T, NS, HD>(a.pts.d[0][p], a.kc, k1);
    int ly = 0, lz = 0;
    if (DIM > 1) { ly = a.pts.i0[1][p] - st.oy; kernel_row<T, NS, HD>(a.pts.d[1][p], a.kc, k2); }
    T d3 = T(0);
    if (DIM > 2) { lz = a.pts.i0[2][p] - st.oz; d3 = a.pts.d[2][p]; }
    const C v = cin[a.pts.idx[p]];
#pragma unroll 1
    for (int dz = 0; dz < NZ; ++dz) {
      const T kz = DIM > 2 ? kernel_tap<T, NS, HD>(d3, dz, a.kc) : T(1);
      C* plane = tile + ((lz + dz) * st.TY + ly) * st.TX + lx;
#pragma unroll
      for (int dy = 0; dy < NY; ++dy) {
        T kyz = T(1);
        if (DIM > 1) kyz = k2[dy];
        if (DIM > 2) kyz *= kz;
        const T vr = v.x * kyz, vi = v.y * kyz;
        C* row = plane + dy * st.TX;
#pragma unroll
        for (int dx = 0; dx < NS; ++dx) smem_add(row + dx, vr * k1[dx], vi * k1[dx]);
      }
    }
  }
  __syncthreads();
  tile_flush<T>(tile, a.fw + (size_t)t * a.g.Nf, st, a.g);
}

// ---------------------------------------------------------------------------
// Method 1: NU-point driven interpolation (gather).
template <typename T, int DIM, int NS>
__global__ void __launch_bounds__(kSpreadThreads)
k_interp_gm(SpreadArgs<T> a) {
  using C = cplx_t<T>;
  constexpr int HD = horner_degree<T>(NS);
  constexpr int NY = DIM > 1 ? NS : 1;
  constexpr int NZ = DIM > 2 ? NS : 1;
  const int nf0 = a.g.nf[0], nf1 = a.g.nf[1], nf2 = a.g.nf[2];
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < a.M; p += gridDim.x * blockDim.x) {
    T k1[NS], k2[NS];
    int xs[NS];
    const int i1 = a.pts.i0[0][p];
    kernel_row<T, NS, HD>(a.pts.d[0][p], a.kc, k1);
#pragma unroll
    for (int j = 0; j < NS; ++j) xs[j] = wrap_idx(i1 + j, nf0);
    int i2 = 0, i3 = 0;
    if (DIM > 1) { i2 = a.pts.i0[1][p]; kernel_row<T, NS, HD>(a.pts.d[1][p], a.kc, k2); }
    T d3 = T(0);
    if (DIM > 2) { i3 = a.pts.i0[2][p]; d3 = a.pts.d[2][p]; }
    const int dst = a.pts.idx[p];
    for (int t = 0; t < a.ntr; ++t) {
      const C* base = a.fw_in + (size_t)t * a.g.Nf;
      T ar = T(0), ai = T(0);
#pragma unroll 1
      for (int dz = 0; dz < NZ; ++dz) {
        const int iz = DIM > 2 ? wrap_idx(i3 + dz, nf2) : 0;
        const T kz = DIM > 2 ? kernel_tap<T, NS, HD>(d3, dz, a.kc) : T(1);
#pragma unroll
        for (int dy = 0; dy < NY; ++dy) {
          const int iy = DIM > 1 ? wrap_idx(i2 + dy, nf1) : 0;
          const C* row = base + ((size_t)iz * nf1 + iy) * nf0;
          T rr = T(0), ri = T(0);
#pragma unroll
          for (int dx = 0; dx < NS; ++dx) {
            const C g = __ldg(row + xs[dx]);
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
      C out;
      out.x = ar;
      out.y = ai;
      a.c_out[(size_t)t * a.M + dst] = out;
    }
  }
}

// ---------------------------------------------------------------------------
// Method 2: shared-memory subproblem interpolation.  grid = (nsub, ntr).

// One point's tile offsets and kernel rows: everything the taps need except
// the tile itself.
template <typename T, int DIM, int NS>
struct InterpPoint {
  T k1[NS], k2[NS];
  T d1, d2, d3;
  int lx, ly, lz;
  // the point's sorted coordinates (first tap, offset)
  __device__ __forceinline__ void fetch(const SpreadArgs<T>& a, int p, const SubTile& st) {
    lx = a.pts.i0[0][p] - st.ox;
    d1 = a.pts.d[0][p];
    ly = lz = 0;
    d2 = d3 = T(0);
    if (DIM > 1) { ly = a.pts.i0[1][p] - st.oy; d2 = a.pts.d[1][p]; }
    if (DIM > 2) { lz = a.pts.i0[2][p] - st.oz; d3 = a.pts.d[2][p]; }
  }
  // kernel rows along x and y (z values are evaluated per plane)
  __device__ __forceinline__ void rows(const SpreadArgs<T>& a) {
    constexpr int HD = horner_degree<T>(NS);
    kernel_row<T, NS, HD>(d1, a.kc, k1);
    if (DIM > 1) kernel_row<T, NS, HD>(d2, a.kc, k2);
  }
  __device__ __forceinline__ cplx_t<T> taps(const SpreadArgs<T>& a, const cplx_t<T>* tile,
                                            const SubTile& st) const {
    using C = cplx_t<T>;
    constexpr int HD = horner_degree<T>(NS);
    constexpr int NY = DIM > 1 ? NS : 1;
    constexpr int NZ = DIM > 2 ? NS : 1;
    C out;
    if constexpr (sizeof(T) == 4) {
      // packed pairs: one fma.rn.f32x2 per complex tap (same IEEE fmas)
      float2 k1p[NS];
#pragma unroll
      for (int dx = 0; dx < NS; ++dx) k1p[dx] = make_float2(k1[dx], k1[dx]);
      float2 acc = make_float2(0.f, 0.f);
#pragma unroll 1
      for (int dz = 0; dz < NZ; ++dz) {
        const T kz = DIM > 2 ? kernel_tap<T, NS, HD>(d3, dz, a.kc) : T(1);
        const C* plane = tile + ((lz + dz) * st.TY + ly) * st.TX + lx;
#pragma unroll
        for (int dy = 0; dy < NY; ++dy) {
          const C* row = plane + dy * st.TX;
          float2 r = make_float2(0.f, 0.f);
#pragma unroll
          for (int dx = 0; dx < NS; ++dx) r = fma2(row[dx], k1p[dx], r);
          T kyz = T(1);
          if (DIM > 1) kyz = k2[dy];
          if (DIM > 2) kyz *= kz;
          acc = fma2(r, make_float2(kyz, kyz), acc);
        }
      }
      out = acc;
    } else {
      T ar = T(0), ai = T(0);
#pragma unroll 1
      for (int dz = 0; dz < NZ; ++dz) {
        const T kz = DIM > 2 ? kernel_tap<T, NS, HD>(d3, dz, a.kc) : T(1);
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
      out.x = ar;
      out.y = ai;
    }
    return out;
  }
};

// The coordinates of every thread's first point are read while the tile is
// still on its way (the bulk copy runs in the background; the per-cell path
// is asynchronous up to its wait).  Its kernel rows are evaluated after the
// wait: evaluated before it, the rows stay live across the wait and the FP32
// kernels spill at the 40-register bound (measured 3.5% slower).
template <typename T, int DIM, int NS>
__global__ void __launch_bounds__(interp_threads<T, DIM>(), sizeof(T) == 4 ? (NS <= 9 ? kInterpBlocksF32 : kInterpBlocksF32 * 2 / 3) : interp_blocks_f64<DIM>())
k_interp_sm(SpreadArgs<T> a, const __grid_constant__ CUtensorMap gmap, int tma) {
  using C = cplx_t<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ __align__(8) unsigned long long tile_bar;
  C* tile = reinterpret_cast<C*>(tma ? smem_align128(smem_raw) : smem_raw);
  if (tma && threadIdx.x == 0) mbar_init(&tile_bar, 1);
  SubTile st = sub_tile_hdr<DIM, NS>(a.bins, blockIdx.x);  // loads in flight across the barrier
  if (tma) __syncthreads();                                 // the barrier's init before any wait on it
  if (tma) {  // the tile row widened as the tensor map's box is (bulk_tile_x)
    st.TX = bulk_tile_x<T>(st.TX);
    st.ntile = st.TX * st.TY * st.TZ;
  }
  const int t = blockIdx.y;
  const C* src = a.fw_in + (size_t)t * a.g.Nf;
  const bool bulk = tma && tile_in_grid(st, a.g) && (sizeof(T) == 8 || (st.ox & 1) == 0);
  if (bulk && threadIdx.x == 0) tile_copy_start<T, DIM>(tile, &gmap, st, t, &tile_bar);
  const int p_end = st.p0 + st.np;
  int p = st.p0 + threadIdx.x;
  InterpPoint<T, DIM, NS> pt;
  if (!bulk) tile_load_periodic<T>(tile, src, st, a.g);
  if (p < p_end) pt.fetch(a, p, st);
  if (bulk) tile_copy_wait<T>(tile, &tile_bar, src, st, a.g, a.status, a.tma_wait_test);
  __syncthreads();
  if (p >= p_end) return;
  pt.rows(a);
  a.c_out[(size_t)t * a.M + a.pts.idx[p]] = pt.taps(a, tile, st);
  for (p += blockDim.x; p < p_end; p += blockDim.x) {
    pt.fetch(a, p, st);
    pt.rows(a);
    a.c_out[(size_t)t * a.M + a.pts.idx[p]] = pt.taps(a, tile, st);
  }
}

// ---------------------------------------------------------------------------
// Double-float interpolation for FP64 plans (SpreadArgs::fp64_df).  GB300's
// FP64 units are a small fraction of its FP32 throughput, and the FP64 tap
// loop (2 FMAs per tap, ns^d taps) plus the FP64 kernel evaluation (a Horner
// step per tap value and degree) bound FP64 interpolation.  Here the tile
// (loaded as for k_interp_sm) is converted in place to FP32 pairs (hi, lo per
// component, the same 16 bytes per cell), the kernel rows are evaluated in
// double-float (the fitted polynomials from FP32-pair coefficients, or the
// FP64 exp form rounded to pairs), and the taps accumulate as a float sum
// plus a float error term (two-sum and FMA product errors): ~2^-46
// relative, ample for tol >= 1e-13, with FP32 instructions only.
struct DFAcc {
  float s, t;
  __device__ __forceinline__ void zero() { s = t = 0.f; }
  // += a * b
  __device__ __forceinline__ void add_prod(DF a, float bh, float bl) {
    const float p = __fmul_rn(a.h, bh);
    float pe = __fmaf_rn(a.h, bh, -p);
    pe = __fmaf_rn(a.h, bl, pe);
    pe = __fmaf_rn(a.l, bh, pe);
    float ns, e;
    two_sum(s, p, ns, e);
    s = ns;
    t = __fadd_rn(t, __fadd_rn(e, pe));
  }
  __device__ __forceinline__ DF value() const { return df_renorm(s, t); }
};

// The kernel's power-of-two scale E = round(beta log2 e): kernel values are
// taken times 2^-E and grid values times 2^(dim E), products unchanged
// (exact scalings), every factor near 1 in FP32's exponent range.
__device__ __forceinline__ int df_scale_exp(double beta) { return (int)rint(beta * 1.44269504088896340736); }

// Kernel value phi(d - ns/2 + j) 2^-E in double-float.
template <int NS, int HD>
__device__ __forceinline__ DF df_kernel_tap(double d, int j, const KernelCoeffs<double>& kc) {
  if (kc.horner) {
    const DF z = df_from(2.0 * d - 1.0);
    DF v;
    v.h = kc.df.hi[j];
    v.l = kc.df.lo[j];
#pragma unroll
    for (int k = 1; k <= HD; ++k) {
      DF c;
      c.h = kc.df.hi[k * NS + j];
      c.l = kc.df.lo[k * NS + j];
      v = df_fma(v, z, c);
    }
    return v;
  }
  const double x = d - 0.5 * NS + j;
  return df_from(ldexp(es_value(kc.c * x * x, kc.beta), -df_scale_exp(kc.beta)));
}

template <int DIM, int NS>
__global__ void __launch_bounds__(interp_threads_f64<DIM>(), interp_blocks_f64<DIM>())
k_interp_sm_df(SpreadArgs<double> a, const __grid_constant__ CUtensorMap gmap, int tma) {
  using C = double2;
  constexpr int HD = horner_degree<double>(NS);
  constexpr int NY = DIM > 1 ? NS : 1;
  constexpr int NZ = DIM > 2 ? NS : 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ __align__(8) unsigned long long tile_bar;
  C* tile = reinterpret_cast<C*>(tma ? smem_align128(smem_raw) : smem_raw);
  if (tma && threadIdx.x == 0) mbar_init(&tile_bar, 1);
  SubTile st = sub_tile_hdr<DIM, NS>(a.bins, blockIdx.x);
  if (tma) __syncthreads();
  const int t = blockIdx.y;
  const C* src = a.fw_in + (size_t)t * a.g.Nf;
  const bool bulk = tma && tile_in_grid(st, a.g);
  if (bulk && threadIdx.x == 0) tile_copy_start<double, DIM>(tile, &gmap, st, t, &tile_bar);
  if (!bulk) tile_load_periodic<double>(tile, src, st, a.g);
  if (bulk) tile_copy_wait<double>(tile, &tile_bar, src, st, a.g, a.status, a.tma_wait_test);
  __syncthreads();
  // the tile in place as FP32 pairs: (re hi, re lo, im hi, im lo) per cell,
  // scaled by 2^(DIM E) (exact)
  float4* tdf = reinterpret_cast<float4*>(tile);
  const double gscale = ldexp(1.0, DIM * df_scale_exp(a.kc.beta));
  for (int i = threadIdx.x; i < st.ntile; i += blockDim.x) {
    const C v = tile[i];
    const DF r = df_from(v.x * gscale), m = df_from(v.y * gscale);
    tdf[i] = make_float4(r.h, r.l, m.h, m.l);
  }
  __syncthreads();
  const int p_end = st.p0 + st.np;
  for (int p = st.p0 + threadIdx.x; p < p_end; p += blockDim.x) {
    const int lx = a.pts.i0[0][p] - st.ox;
    const int ly = DIM > 1 ? a.pts.i0[1][p] - st.oy : 0;
    const int lz = DIM > 2 ? a.pts.i0[2][p] - st.oz : 0;
    DF kx[NS], ky[NY];
    const double d1 = a.pts.d[0][p];
#pragma unroll
    for (int j = 0; j < NS; ++j) kx[j] = df_kernel_tap<NS, HD>(d1, j, a.kc);
    if (DIM > 1) {
      const double d2 = a.pts.d[1][p];
#pragma unroll
      for (int j = 0; j < NY; ++j) ky[j] = df_kernel_tap<NS, HD>(d2, j, a.kc);
    } else {
      ky[0].h = 1.f;
      ky[0].l = 0.f;
    }
    const double d3 = DIM > 2 ? a.pts.d[2][p] : 0.0;
    DFAcc are, aim;
    are.zero();
    aim.zero();
#pragma unroll 1
    for (int dz = 0; dz < NZ; ++dz) {
      DF kz;
      if (DIM > 2) kz = df_kernel_tap<NS, HD>(d3, dz, a.kc);
      const float4* plane = tdf + ((lz + dz) * st.TY + ly) * st.TX + lx;
      // rows rolled: a fully unrolled ns x ns body of double-float taps
      // outgrows the instruction cache (ncu: instruction-fetch stalls first);
      // ky[dy] is then read from an L1-resident local array.  Measured: 3D
      // ns 11 interp 66.1 -> 53.7 ms, 2D ns 14 1.01 -> 0.90 ms
#pragma unroll 1
      for (int dy = 0; dy < NY; ++dy) {
        const float4* row = plane + dy * st.TX;
        DFAcc rre, rim;
        rre.zero();
        rim.zero();
#pragma unroll
        for (int dx = 0; dx < NS; ++dx) {
          const float4 g = row[dx];
          rre.add_prod(kx[dx], g.x, g.y);
          rim.add_prod(kx[dx], g.z, g.w);
        }
        DF w = ky[dy];
        if (DIM > 2) w = df_mul(w, kz);
        const DF vr = rre.value(), vi = rim.value();
        are.add_prod(w, vr.h, vr.l);
        aim.add_prod(w, vi.h, vi.l);
      }
    }
    C o;
    o.x = df_to(are.value());
    o.y = df_to(aim.value());
    a.c_out[(size_t)t * a.M + a.pts.idx[p]] = o;
  }
}


// ---------------------------------------------------------------------------
// Warp-cooperative variants.  A warp works on PPW = 32 / L points at a time;
// the L >= ns lanes of a point cover its x taps, so every warp-wide memory
// instruction touches PPW contiguous runs of ns cells (one row of each
// point) instead of 32 scattered cells.  Lane j evaluates the x, y and z
// kernel values of tap j; the y/z values of a row are broadcast with one
// shuffle.  Interpolation reduces the L per-tap partial sums of a point with
// a butterfly at the end.
template <int NS> constexpr int lanes_per_point() {
  return NS <= 2 ? 2 : (NS <= 4 ? 4 : (NS <= 8 ? 8 : 16));
}
// Spreading needs no butterfly, so its lane groups are exactly ns wide:
// floor(32/ns) points per warp step (5 at ns = 6 instead of 4).
template <int NS> constexpr int spread_lanes() { return NS; }

template <typename T, int DIM, int NS>
__global__ void __launch_bounds__(kSpreadThreads)
k_interp_gm_wc(SpreadArgs<T> a) {
  using C = cplx_t<T>;
  constexpr int HD = horner_degree<T>(NS);
  constexpr int L = lanes_per_point<NS>();
  constexpr int PPW = 32 / L;
  constexpr int NY = DIM > 1 ? NS : 1;
  constexpr int NZ = DIM > 2 ? NS : 1;
  const int lane = threadIdx.x & 31, g = lane / L, j = lane % L;
  const bool tap = j < NS;
  const int jj = tap ? j : 0;
  const long long wid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  const int nf0 = a.g.nf[0], nf1 = a.g.nf[1], nf2 = a.g.nf[2];
  for (long long base = wid * PPW; base < a.M; base += nw * PPW) {
    const long long pl = base + g;
    const bool valid = pl < a.M;
    const int p = valid ? (int)pl : a.M - 1;
    const int xj = wrap_idx(a.pts.i0[0][p] + jj, nf0);
    const T kx = kernel_tap<T, NS, HD>(a.pts.d[0][p], jj, a.kc);
    T ky = T(1), kz = T(1);
    int i2 = 0, i3 = 0;
    if (DIM > 1) { i2 = a.pts.i0[1][p]; ky = kernel_tap<T, NS, HD>(a.pts.d[1][p], jj, a.kc); }
    if (DIM > 2) { i3 = a.pts.i0[2][p]; kz = kernel_tap<T, NS, HD>(a.pts.d[2][p], jj, a.kc); }
    const int dst = a.pts.idx[p];
    for (int t = 0; t < a.ntr; ++t) {
      const C* gt = a.fw_in + (size_t)t * a.g.Nf + xj;
      T ar = T(0), ai = T(0);
#pragma unroll 1
      for (int dz = 0; dz < NZ; ++dz) {
        const T kzv = DIM > 2 ? __shfl_sync(0xffffffffu, kz, g * L + dz) : T(1);
        const int iz = DIM > 2 ? wrap_idx(i3 + dz, nf2) : 0;
#pragma unroll
        for (int dy = 0; dy < NY; ++dy) {
          const T kyv = DIM > 1 ? __shfl_sync(0xffffffffu, ky, g * L + dy) : T(1);
          const int iy = DIM > 1 ? wrap_idx(i2 + dy, nf1) : 0;
          if (tap) {
            const C v = __ldg(gt + ((size_t)iz * nf1 + iy) * nf0);
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
        a.c_out[(size_t)t * a.M + dst] = o;
      }
    }
  }
}

template <typename T, int DIM, int NS>
__global__ void __launch_bounds__(kSpreadThreads)
k_spread_gm_wc(SpreadArgs<T> a) {
  using C = cplx_t<T>;
  constexpr int HD = horner_degree<T>(NS);
  constexpr int L = spread_lanes<NS>();
  constexpr int PPW = 32 / L;
  constexpr int NY = DIM > 1 ? NS : 1;
  constexpr int NZ = DIM > 2 ? NS : 1;
  const int lane = threadIdx.x & 31, g = lane / L, j = lane % L;
  const bool tap = j < NS;
  const int jj = tap ? j : 0;
  const long long wid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  const int nf0 = a.g.nf[0], nf1 = a.g.nf[1], nf2 = a.g.nf[2];
  for (long long base = wid * PPW; base < a.M; base += nw * PPW) {
    const long long pl = base + g;
    const bool valid = g < PPW && pl < a.M;
    const int p = valid ? (int)pl : a.M - 1;
    const int xj = wrap_idx(a.pts.i0[0][p] + jj, nf0);
    const T kx = kernel_tap<T, NS, HD>(a.pts.d[0][p], jj, a.kc);
    T ky = T(1), kz = T(1);
    int i2 = 0, i3 = 0;
    if (DIM > 1) { i2 = a.pts.i0[1][p]; ky = kernel_tap<T, NS, HD>(a.pts.d[1][p], jj, a.kc); }
    if (DIM > 2) { i3 = a.pts.i0[2][p]; kz = kernel_tap<T, NS, HD>(a.pts.d[2][p], jj, a.kc); }
    const int src = a.pts.idx[p];
    for (int t = 0; t < a.ntr; ++t) {
      const C v = a.c_in[(size_t)t * a.M + src];
      const T vr = v.x * kx, vi = v.y * kx;
      C* gt = a.fw + (size_t)t * a.g.Nf + xj;
#pragma unroll 1
      for (int dz = 0; dz < NZ; ++dz) {
        const T kzv = DIM > 2 ? __shfl_sync(0xffffffffu, kz, g * L + dz) : T(1);
        const int iz = DIM > 2 ? wrap_idx(i3 + dz, nf2) : 0;
#pragma unroll
        for (int dy = 0; dy < NY; ++dy) {
          const T kyv = DIM > 1 ? __shfl_sync(0xffffffffu, ky, g * L + dy) : T(1);
          const int iy = DIM > 1 ? wrap_idx(i2 + dy, nf1) : 0;
          const T w = kyv * kzv;
          if (tap && valid) red_add(gt + ((size_t)iz * nf1 + iy) * nf0, vr * w, vi * w);
        }
      }
    }
  }
}

// The tile is held as two planes (real parts, then imaginary parts): the ns
// taps of a point's row are then ns consecutive words of one plane, so a
// warp's shared atomics touch ns consecutive banks per point instead of every
// other bank of 2 ns (interleaved complex), halving bank conflicts.
template <typename T>
__device__ __forceinline__ void plane_flush(const T* re, const T* im, cplx_t<T>* grid,
                                            const SubTile& st, const GridGeom& g) {
  const int pitch = st.TX;  // row pitch of the planes (elements)
  const int lane = threadIdx.x & 31, nwb = blockDim.x >> 5;
  const int rows = st.TY * st.TZ;
  TileRows rw(threadIdx.x >> 5, st.TY);
  if (tile_in_grid(st, g)) {  // no wrap
    for (int r = threadIdx.x >> 5; r < rows; r += nwb, rw.next(nwb, st.TY)) {
      cplx_t<T>* dst = grid + ((size_t)(st.oz + rw.iz) * g.nf[1] + st.oy + rw.iy) * g.nf[0] + st.ox;
      const T* rr = re + r * pitch;
      const T* ri = im + r * pitch;
      for (int ix = lane; ix < st.TX; ix += 32) {
        const T vr = rr[ix], vi = ri[ix];
        if (vr == T(0) && vi == T(0)) continue;
        red_add(dst + ix, vr, vi);
      }
    }
    return;
  }
  for (int r = threadIdx.x >> 5; r < rows; r += nwb, rw.next(nwb, st.TY)) {
    const int gy = wrap3(st.oy + rw.iy, g.nf[1]), gz = wrap3(st.oz + rw.iz, g.nf[2]);
    cplx_t<T>* dst = grid + ((size_t)gz * g.nf[1] + gy) * g.nf[0];
    for (int ix = lane; ix < st.TX; ix += 32) {
      const T vr = re[r * pitch + ix], vi = im[r * pitch + ix];
      if (vr == T(0) && vi == T(0)) continue;
      red_add(dst + wrap3(st.ox + ix, g.nf[0]), vr, vi);
    }
  }
}

template <typename T, int DIM, int NS>
__global__ void __launch_bounds__(kSpreadThreads)
k_spread_sm_wc(SpreadArgs<T> a) {
  using C = cplx_t<T>;
  constexpr int HD = horner_degree<T>(NS);
  constexpr int L = spread_lanes<NS>();
  constexpr int PPW = 32 / L;
  constexpr int NY = DIM > 1 ? NS : 1;
  constexpr int NZ = DIM > 2 ? NS : 1;
  if (a.sub_dense && a.sub_dense[blockIdx.x]) return;  // cell-run layout: done by k_spread_sm_run
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const SubTile st = sub_tile_block<DIM, NS>(a.bins, blockIdx.x);
  T* re = reinterpret_cast<T*>(smem_raw);
  T* im = re + st.ntile;
  const int t = blockIdx.y;
  for (int i = threadIdx.x; i < 2 * st.ntile; i += blockDim.x) re[i] = T(0);
  __syncthreads();
  const int lane = threadIdx.x & 31, g = lane / L, j = lane % L;
  const bool tap = j < NS;
  const int jj = tap ? j : 0;
  const int warp = threadIdx.x >> 5, nwb = blockDim.x >> 5;
  const C* cin = a.c_in + (size_t)t * a.M;
  for (int base = warp * PPW; base < st.np; base += nwb * PPW) {
    const int pl = base + g;
    const bool valid = g < PPW && pl < st.np;
    const int p = st.p0 + (valid ? pl : st.np - 1);
    const int lx = a.pts.i0[0][p] - st.ox;
    const T kx = kernel_tap<T, NS, HD>(a.pts.d[0][p], jj, a.kc);
    T ky = T(1), kz = T(1);
    int ly = 0, lz = 0;
    if (DIM > 1) { ly = a.pts.i0[1][p] - st.oy; ky = kernel_tap<T, NS, HD>(a.pts.d[1][p], jj, a.kc); }
    if (DIM > 2) { lz = a.pts.i0[2][p] - st.oz; kz = kernel_tap<T, NS, HD>(a.pts.d[2][p], jj, a.kc); }
    const C v = cin[a.pts.idx[p]];
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
  plane_flush<T>(re, im, a.fw + (size_t)t * a.g.Nf, st, a.g);
}

// ---------------------------------------------------------------------------
// Slab-owned 3D spreading (method 2, the default for sparse 3D subproblems).
// Shared FP32 atomicAdd runs at about a third of the int32 rate and costs
// several shared wavefronts per warp instruction, which bound the
// warp-cooperative kernel.  Here the tile's z-planes are owned: the block has
// NS warps and warp w alone writes the planes z = w (mod NS).  A point's
// support covers NS consecutive planes, one of each residue, so every warp
// handles exactly one plane of every point, and it adds the point's NS x NS
// taps there with plain shared loads and stores of complex cells: lanes over
// (x, y) taps, R = 32 / NS rows per instruction, distinct cells, and a
// __syncwarp between points, which orders one point's stores before the next
// point's loads.  The block stages the kernel values of CH points at a time
// (c kx as complex, ky, kz, the point's tile offset) in a double buffer, one
// block barrier per chunk.  Rows are padded to a pitch PX = NS (mod 16)
// complex cells, so lane l's cell is l (mod 16): the rows of one instruction
// fall in distinct banks.  Results equal the atomic kernels' up to the order
// of additions.
constexpr int kSlabChunk = 64;

__host__ __device__ constexpr int slab_pitch(int tx, int ns) {
  return tx + (((ns - tx) % 16) + 16) % 16;
}

// FP32 kernel rows along y staged in pairs, for widths whose point takes two
// or more row instructions (R = 32 / ns rows each, NR of them): slot
// m R + y holds (ky[2m R + y], ky[(2m + 1) R + y]), so lane (dx, y) reads one
// float2 per two row instructions instead of one float per instruction.
// Point q of a stage of n points sits at slot (n + 1) + q: the R slots one
// instruction reads are 8 (n + 1) bytes apart, two banks apart for n = 32 or
// 64 (distinct banks, one wavefront), and consecutive points are consecutive
// words (conflict-free staging stores).
__host__ __device__ constexpr int ky_rows_per_instr(int ns) { return 32 / ns; }
__host__ __device__ constexpr int ky_instrs(int ns) { return (ns + 32 / ns - 1) / (32 / ns); }
__host__ __device__ constexpr bool ky_paired(int ns, int real_bytes) { return real_bytes == 4 && ky_instrs(ns) >= 2; }
__host__ __device__ constexpr int ky_pair_slots(int ns) { return (ky_instrs(ns) + 1) / 2 * ky_rows_per_instr(ns); }

template <typename T>
size_t slab_bytes(int ns, const BinTables& bt) {
  const size_t px = slab_pitch(bt.bs[0] + ns - 1, ns);
  const size_t cells = px * (bt.bs[1] + ns - 1) * (bt.bs[2] + ns - 1);
  const size_t ky = ky_paired(ns, sizeof(T)) ? (size_t)ky_pair_slots(ns) * (kSlabChunk + 1) * sizeof(float2)
                                             : (size_t)kSlabChunk * ns * sizeof(T);
  const size_t stage = (size_t)kSlabChunk * ns * (sizeof(cplx_t<T>) + sizeof(T)) + ky + kSlabChunk * sizeof(int2);
  return cells * sizeof(cplx_t<T>) + 16 + 2 * stage;  // stage aligned to 16 bytes
}

// Flush of an interleaved complex tile with row pitch `pitch` (cells).
template <typename T>
__device__ __forceinline__ void cplx_flush(const cplx_t<T>* tile, cplx_t<T>* grid, const SubTile& st,
                                           const GridGeom& g, int pitch) {
  const int lane = threadIdx.x & 31, nwb = blockDim.x >> 5;
  const int rows = st.TY * st.TZ;
  TileRows rw(threadIdx.x >> 5, st.TY);
  const bool inside = tile_in_grid(st, g);
  for (int r = threadIdx.x >> 5; r < rows; r += nwb, rw.next(nwb, st.TY)) {
    const int gy = inside ? st.oy + rw.iy : wrap3(st.oy + rw.iy, g.nf[1]);
    const int gz = inside ? st.oz + rw.iz : wrap3(st.oz + rw.iz, g.nf[2]);
    cplx_t<T>* dst = grid + ((size_t)gz * g.nf[1] + gy) * g.nf[0];
    const cplx_t<T>* src = tile + (size_t)r * pitch;
    for (int ix = lane; ix < st.TX; ix += 32) {
      const cplx_t<T> v = src[ix];
      if (v.x == T(0) && v.y == T(0)) continue;
      red_add(dst + (inside ? st.ox + ix : wrap3(st.ox + ix, g.nf[0])), v.x, v.y);
    }
  }
}

template <typename T, int NS>
__global__ void __launch_bounds__(32 * NS)
k_spread_sm_slab(SpreadArgs<T> a, int split) {
  using C = cplx_t<T>;
  constexpr int HD = horner_degree<T>(NS);
  constexpr int R = 32 / NS;                 // tile rows per warp instruction
  constexpr int NR = (NS + R - 1) / R;       // instructions per plane
  constexpr int CH = kSlabChunk;
  constexpr bool kPairs = ky_paired(NS, sizeof(T));
  constexpr int NPR = (NR + 1) / 2;          // ky pairs per lane (kPairs)
  // cell-run layout: a subproblem that starts on a dense cell leaves its
  // leading dense points to k_spread_sm_run (split) or all of them (not)
  int first = 0;
  if (a.sub_dense && a.sub_dense[blockIdx.x]) {
    if (!split) return;
    first = a.sub_ndense[blockIdx.x];
  }
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const SubTile st = sub_tile_block<3, NS>(a.bins, blockIdx.x);
  if (first >= st.np) return;  // block-uniform
  const int PX = slab_pitch(st.TX, NS);
  const int PP = PX * st.TY;                  // plane stride
  const int ncell = PP * st.TZ;
  C* tile = reinterpret_cast<C*>(smem_raw);
  // double-buffered stage: [c kx (complex) | kz] x CH x NS, ky (CH x NS, or
  // in pairs: ky_pair_slots x (CH + 1) float2), then (tile offset, lz mod NS)
  // per point
  unsigned char* stage0 = smem_raw + (((size_t)ncell * sizeof(C) + 15) & ~(size_t)15);
  constexpr size_t kKyBytes =
      kPairs ? (size_t)ky_pair_slots(NS) * (CH + 1) * sizeof(float2) : (size_t)CH * NS * sizeof(T);
  const size_t stage_sz = (size_t)CH * NS * (sizeof(C) + sizeof(T)) + kKyBytes + CH * sizeof(int2);
  const int t = blockIdx.y;
  for (int i = threadIdx.x; i < ncell; i += blockDim.x) tile[i] = C{T(0), T(0)};
  const C* cin = a.c_in + (size_t)t * a.M;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int dx = lane % NS, dyl = lane / NS;
  const bool lane_on = lane < R * NS;
  constexpr bool kFullRows = 32 % NS == 0 && (NS * NS) % 32 == 0;  // ns 8, 16: all lanes, rows in range
  for (int c0 = first, buf = 0; c0 < st.np; c0 += CH, buf ^= 1) {
    unsigned char* sb = stage0 + buf * stage_sz;
    C* s_ck = reinterpret_cast<C*>(sb);
    T* s_kz = reinterpret_cast<T*>(s_ck + CH * NS);
    T* s_ky = s_kz + CH * NS;  // kPairs: float2 slots, see ky_pair_slots
    int2* s_bl = reinterpret_cast<int2*>(reinterpret_cast<unsigned char*>(s_ky) + kKyBytes);
    const int nq = min(CH, st.np - c0);
    for (int i = threadIdx.x; i < nq * NS; i += blockDim.x) {
      const int q = i / NS, j = i - q * NS;
      const int p = st.p0 + c0 + q;
      const C v = cin[a.pts.idx[p]];
      const T kx = kernel_tap<T, NS, HD>(a.pts.d[0][p], j, a.kc);
      s_ck[i] = C{v.x * kx, v.y * kx};
      const T kyj = kernel_tap<T, NS, HD>(a.pts.d[1][p], j, a.kc);
      if constexpr (kPairs) {
        const int r = j / R, y = j - r * R;  // row instruction and lane row of tap j
        s_ky[(((r >> 1) * R + y) * (CH + 1) + q) * 2 + (r & 1)] = kyj;
      } else {
        s_ky[i] = kyj;
      }
      s_kz[i] = kernel_tap<T, NS, HD>(a.pts.d[2][p], j, a.kc);
      if (j == 0) {
        const int lx = a.pts.i0[0][p] - st.ox, ly = a.pts.i0[1][p] - st.oy, lz = a.pts.i0[2][p] - st.oz;
        s_bl[q] = make_int2((lz * st.TY + ly) * PX + lx, lz % NS);
      }
    }
    __syncthreads();  // (also: the tile is zeroed; the other buffer is free)
    for (int q = 0; q < nq; ++q) {
      const int2 bl = s_bl[q];
      int dz = warp - bl.y;
      dz += dz < 0 ? NS : 0;                  // the plane of residue `warp`
      const T kz = s_kz[q * NS + dz];
      const C ck = s_ck[q * NS + dx];
      const T ur = ck.x * kz, ui = ck.y * kz;
      const int base = bl.x + dz * PP + dx;
      T ky[NR];
      if constexpr (kPairs) {
        const float2* kp = reinterpret_cast<const float2*>(s_ky) + min(dyl, R - 1) * (CH + 1) + q;
#pragma unroll
        for (int m = 0; m < NPR; ++m) {
          const float2 v = kp[m * R * (CH + 1)];
          ky[2 * m] = v.x;
          if (2 * m + 1 < NR) ky[2 * m + 1] = v.y;
        }
      } else {
#pragma unroll
        for (int r = 0; r < NR; ++r) ky[r] = s_ky[q * NS + min(r * R + dyl, NS - 1)];
      }
#pragma unroll
      for (int r = 0; r < NR; ++r) {
        const int dy = r * R + dyl;
        if (kFullRows || (lane_on && dy < NS)) {
          C v = tile[base + dy * PX];
          v.x = fma_rn(ur, ky[r], v.x);
          v.y = fma_rn(ui, ky[r], v.y);
          tile[base + dy * PX] = v;
        }
      }
      __syncwarp();  // this point's stores before the next point's loads
    }
  }
  __syncthreads();
  cplx_flush<T>(tile, a.fw + (size_t)t * a.g.Nf, st, a.g, PX);
}

// ---------------------------------------------------------------------------
// Private-tile 2D spreading (method 2, the default for 2D subproblems).  A 2D
// tile is small (39 x 40 cells at ns 8 with 32 x 32 bins), so each of the
// block's kPrivWarps warps accumulates its share of the subproblem's points
// into a private copy of complex cells with plain shared loads and stores --
// lanes over the point's (x, y) taps, 32 / NS rows per instruction, a
// __syncwarp between points -- and the copies are summed cell by cell once at
// the end (one thread per cell, no atomics) and flushed.  Each warp stages
// the kernel rows of 32 points at a time in warp-private shared memory (c kx
// as complex, ky, the tile offset): lane q evaluates point q's rows.  Rows
// are padded to the slab kernel's pitch (NS mod 16 cells), so the rows of one
// instruction fall in distinct banks.  Results equal the atomic kernel's up
// to the order of additions.
constexpr int kPrivWarps = 4;

// Bytes of one warp's stage: c kx (complex), ky (32 x ns, or in pairs:
// ky_pair_slots x 33 float2), the tile offset.
__host__ __device__ constexpr size_t priv_stage_bytes(int ns, int real_bytes) {
  return (32 * (size_t)ns * 2 * real_bytes +
          (ky_paired(ns, real_bytes) ? (size_t)ky_pair_slots(ns) * 33 * 8 : 32 * (size_t)ns * real_bytes) +
          32 * sizeof(int) + 15) &
         ~(size_t)15;
}

template <typename T>
size_t priv_bytes(int ns, const BinTables& bt) {
  const size_t px = slab_pitch(bt.bs[0] + ns - 1, ns);
  const size_t copy = px * (bt.bs[1] + ns - 1) * sizeof(cplx_t<T>);
  return kPrivWarps * (((copy + 15) & ~(size_t)15) + priv_stage_bytes(ns, sizeof(T)));
}

template <typename T, int NS>
__global__ void __launch_bounds__(32 * kPrivWarps)
k_spread_sm_priv(SpreadArgs<T> a, int split) {
  using C = cplx_t<T>;
  constexpr int R = 32 / NS;                 // tile rows per warp instruction
  constexpr int NR = (NS + R - 1) / R;       // instructions per point
  constexpr int HD = horner_degree<T>(NS);
  constexpr bool kPairs = ky_paired(NS, sizeof(T));
  constexpr int NPR = (NR + 1) / 2;          // ky pairs per lane (kPairs)
  int first = 0;
  if (a.sub_dense && a.sub_dense[blockIdx.x]) {  // cell-run layout: dense prefixes by k_spread_sm_run
    if (!split) return;
    first = a.sub_ndense[blockIdx.x];
  }
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const SubTile st = sub_tile_block<2, NS>(a.bins, blockIdx.x);
  if (first >= st.np) return;  // block-uniform
  const int PX = slab_pitch(st.TX, NS);
  const int ncell = PX * st.TY;
  const size_t copy_sz = ((size_t)ncell * sizeof(C) + 15) & ~(size_t)15;
  constexpr size_t stage_sz = priv_stage_bytes(NS, sizeof(T));
  constexpr size_t kKyBytes = kPairs ? (size_t)ky_pair_slots(NS) * 33 * sizeof(float2) : (size_t)32 * NS * sizeof(T);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  C* tile = reinterpret_cast<C*>(smem_raw + warp * copy_sz);
  unsigned char* sb = smem_raw + kPrivWarps * copy_sz + warp * stage_sz;
  C* s_ck = reinterpret_cast<C*>(sb);
  T* s_ky = reinterpret_cast<T*>(s_ck + 32 * NS);  // kPairs: float2 slots, see ky_pair_slots
  int* s_base = reinterpret_cast<int*>(reinterpret_cast<unsigned char*>(s_ky) + kKyBytes);
  for (int i = lane; i < ncell; i += 32) tile[i] = C{T(0), T(0)};
  const int t = blockIdx.y;
  const C* cin = a.c_in + (size_t)t * a.M;
  const int dx = lane % NS, dyl = lane / NS;
  const bool lane_on = lane < R * NS;
  constexpr bool kFullRows = 32 % NS == 0 && (NS * NS) % 32 == 0;  // ns 8, 16: all lanes, rows in range
  // warp w takes points first + [w S, (w + 1) S) of the subproblem
  const int npts = st.np - first;
  const int S = (npts + kPrivWarps - 1) / kPrivWarps;
  const int beg = first + warp * S, end = min(st.np, beg + S);
  // lane q holds point q of the next chunk in registers (loaded while the
  // current chunk's points are added), then stages its kernel rows
  T d0 = T(0), d1 = T(0);
  int i00 = 0, i01 = 0;
  C cv = C{T(0), T(0)};
  auto load_pt = [&](int c0) {
    if (c0 + lane < end) {
      const int p = st.p0 + c0 + lane;
      d0 = a.pts.d[0][p];
      d1 = a.pts.d[1][p];
      i00 = a.pts.i0[0][p];
      i01 = a.pts.i0[1][p];
      cv = cin[a.pts.idx[p]];
    }
  };
  if (beg < end) load_pt(beg);
  for (int c0 = beg; c0 < end; c0 += 32) {
    const int nq = min(32, end - c0);
    __syncwarp();  // the previous chunk's reads of the stage are done
    if (lane < nq) {
      T kr[NS];
      kernel_row<T, NS, HD>(d0, a.kc, kr);
#pragma unroll
      for (int j = 0; j < NS; ++j) s_ck[lane * NS + j] = C{cv.x * kr[j], cv.y * kr[j]};
      kernel_row<T, NS, HD>(d1, a.kc, kr);
      if constexpr (kPairs) {
        float2* kp = reinterpret_cast<float2*>(s_ky) + lane;
#pragma unroll
        for (int m = 0; m < NPR; ++m)
#pragma unroll
          for (int y = 0; y < R; ++y) {
            const int j0 = 2 * m * R + y, j1 = j0 + R;
            kp[(m * R + y) * 33] = make_float2(j0 < NS ? kr[j0] : 0.f, j1 < NS ? kr[j1] : 0.f);
          }
      } else {
#pragma unroll
        for (int j = 0; j < NS; ++j) s_ky[lane * NS + j] = kr[j];
      }
      s_base[lane] = (i01 - st.oy) * PX + (i00 - st.ox);
    }
    if (c0 + 32 < end) load_pt(c0 + 32);
    __syncwarp();
    // the next point's staged values are read while this point's cells are
    // read, added to and written
    // lane (dx, dyl)'s y rows of point q: one float2 per pair of row
    // instructions (kPairs), else one value per instruction
    auto load_ky = [&](int q, T* ky) {
      if constexpr (kPairs) {
        const float2* kp = reinterpret_cast<const float2*>(s_ky) + min(dyl, R - 1) * 33 + q;
#pragma unroll
        for (int m = 0; m < NPR; ++m) {
          const float2 v = kp[m * R * 33];
          ky[2 * m] = v.x;
          if (2 * m + 1 < NR) ky[2 * m + 1] = v.y;
        }
      } else {
#pragma unroll
        for (int r = 0; r < NR; ++r) ky[r] = s_ky[q * NS + min(r * R + dyl, NS - 1)];
      }
    };
    C ck = s_ck[dx];
    int base = s_base[0] + dx;
    T ky[NR];
    load_ky(0, ky);
    for (int q = 0; q < nq; ++q) {
      const int qn = min(q + 1, nq - 1);
      const C ckn = s_ck[qn * NS + dx];
      const int basen = s_base[qn] + dx;
      T kyn[NR];
      load_ky(qn, kyn);
#pragma unroll
      for (int r = 0; r < NR; ++r) {
        const int dy = r * R + dyl;
        if (kFullRows || (lane_on && dy < NS)) {
          C v = tile[base + dy * PX];
          v.x = fma_rn(ck.x, ky[r], v.x);
          v.y = fma_rn(ck.y, ky[r], v.y);
          tile[base + dy * PX] = v;
        }
      }
      __syncwarp();  // this point's stores before the next point's loads
      ck = ckn;
      base = basen;
#pragma unroll
      for (int r = 0; r < NR; ++r) ky[r] = kyn[r];
    }
  }
  __syncthreads();
  // sum the private copies into copy 0, one thread per cell
  C* tile0 = reinterpret_cast<C*>(smem_raw);
  for (int i = threadIdx.x; i < ncell; i += blockDim.x) {
    C sum = tile0[i];
#pragma unroll
    for (int w = 1; w < kPrivWarps; ++w) {
      const C v = reinterpret_cast<const C*>(smem_raw + w * copy_sz)[i];
      sum.x += v.x;
      sum.y += v.y;
    }
    tile0[i] = sum;
  }
  __syncthreads();
  cplx_flush<T>(tile0, a.fw + (size_t)t * a.g.Nf, st, a.g, PX);
}

// CUFINUFFT_SPREAD_PRIV=0: 2D subproblem spreading by the warp-cooperative
// atomic kernel instead of the private-tile one.
inline bool priv_spread_enabled() {
  const char* v = std::getenv("CUFINUFFT_SPREAD_PRIV");
  return !(v && v[0] == '0');
}

// CUFINUFFT_SPREAD_SLAB=0: 3D subproblem spreading by the warp-cooperative
// atomic kernel instead of the slab-owned one.
inline bool slab_spread_enabled() {
  const char* v = std::getenv("CUFINUFFT_SPREAD_SLAB");
  return !(v && v[0] == '0');
}

// ---------------------------------------------------------------------------
// Cell-run spreading (method 2 over cell-ordered points, a layout class of
// its own).  setpts sorts a bin's points by first-tap cell, so dense regions
// arrive as long runs of points that all add into the same ns^d cells.  A
// warp walks its slice of the subproblem in chunks of 32 points.  A chunk
// whose points share one cell is summed in registers -- in 3D (ns >= 5)
// lane (x, y0) owns the taps (x, y0 + m 32/ns, z) for every z, otherwise
// lane l takes the taps l, l + 32, ..., four at a time -- from the points'
// kernel values staged in warp-private shared memory, then each tap sum is
// added to the tile once (conflict-free: the lanes' taps differ).  Any other
// chunk is spread point by point with shared atomics, lanes over x taps as
// in k_spread_sm_wc.  Dense chunks thus cost FMAs instead of 2 ns^d
// same-address atomics per point.  Taps per point <= 512.  Subproblems that
// start on a sparse cell, and (split) the sparse tails of the others, are
// left to the sparse kernel launched beside this one (slab-owned in 3D,
// private-tile in 2D, warp-cooperative otherwise).
template <int DIM, int NS> constexpr int run_taps() {
  return DIM == 1 ? NS : (DIM == 2 ? NS * NS : NS * NS * NS);
}
template <int DIM, int NS> constexpr bool run_ok() { return run_taps<DIM, NS>() <= 512; }

// One subproblem of the cell-run spread into the zeroed tile planes re/im
// (shared by the per-plan and the multi-plan kernels): krow(d, out) writes a
// point's NS kernel values along one axis, ktap(d, j) returns one of them.
template <typename T, int DIM, int NS, class KRow, class KTap>
__device__ __forceinline__ void run_subproblem(const SubTile& st, T* re, T* im, const SortedPts<T>& pts,
                                               const cplx_t<T>* cin, KRow krow, KTap ktap,
                                               int nd = 0) {
  using C = cplx_t<T>;
  constexpr int NT = run_taps<DIM, NS>();
  constexpr int KV = DIM * NS;
  constexpr int NWARP = kSpreadThreads / 32;
  constexpr int GK = 4;                            // taps per lane per pass over a chunk
  constexpr int NPASS = (NT + 32 * GK - 1) / (32 * GK);
  constexpr int L = spread_lanes<NS>();
  constexpr int PPW = 32 / L;
  constexpr int NY = DIM > 1 ? NS : 1;
  constexpr int NZ = DIM > 2 ? NS : 1;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T* kvw = im + st.ntile + warp * 32 * KV;  // staged kernel values of a dense chunk
  C* cvw = reinterpret_cast<C*>(im + st.ntile + NWARP * 32 * KV) + warp * 32;
  for (int i = threadIdx.x; i < 2 * st.ntile; i += blockDim.x) re[i] = T(0);
  __syncthreads();
  const int S = (((st.np + NWARP - 1) / NWARP) + 31) & ~31;
  const int beg = warp * S;
  const int end = min(st.np, beg + S);
  // The cursor follows the runs: a window of 32 points whose leading run
  // (points on the window's first cell) has at least dense_run(DIM) points is
  // accumulated -- the run's first n <= 32 points -- and the cursor moves by
  // n, so the next window starts at a run boundary; any other window is
  // spread point by point and the cursor moves by 32.  Inside the
  // subproblem's dense prefix (its first nd points, every cell a run) a
  // leading run of at least 4 points is accumulated too, and a shorter one
  // (a run's remainder) is spread point by point alone: there the cursor
  // never leaves a run boundary.
  int cs = beg;
  while (cs < end) {  // warp-uniform
    const bool in_prefix = cs < nd;
    const int kMinRun = in_prefix ? 4 : dense_run(DIM);
    const int ql = cs + lane;
    const bool valid = ql < end;
    const int p = st.p0 + (valid ? ql : cs);
    const int lx = pts.i0[0][p] - st.ox;
    const int ly = DIM > 1 ? pts.i0[1][p] - st.oy : 0;
    const int lz = DIM > 2 ? pts.i0[2][p] - st.oz : 0;
    const int key = lx + st.TX * (ly + st.TY * lz);
    const int key0 = __shfl_sync(0xffffffffu, key, 0);
    const unsigned same = __ballot_sync(0xffffffffu, valid && key == key0);
    const int nrun = same == 0xffffffffu ? 32 : __ffs(~same) - 1;  // leading run length
    if (nrun >= kMinRun) {
      // run chunk: stage the first nrun points' kernel values, then every
      // lane sums its taps over them, GK taps per pass, one add per tap
      T kr[NS];
      T* kv = kvw + lane * KV;
      krow(pts.d[0][p], kr);
#pragma unroll
      for (int j = 0; j < NS; ++j) kv[j] = kr[j];
      if (DIM > 1) {
        krow(pts.d[1][p], kr);
#pragma unroll
        for (int j = 0; j < NS; ++j) kv[NS + j] = kr[j];
      }
      if (DIM > 2) {
        krow(pts.d[2][p], kr);
#pragma unroll
        for (int j = 0; j < NS; ++j) kv[2 * NS + j] = kr[j];
      }
      cvw[lane] = cin[pts.idx[p]];
      __syncwarp();
      if constexpr (DIM == 3 && NS >= 5) {
        // factorised: lane (ix, iy0) owns the taps (ix, iy0 + m R3, iz) for
        // all iz; per point it reads c, kx[ix], its ky values and the ns kz
        // values (broadcast), and adds (c kx ky) kz to NR3 x NS sums
        constexpr int R3 = 32 / NS, NR3 = (NS + R3 - 1) / R3;
        const int fx = lane % NS, fy = lane / NS;
        T accr[NR3][NS], acci[NR3][NS];
#pragma unroll
        for (int m = 0; m < NR3; ++m)
#pragma unroll
          for (int iz = 0; iz < NS; ++iz) accr[m][iz] = acci[m][iz] = T(0);
#pragma unroll 2
        for (int q = 0; q < nrun; ++q) {
          const T* kq = kvw + q * KV;
          const C cq = cvw[q];
          const T kxv = kq[fx];
          const T cr = cq.x * kxv, ci = cq.y * kxv;
          T kzv[NS];
#pragma unroll
          for (int iz = 0; iz < NS; ++iz) kzv[iz] = kq[2 * NS + iz];
#pragma unroll
          for (int m = 0; m < NR3; ++m) {
            const T kyv = kq[NS + min(fy + m * R3, NS - 1)];
            const T wr = cr * kyv, wi = ci * kyv;
#pragma unroll
            for (int iz = 0; iz < NS; ++iz) {
              accr[m][iz] = fma_rn(wr, kzv[iz], accr[m][iz]);
              acci[m][iz] = fma_rn(wi, kzv[iz], acci[m][iz]);
            }
          }
        }
        if (lane < R3 * NS) {
#pragma unroll
          for (int m = 0; m < NR3; ++m) {
            const int iy = fy + m * R3;
            if (iy < NS) {
#pragma unroll
              for (int iz = 0; iz < NS; ++iz) {
                const int off = key0 + fx + st.TX * (iy + st.TY * iz);
                atomicAdd(re + off, accr[m][iz]);
                atomicAdd(im + off, acci[m][iz]);
              }
            }
          }
        }
        __syncwarp();  // the staging area is rewritten by the next chunk
        cs += nrun;
        continue;
      }
#pragma unroll 1
      for (int pass = 0; pass < NPASS; ++pass) {
        int ix[GK], iy[GK], iz[GK];
        bool on[GK];
        T ar[GK], ai[GK];
#pragma unroll
        for (int k = 0; k < GK; ++k) {
          const int tt = lane + 32 * (pass * GK + k);
          on[k] = tt < NT;
          ix[k] = tt % NS;
          iy[k] = NS + (tt / NS) % NS;
          iz[k] = 2 * NS + tt / (NS * NS);
          ar[k] = T(0);
          ai[k] = T(0);
        }
#pragma unroll 4
        for (int q = 0; q < nrun; ++q) {
          const T* kq = kvw + q * KV;
          const C cq = cvw[q];
#pragma unroll
          for (int k = 0; k < GK; ++k) {
            T wgt = kq[on[k] ? ix[k] : 0];
            if (DIM > 1) wgt *= kq[on[k] ? iy[k] : 0];
            if (DIM > 2) wgt *= kq[on[k] ? iz[k] : 0];
            ar[k] = fma_rn(cq.x, wgt, ar[k]);
            ai[k] = fma_rn(cq.y, wgt, ai[k]);
          }
        }
#pragma unroll
        for (int k = 0; k < GK; ++k) {
          if (on[k]) {
            const int off = key0 + (ix[k] + st.TX * ((iy[k] - NS) + st.TY * (iz[k] - 2 * NS)));
            atomicAdd(re + off, ar[k]);
            atomicAdd(im + off, ai[k]);
          }
        }
      }
      __syncwarp();  // the staging area is rewritten by the next chunk
      cs += nrun;
    } else {
      const int g = lane / L, j = lane % L;
      const bool tap = j < NS;
      const int jj = tap ? j : 0;
      const int lim = in_prefix ? nrun : 32;  // points of this window
      // cell-ordered neighbours overlap: group g takes points it + g * NIT,
      // so the PPW points of one warp instruction lie far apart in the chunk
      const int NIT = (lim + PPW - 1) / PPW;
      for (int it = 0; it < NIT; ++it) {  // warp-uniform
        const int qq = it + g * NIT;
        const bool v2 = g < PPW && qq < lim && cs + qq < end;
        const int p2 = st.p0 + (v2 ? cs + qq : cs);
        const int lx2 = pts.i0[0][p2] - st.ox;
        const T kx = ktap(pts.d[0][p2], jj);
        T ky = T(1), kz = T(1);
        int ly2 = 0, lz2 = 0;
        if (DIM > 1) { ly2 = pts.i0[1][p2] - st.oy; ky = ktap(pts.d[1][p2], jj); }
        if (DIM > 2) { lz2 = pts.i0[2][p2] - st.oz; kz = ktap(pts.d[2][p2], jj); }
        const C v = cin[pts.idx[p2]];
        const T vr = v.x * kx, vi = v.y * kx;
        const int off0 = (lz2 * st.TY + ly2) * st.TX + lx2 + jj;
#pragma unroll 1
        for (int dz = 0; dz < NZ; ++dz) {
          const T kzv = DIM > 2 ? __shfl_sync(0xffffffffu, kz, g * L + dz) : T(1);
#pragma unroll
          for (int dy = 0; dy < NY; ++dy) {
            const T kyv = DIM > 1 ? __shfl_sync(0xffffffffu, ky, g * L + dy) : T(1);
            const T w = kyv * kzv;
            if (tap && v2) {
              const int off = off0 + (dz * st.TY + dy) * st.TX;
              atomicAdd(re + off, vr * w);
              atomicAdd(im + off, vi * w);
            }
          }
        }
      }
      cs += lim;
    }
  }
}

template <typename T, int DIM, int NS>
__global__ void __launch_bounds__(kSpreadThreads)
k_spread_sm_run(SpreadArgs<T> a, int split) {
  constexpr int HD = horner_degree<T>(NS);
  if (a.sub_dense && !a.sub_dense[blockIdx.x]) return;  // sparse: done by k_spread_sm_wc / slab
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SubTile st = sub_tile_block<DIM, NS>(a.bins, blockIdx.x);
  const int nd = a.sub_ndense ? a.sub_ndense[blockIdx.x] : 0;  // leading dense points
  if (split) st.np = nd;  // the rest: k_spread_sm_slab
  T* re = reinterpret_cast<T*>(smem_raw);
  T* im = re + st.ntile;
  const int t = blockIdx.y;
  for (int i = threadIdx.x; i < 2 * st.ntile; i += blockDim.x) re[i] = T(0);
  __syncthreads();
  const KernelCoeffs<T>& kc = a.kc;
  run_subproblem<T, DIM, NS>(
      st, re, im, a.pts, a.c_in + (size_t)t * a.M,
      [&](T dv, T* out) { kernel_row<T, NS, HD>(dv, kc, out); },
      [&](T dv, int j) { return kernel_tap<T, NS, HD>(dv, j, kc); }, nd);
  __syncthreads();
  plane_flush<T>(re, im, a.fw + (size_t)t * a.g.Nf, st, a.g);
}

// Shared memory of the cell-run kernel: the tile planes, the staged kernel
// values and the strengths of every warp's dense chunk.
template <typename T, int DIM>
size_t run_bytes(int ns, const BinTables& bt) {
  const size_t nw = kSpreadThreads / 32;
  return tile_cells(DIM, ns, bt.bs) * 2 * sizeof(T) + nw * 32 * (size_t)(DIM * ns) * sizeof(T) +
         nw * 32 * sizeof(cplx_t<T>);
}

// ---------------------------------------------------------------------------
// Tensor-core cell-run spreading (3D FP32, ns <= 8; CUFINUFFT_TC_SPREAD=1).
// A chunk of n <= 32 points on one cell adds, to the cell's ns^3 taps,
//   S[ix][iy][iz] = sum_q (c_q kx_q[ix]) (ky_q[iy] kz_q[iz]),
// a product D = A B^T with A[m][q] = ky_q[iy] kz_q[iz] (m = iy + ns iz,
// M = 128 rows, ns^2 used) and B[n][q] = kx_q[ix] Re/Im(c_q) (n = 2 ix + re/im,
// N = 16): tcgen05.mma kind::tf32 with K = 8 points per instruction, each
// operand split into a TF32 part and its FP32 remainder (hi hi + hi lo + lo
// hi, FP32 accumulation in tensor memory), the accumulator read back by the
// first warpgroup and added to the tile planes.  The CTA walks the
// subproblem's dense prefix chunk by chunk (a chunk opens a cell whose
// first 32-point window runs at least dense_run(3) points, or continues the
// previous chunk's cell); the points after it are spread point by point as
// in k_spread_sm_wc.
constexpr int kTcK = 32;                   // points per chunk (4 MMA K-steps)
constexpr int kTcWaitPolls = 1 << 22;      // bounded waits on the MMA barrier

__host__ __device__ constexpr size_t tc_operand_floats() {
  return 2 * (kTcK / 8) * 1024 + 2 * (kTcK / 8) * 128;  // A hi/lo, B hi/lo
}
template <int NS>
__host__ __device__ constexpr size_t tc_stage_floats() {
  return (size_t)kTcK * 3 * NS + 2 * kTcK;  // kernel rows, strengths
}
inline size_t tc_run_bytes(int ns, const BinTables& bt) {
  return (tc_operand_floats() + (size_t)kTcK * 3 * ns + 2 * kTcK + 2 * tile_cells(3, ns, bt.bs)) * sizeof(float);
}

template <int NS>
__global__ void __launch_bounds__(kSpreadThreads)
k_spread_sm_run_tc(SpreadArgs<float> a) {
  constexpr int HD = horner_degree<float>(NS);
  constexpr int KV = 3 * NS;
  if (a.sub_dense && !a.sub_dense[blockIdx.x]) return;  // sparse: done by k_spread_sm_wc
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ __align__(8) unsigned long long bar;
  __shared__ unsigned tmem_base;
  __shared__ int s_n, s_key;
  const SubTile st = sub_tile_block<3, NS>(a.bins, blockIdx.x);
  float* A_hi = reinterpret_cast<float*>(smem_raw);
  float* A_lo = A_hi + (kTcK / 8) * 1024;
  float* B_hi = A_lo + (kTcK / 8) * 1024;
  float* B_lo = B_hi + (kTcK / 8) * 128;
  float* kv = B_lo + (kTcK / 8) * 128;                 // [kTcK][3 NS]
  float2* cv = reinterpret_cast<float2*>(kv + kTcK * KV);  // [kTcK]
  float* re = reinterpret_cast<float*>(cv + kTcK);
  float* im = re + st.ntile;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int t = blockIdx.y;
  const float2* cin = a.c_in + (size_t)t * a.M;
  for (int i = tid; i < 2 * st.ntile; i += blockDim.x) re[i] = 0.f;
  // rows NS^2 .. 127 of A stay zero for every chunk: written once
  for (int e = tid; e < (128 - NS * NS) * kTcK; e += blockDim.x) {
    const int m = NS * NS + e % (128 - NS * NS), q = e / (128 - NS * NS);
    const int off = (q >> 3) * 1024 + umma_kmaj_off(m, q & 7);
    A_hi[off] = 0.f;
    A_lo[off] = 0.f;
  }
  if (tid == 0) mbar_init(&bar, 1);
  if (warp == 0) tmem_alloc(&tmem_base, 32);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const unsigned taddr = tmem_base;
  constexpr unsigned idesc = umma_idesc_tf32(128, 16);
  constexpr int kMinRun = dense_run(3);
  int cs = 0, prev_key = -1;
  unsigned phase = 0;
  bool healthy = true;
  while (healthy) {  // block-uniform
    if (warp == 0) {
      const int q = cs + lane;
      const bool valid = q < st.np;
      int key = -1;
      if (valid) {
        const int p = st.p0 + q;
        key = (a.pts.i0[0][p] - st.ox) + st.TX * ((a.pts.i0[1][p] - st.oy) + st.TY * (a.pts.i0[2][p] - st.oz));
      }
      const int key0 = __shfl_sync(0xffffffffu, key, 0);
      const unsigned same = __ballot_sync(0xffffffffu, valid && key == key0);
      const int nrun = same == 0xffffffffu ? 32 : __ffs(~same) - 1;
      const bool dense = cs < st.np && (nrun >= kMinRun || key0 == prev_key);
      if (lane == 0) {
        s_n = dense ? nrun : 0;
        s_key = key0;
      }
    }
    __syncthreads();
    const int n = s_n, key0 = s_key;
    if (n == 0) break;
    // the chunk's kernel values (one tap per thread) and strengths
    for (int e = tid; e < n * KV; e += blockDim.x) {
      const int q = e / KV, r = e - q * KV;
      const int p = st.p0 + cs + q;
      kv[e] = kernel_tap<float, NS, HD>(a.pts.d[r / NS][p], r % NS, a.kc);
    }
    if (tid < n) cv[tid] = cin[a.pts.idx[st.p0 + cs + tid]];
    __syncthreads();
    // operands, K padded to kTcK with zero points (rows >= NS^2 are zero)
    for (int e = tid; e < NS * NS * kTcK; e += blockDim.x) {
      const int m = e % (NS * NS), q = e / (NS * NS);
      float v = 0.f;
      if (q < n) v = kv[q * KV + NS + m % NS] * kv[q * KV + 2 * NS + m / NS];
      float hi, lo;
      tf32_split(v, hi, lo);
      const int off = (q >> 3) * 1024 + umma_kmaj_off(m, q & 7);
      A_hi[off] = hi;
      A_lo[off] = lo;
    }
    for (int e = tid; e < 16 * kTcK; e += blockDim.x) {
      const int nn = e & 15, q = e >> 4;
      const int ix = nn >> 1;
      float v = 0.f;
      if (ix < NS && q < n) v = kv[q * KV + ix] * ((nn & 1) ? cv[q].y : cv[q].x);
      float hi, lo;
      tf32_split(v, hi, lo);
      const int off = (q >> 3) * 128 + umma_kmaj_off(nn, q & 7);
      B_hi[off] = hi;
      B_lo[off] = lo;
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    if (tid == 0) {
      tc_fence_after();
      const int ksteps = (n + 7) >> 3;
      for (int s = 0; s < ksteps; ++s) {
        const uint64_t ah = umma_sdesc(A_hi + s * 1024, kUmmaLbo, kUmmaSbo);
        const uint64_t al = umma_sdesc(A_lo + s * 1024, kUmmaLbo, kUmmaSbo);
        const uint64_t bh = umma_sdesc(B_hi + s * 128, kUmmaLbo, kUmmaSbo);
        const uint64_t bl = umma_sdesc(B_lo + s * 128, kUmmaLbo, kUmmaSbo);
        umma_tf32(taddr, ah, bh, idesc, s > 0 ? 1u : 0u);
        umma_tf32(taddr, ah, bl, idesc, 1u);
        umma_tf32(taddr, al, bh, idesc, 1u);
      }
      umma_commit(&bar);
    }
    bool done = mbar_wait(&bar, phase, kTcWaitPolls);
    if (!done) {
      // record the stall; wait again (bounded) so no MMA is in flight when
      // the tile or tensor memory is reused or freed
      status_set(a.status, 0);
      done = mbar_wait(&bar, phase, kTcWaitPolls);
      if (!done) status_set(a.status, 1);
    }
    phase ^= 1u;
    healthy = __syncthreads_and(done ? 1 : 0) != 0;
    tc_fence_after();
    if (healthy && warp < 4) {
      float d[16];
      tmem_ld16(taddr + ((unsigned)(32 * warp) << 16), d);
      const int m = 32 * warp + lane;
      if (m < NS * NS) {
        const int base = key0 + st.TX * ((m % NS) + st.TY * (m / NS));
#pragma unroll
        for (int ix = 0; ix < NS; ++ix) {
          re[base + ix] += d[2 * ix];
          im[base + ix] += d[2 * ix + 1];
        }
      }
    }
    tc_fence_before();
    __syncthreads();
    prev_key = key0;
    cs += n;
  }
  // the points after the dense prefix, one at a time (lanes over x taps)
  {
    constexpr int L = spread_lanes<NS>();
    constexpr int PPW = 32 / L;
    const int g = lane / L, j = lane % L;
    const bool tap = j < NS;
    const int jj = tap ? j : 0;
    const int nwb = blockDim.x >> 5;
    for (int base = cs + warp * PPW; base < st.np; base += nwb * PPW) {
      const int pl = base + g;
      const bool valid = g < PPW && pl < st.np;
      const int p = st.p0 + (valid ? pl : st.np - 1);
      const int lx = a.pts.i0[0][p] - st.ox, ly = a.pts.i0[1][p] - st.oy, lz = a.pts.i0[2][p] - st.oz;
      const float kx = kernel_tap<float, NS, HD>(a.pts.d[0][p], jj, a.kc);
      const float ky = kernel_tap<float, NS, HD>(a.pts.d[1][p], jj, a.kc);
      const float kz = kernel_tap<float, NS, HD>(a.pts.d[2][p], jj, a.kc);
      const float2 v = cin[a.pts.idx[p]];
      const float vr = v.x * kx, vi = v.y * kx;
      const int off0 = (lz * st.TY + ly) * st.TX + lx + jj;
#pragma unroll 1
      for (int dz = 0; dz < NS; ++dz) {
        const float kzv = __shfl_sync(0xffffffffu, kz, g * L + dz);
#pragma unroll
        for (int dy = 0; dy < NS; ++dy) {
          const float w = __shfl_sync(0xffffffffu, ky, g * L + dy) * kzv;
          if (tap && valid) {
            const int off = off0 + (dz * st.TY + dy) * st.TX;
            atomicAdd(re + off, vr * w);
            atomicAdd(im + off, vi * w);
          }
        }
      }
    }
  }
  __syncthreads();
  plane_flush<float>(re, im, a.fw + (size_t)t * a.g.Nf, st, a.g);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) tmem_dealloc(taddr, 32);
}

template <typename T, int DIM, int NS>
__global__ void __launch_bounds__(kSpreadThreads)
k_interp_sm_wc(SpreadArgs<T> a) {
  using C = cplx_t<T>;
  constexpr int HD = horner_degree<T>(NS);
  constexpr int L = lanes_per_point<NS>();
  constexpr int PPW = 32 / L;
  constexpr int NY = DIM > 1 ? NS : 1;
  constexpr int NZ = DIM > 2 ? NS : 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* tile = reinterpret_cast<C*>(smem_raw);
  const SubTile st = sub_tile_block<DIM, NS>(a.bins, blockIdx.x);
  const int t = blockIdx.y;
  tile_load<T>(tile, a.fw_in + (size_t)t * a.g.Nf, st, a.g);
  __syncthreads();
  const int lane = threadIdx.x & 31, g = lane / L, j = lane % L;
  const bool tap = j < NS;
  const int jj = tap ? j : 0;
  const int warp = threadIdx.x >> 5, nwb = blockDim.x >> 5;
  for (int base = warp * PPW; base < st.np; base += nwb * PPW) {
    const int pl = base + g;
    const bool valid = pl < st.np;
    const int p = st.p0 + (valid ? pl : st.np - 1);
    const int lx = a.pts.i0[0][p] - st.ox;
    const T kx = kernel_tap<T, NS, HD>(a.pts.d[0][p], jj, a.kc);
    T ky = T(1), kz = T(1);
    int ly = 0, lz = 0;
    if (DIM > 1) { ly = a.pts.i0[1][p] - st.oy; ky = kernel_tap<T, NS, HD>(a.pts.d[1][p], jj, a.kc); }
    if (DIM > 2) { lz = a.pts.i0[2][p] - st.oz; kz = kernel_tap<T, NS, HD>(a.pts.d[2][p], jj, a.kc); }
    const C* row0 = tile + (lz * st.TY + ly) * st.TX + lx + jj;
    T ar = T(0), ai = T(0);
#pragma unroll 1
    for (int dz = 0; dz < NZ; ++dz) {
      const T kzv = DIM > 2 ? __shfl_sync(0xffffffffu, kz, g * L + dz) : T(1);
#pragma unroll
      for (int dy = 0; dy < NY; ++dy) {
        const T kyv = DIM > 1 ? __shfl_sync(0xffffffffu, ky, g * L + dy) : T(1);
        if (tap) {
          const C v = row0[(dz * st.TY + dy) * st.TX];
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
      a.c_out[(size_t)t * a.M + a.pts.idx[p]] = o;
    }
  }
}

// ---------------------------------------------------------------------------
// Launchers, instantiated per (T, DIM) in si_*.cu.

inline int grid_for(long long n, int threads) {
  long long b = (n + threads - 1) / threads;
  const long long cap = 152LL * 32;  // grid-stride beyond this
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (int)b;
}

template <typename T, int DIM>
size_t tile_bytes(int ns, const BinTables& bt) {
  return tile_cells(DIM, ns, bt.bs) * sizeof(cplx_t<T>);
}

template <typename K>
cudaError_t prepare_smem(K kernel, size_t bytes) {
  if (bytes <= 48 * 1024) return cudaSuccess;
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

// CUFINUFFT_TC_SPREAD=1: the dense runs of 3D FP32 cell-run subproblems go
// to the tensor-core kernel (k_spread_sm_run_tc).
inline bool tc_spread_enabled() {
  const char* v = std::getenv("CUFINUFFT_TC_SPREAD");
  return v && v[0] == '1';
}

// Kernel family per stage (SpreadArgs::variant 0 = the measured default):
// spreading is warp-cooperative for method 1; for method 2 it is the
// slab-owned kernel in 3D and the private-tile kernel in 2D (the
// warp-cooperative atomic kernel in 1D, and wherever their shared memory does
// not fit), with the cell-run kernel on dense prefixes of the cell-run
// layout; interpolation is warp-cooperative for method 1 and
// one-thread-per-point for method 2 (double-float for FP64 plans at
// tol >= 1e-13).  variant 1 forces one thread per point, 2 forces
// warp-cooperative.
template <typename T, int DIM, int NS>
cudaError_t spread_ns(int method, const SpreadArgs<T>& a, cudaStream_t s) {
  if (a.M == 0) return cudaSuccess;
  const bool wc = a.variant != 1;
  if (method == 1) {
    if (wc) {
      constexpr int PPW = 32 / spread_lanes<NS>();
      k_spread_gm_wc<T, DIM, NS><<<grid_for(((long long)a.M + PPW - 1) / PPW * 32, kSpreadThreads),
                                   kSpreadThreads, 0, s>>>(a);
    } else {
      k_spread_gm<T, DIM, NS><<<grid_for(a.M, kSpreadThreads), kSpreadThreads, 0, s>>>(a);
    }
  } else {
    if (a.bins.nsub == 0) return cudaSuccess;
    // 3D sparse subproblems: the slab-owned kernel unless a variant is forced
    bool slab = false, split = false, priv = false;
    if constexpr (DIM == 2) {
      priv = a.variant == 0 && priv_spread_enabled();
      if (priv) {  // the private copies and stages must fit (else the atomic kernel)
        int dev = 0, optin = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        if (e != cudaSuccess) return e;
        priv = priv_bytes<T>(NS, a.bins) <= (size_t)optin;
      }
      split = priv && a.run && a.sub_ndense != nullptr;
    }
    if constexpr (DIM == 3) {
      slab = a.variant == 0 && slab_spread_enabled();
      if (slab) {  // its padded tile and staging must fit (else the atomic kernel)
        int dev = 0, optin = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        if (e != cudaSuccess) return e;
        slab = slab_bytes<T>(NS, a.bins) <= (size_t)optin;
      }
      // cell-run layout: the slab kernel also takes the sparse tails of the
      // dense subproblems (the tensor-core form walks whole subproblems)
      bool tc = false;
      if constexpr (sizeof(T) == 4 && NS <= 8) tc = tc_spread_enabled();
      split = slab && a.run && a.sub_ndense != nullptr && !tc;
    }
    auto sparse = [&]() -> cudaError_t {
      if constexpr (DIM == 2) {
        if (priv) {
          const size_t smb = priv_bytes<T>(NS, a.bins);
          cudaError_t e = prepare_smem(k_spread_sm_priv<T, NS>, smb);
          if (e != cudaSuccess) return e;
          k_spread_sm_priv<T, NS><<<dim3(a.bins.nsub, a.ntr), 32 * kPrivWarps, smb, s>>>(a, split ? 1 : 0);
          return cudaGetLastError();
        }
      }
      if constexpr (DIM == 3) {
        if (slab) {
          const size_t smb = slab_bytes<T>(NS, a.bins);
          cudaError_t e = prepare_smem(k_spread_sm_slab<T, NS>, smb);
          if (e != cudaSuccess) return e;
          k_spread_sm_slab<T, NS><<<dim3(a.bins.nsub, a.ntr), 32 * NS, smb, s>>>(a, split ? 1 : 0);
          return cudaGetLastError();
        }
      }
      const size_t smw = tile_bytes<T, DIM>(NS, a.bins);
      cudaError_t e = prepare_smem(k_spread_sm_wc<T, DIM, NS>, smw);
      if (e != cudaSuccess) return e;
      k_spread_sm_wc<T, DIM, NS><<<dim3(a.bins.nsub, a.ntr), kSpreadThreads, smw, s>>>(a);
      return cudaGetLastError();
    };
    if constexpr (run_ok<DIM, NS>()) {
      if (a.run) {
        // subproblems starting on a dense cell take the cell-run kernel, the
        // others the sparse kernel (each kernel skips the other kind)
        cudaError_t e = sparse();
        if (e != cudaSuccess) return e;
        if constexpr (sizeof(T) == 4 && DIM == 3 && NS <= 8) {
          if (tc_spread_enabled()) {
            const size_t smt = tc_run_bytes(NS, a.bins);
            e = prepare_smem(k_spread_sm_run_tc<NS>, smt);
            if (e != cudaSuccess) return e;
            k_spread_sm_run_tc<NS><<<dim3(a.bins.nsub, a.ntr), kSpreadThreads, smt, s>>>(a);
            return cudaGetLastError();
          }
        }
        const size_t sm = run_bytes<T, DIM>(NS, a.bins);
        e = prepare_smem(k_spread_sm_run<T, DIM, NS>, sm);
        if (e != cudaSuccess) return e;
        k_spread_sm_run<T, DIM, NS><<<dim3(a.bins.nsub, a.ntr), kSpreadThreads, sm, s>>>(a, split ? 1 : 0);
        return cudaGetLastError();
      }
    }
    if (a.run) return cudaErrorInvalidValue;  // more than 512 taps per point
    if (slab || priv) return sparse();
    size_t sm = tile_bytes<T, DIM>(NS, a.bins);
    cudaError_t e = wc ? prepare_smem(k_spread_sm_wc<T, DIM, NS>, sm)
                       : prepare_smem(k_spread_sm<T, DIM, NS>, sm);
    if (e != cudaSuccess) return e;
    dim3 grid(a.bins.nsub, a.ntr);
    if (wc) k_spread_sm_wc<T, DIM, NS><<<grid, kSpreadThreads, sm, s>>>(a);
    else k_spread_sm<T, DIM, NS><<<grid, kSpreadThreads, sm, s>>>(a);
  }
  return cudaGetLastError();
}

template <typename T, int DIM, int NS>
cudaError_t interp_ns(int method, const SpreadArgs<T>& a, cudaStream_t s) {
  if (a.M == 0) return cudaSuccess;
  const bool wc = method == 1 ? a.variant != 1 : a.variant == 2;
  if (method == 1) {
    if (wc) {
      constexpr int PPW = 32 / lanes_per_point<NS>();
      k_interp_gm_wc<T, DIM, NS><<<grid_for(((long long)a.M + PPW - 1) / PPW * 32, kSpreadThreads),
                                   kSpreadThreads, 0, s>>>(a);
    } else {
      k_interp_gm<T, DIM, NS><<<grid_for(a.M, kSpreadThreads), kSpreadThreads, 0, s>>>(a);
    }
  } else {
    if (a.bins.nsub == 0) return cudaSuccess;
    if (!wc && a.bins.hdr == nullptr) return cudaErrorInvalidValue;  // k_interp_sm reads the headers
    size_t sm = tile_bytes<T, DIM>(NS, a.bins);
    CUtensorMap gmap;
    int tma = 0;
    if (!wc) {
      std::memset(&gmap, 0, sizeof(gmap));
      tma = grid_tensor_map<T, DIM>(&gmap, a.fw_in, a.g, a.ntr, a.bins.bs, NS) ? 1 : 0;
      if (tma) {
        // widened rows, and room to align the tile for the bulk copy
        const int tx = a.bins.bs[0] + NS - 1;
        const size_t smb = sm / tx * bulk_tile_x<T>(tx) + 128;
        int dev = 0, optin = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        if (e != cudaSuccess) return e;
        if (smb <= (size_t)optin) sm = smb;
        else tma = 0;
      }
    }
    if constexpr (sizeof(T) == 8) {
      if (!wc && a.fp64_df) {
        cudaError_t e = prepare_smem(k_interp_sm_df<DIM, NS>, sm);
        if (e != cudaSuccess) return e;
        k_interp_sm_df<DIM, NS><<<dim3(a.bins.nsub, a.ntr), interp_threads_f64<DIM>(), sm, s>>>(a, gmap, tma);
        return cudaGetLastError();
      }
    }
    cudaError_t e = wc ? prepare_smem(k_interp_sm_wc<T, DIM, NS>, sm)
                       : prepare_smem(k_interp_sm<T, DIM, NS>, sm);
    if (e != cudaSuccess) return e;
    dim3 grid(a.bins.nsub, a.ntr);
    if (wc) k_interp_sm_wc<T, DIM, NS><<<grid, kSpreadThreads, sm, s>>>(a);
    else k_interp_sm<T, DIM, NS><<<grid, interp_threads<T, DIM>(), sm, s>>>(a, gmap, tma);
  }
  return cudaGetLastError();
}

#define CFG_NS_SWITCH(FN, T, DIM, ...)            \
  switch (ns) {                                   \
    case 2: return FN<T, DIM, 2>(__VA_ARGS__);    \
    case 3: return FN<T, DIM, 3>(__VA_ARGS__);    \
    case 4: return FN<T, DIM, 4>(__VA_ARGS__);    \
    case 5: return FN<T, DIM, 5>(__VA_ARGS__);    \
    case 6: return FN<T, DIM, 6>(__VA_ARGS__);    \
    case 7: return FN<T, DIM, 7>(__VA_ARGS__);    \
    case 8: return FN<T, DIM, 8>(__VA_ARGS__);    \
    case 9: return FN<T, DIM, 9>(__VA_ARGS__);    \
    case 10: return FN<T, DIM, 10>(__VA_ARGS__);  \
    case 11: return FN<T, DIM, 11>(__VA_ARGS__);  \
    case 12: return FN<T, DIM, 12>(__VA_ARGS__);  \
    case 13: return FN<T, DIM, 13>(__VA_ARGS__);  \
    case 14: return FN<T, DIM, 14>(__VA_ARGS__);  \
    case 15: return FN<T, DIM, 15>(__VA_ARGS__);  \
    case 16: return FN<T, DIM, 16>(__VA_ARGS__);  \
    default: return cudaErrorInvalidValue;        \
  }

template <typename T, int DIM>
cudaError_t spread_dim(int method, int ns, const SpreadArgs<T>& a, cudaStream_t s) {
  CFG_NS_SWITCH(spread_ns, T, DIM, method, a, s)
}

template <typename T, int DIM>
cudaError_t interp_dim(int method, int ns, const SpreadArgs<T>& a, cudaStream_t s) {
  CFG_NS_SWITCH(interp_ns, T, DIM, method, a, s)
}

}  // namespace cfg
