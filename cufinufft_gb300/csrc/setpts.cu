// setpts.cu -- bin sort of the nonuniform points (the setpts stage).
//
// The reference sorts in four launches per call (src/2d/spread2d_wrapper.cu:
// 386-613): CalcBinSize_noghost (per-point bin + atomic rank), a Thrust
// exclusive scan, CalcInvertofGlobalSortIdx (scatter of the permutation),
// then CalcSubProb / inclusive scan / MapBintoSubProb for the subproblem
// method.  Here:
//   * k_bin_count places every point on the fine grid (place_coord) and ranks
//     it inside its bin with warp-aggregated atomics (one atomic per distinct
//     bin in a warp, so clustered points do not serialise on one counter);
//   * a three-phase block scan produces the bin starts and the subproblem
//     starts (mode 1 scans ceil(count/maxsub) directly);
//   * k_permute writes the sorted structure-of-arrays copy the spread and
//     interp kernels stream: caller index, first tap and offset per axis;
//   * k_sub_to_bin maps subproblems to bins by binary search (one thread per
//     subproblem, balanced even when one bin holds most of the points).
#include "device_common.cuh"
#include "kernels.h"

namespace cfg {

constexpr int kPlaceThreads = 256;

template <typename T>
__device__ __forceinline__ int point_bin(const PlaceArgs<T>& a, int i, int i0[3], T d[3]) {
  int b = 0, mul = 1;
  for (int k = 0; k < 3; ++k) {
    if (k < a.dim) {
      place_coord<T>(a.x[k][i], a.ax[k], i0[k], d[k]);
      b += mul * (i0[k] / a.bs[k]);
      mul *= a.nb[k];
    }
  }
  return b;
}

// Bank class of a point whose first taps are i0 (see BankOrder).
__device__ __forceinline__ int bank_class(const BankOrder& o, const int* bs, int dim, const int i0[3]) {
  const int lx = i0[0] % bs[0];
  const int ly = dim > 1 ? i0[1] % bs[1] : 0;
  const int lz = dim > 2 ? i0[2] % bs[2] : 0;
  return (lx + o.tx * (ly + o.ty * lz)) & (o.ncls - 1);
}

// Class of a point inside its bin: its bank class, or its cell (cell order).
__device__ __forceinline__ int order_class(const BankOrder& o, const int* bs, int dim, const int i0[3]) {
  if (!o.cell_order) return bank_class(o, bs, dim, i0);
  const int lx = i0[0] % bs[0];
  const int ly = dim > 1 ? i0[1] % bs[1] : 0;
  const int lz = dim > 2 ? i0[2] % bs[2] : 0;
  return lx + bs[0] * (ly + bs[1] * lz);
}

// Position of a ranked point: cell order reads the scanned (bin, cell)
// starts; bank order interleaves inside the bin.
__device__ __forceinline__ int interleave_pos(const BankOrder& o, int b, int c, int r);
__device__ __forceinline__ int ordered_pos(const BankOrder& o, const int* start, int b, int c, int r) {
  return start[b] + interleave_pos(o, b, c, r);
}

// Warp-aggregated rank: one atomic per distinct key in the warp.
__device__ __forceinline__ int agg_rank(unsigned act, int key, int* counter) {
  const int lane = threadIdx.x & 31;
  const unsigned peers = __match_any_sync(act, key);
  const int leader = __ffs(peers) - 1;
  int first = 0;
  if (lane == leader) first = atomicAdd(counter, __popc(peers));
  first = __shfl_sync(peers, first, leader);
  return first + __popc(peers & ((1u << lane) - 1u));
}

// Cell order (BankOrder::cell_order): a bin's points on dense cells (at least
// dense_min points) come first, sorted by cell -- cls_start is the exclusive
// scan of the dense cells' counts only -- then the bin's other points in
// arbitrary order, ranked by the per-bin counter sparse_count.  r is the
// point's rank inside its cell.  Called by the lanes in act together.
__device__ __forceinline__ int cell_position(const BankOrder& o, const int* start, unsigned act, int b,
                                             int c, int r) {
  const long long k0 = (long long)b * o.ncls;
  const int bin0 = o.cls_start[k0];
  const bool dense = o.cls_count[k0 + c] >= o.dense_min;
  const unsigned sparse_lanes = __ballot_sync(act, !dense);
  if (dense) return start[b] + (o.cls_start[k0 + c] - bin0) + r;
  const int sr = agg_rank(sparse_lanes, b, o.sparse_count + b);
  return start[b] + (o.cls_start[k0 + o.ncls] - bin0) + sr;
}

// Position inside its bin of the point ranked r in class c: round-robin over
// the classes, rounds shrinking as classes run out.
__device__ __forceinline__ int interleave_pos(const BankOrder& o, int b, int c, int r) {
  const int* cnt = o.cls_count + (long long)b * o.ncls;
  int pos = 0;
  for (int k = 0; k < o.ncls; ++k) {
    const int n = __ldg(cnt + k);
    pos += min(n, r) + ((k < c && n > r) ? 1 : 0);
  }
  return pos;
}

template <typename T>
__global__ void __launch_bounds__(kPlaceThreads) k_bin_count(PlaceArgs<T> a) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  // warp-uniform trip count so the warp stays converged for __match_any_sync
  for (long long base = (long long)blockIdx.x * blockDim.x; base < a.M; base += stride) {
    const long long ii = base + threadIdx.x;
    const bool active = ii < a.M;
    const unsigned act = __ballot_sync(0xffffffffu, active);
    if (!active) continue;
    const int i = (int)ii;
    int i0[3];
    T d[3];
    const int b = point_bin(a, i, i0, d);
    const int r = agg_rank(act, b, &a.count[b]);
    if (a.bank.cls_count) {
      const int key = b * a.bank.ncls + order_class(a.bank, a.bs, a.dim, i0);
      a.rank[i] = agg_rank(act, key, a.bank.cls_count + key);
    } else {
      a.rank[i] = r;
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(kPlaceThreads) k_permute(PlaceArgs<T> a) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  // warp-uniform trip count: cell order ranks sparse points warp-aggregated
  for (long long base = (long long)blockIdx.x * blockDim.x; base < a.M; base += stride) {
    const long long ii = base + threadIdx.x;
    const bool active = ii < a.M;
    const unsigned act = __ballot_sync(0xffffffffu, active);
    if (!active) continue;
    const int i = (int)ii;
    int i0[3];
    T d[3];
    const int b = point_bin(a, i, i0, d);
    int pos;
    if (!a.bank.cls_count) pos = a.start[b] + a.rank[i];
    else if (a.bank.cell_order) pos = cell_position(a.bank, a.start, act, b, order_class(a.bank, a.bs, a.dim, i0), a.rank[i]);
    else pos = ordered_pos(a.bank, a.start, b, order_class(a.bank, a.bs, a.dim, i0), a.rank[i]);
    a.idx[pos] = i;
    for (int k = 0; k < 3; ++k) {
      if (k < a.dim) {
        a.i0[k][pos] = i0[k];
        a.d[k][pos] = d[k];
      }
    }
  }
}

// gpu_sort = 0 with method 1 keeps the caller's order (reference "GM",
// TrivialGlobalSortIdx, src/precision_independent.cu:98-105).
template <typename T>
__global__ void __launch_bounds__(kPlaceThreads) k_place_unsorted(PlaceArgs<T> a) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.M; i += gridDim.x * blockDim.x) {
    a.idx[i] = i;
    for (int k = 0; k < 3; ++k) {
      if (k < a.dim) {
        int i0;
        T d;
        place_coord<T>(a.x[k][i], a.ax[k], i0, d);
        a.i0[k][i] = i0;
        a.d[k][i] = d;
      }
    }
  }
}

__global__ void __launch_bounds__(kPlaceThreads) k_place_narrow(NarrowPlaceArgs a) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.M; i += gridDim.x * blockDim.x) {
    a.idx[i] = i;
    for (int k = 0; k < 3; ++k) {
      if (k < a.dim) {
        int i0;
        double d;
        place_coord<double>(a.x[k][i], a.ax[k], i0, d);
        a.i0[k][i] = i0;
        a.d[k][i] = (float)d;
      }
    }
  }
}

static int place_grid(int M) {
  long long b = ((long long)M + kPlaceThreads - 1) / kPlaceThreads;
  if (b > 152LL * 64) b = 152LL * 64;
  return b < 1 ? 1 : (int)b;
}

template <typename T> cudaError_t launch_bin_count(const PlaceArgs<T>& a, cudaStream_t s) {
  if (a.M == 0) return cudaSuccess;
  k_bin_count<T><<<place_grid(a.M), kPlaceThreads, 0, s>>>(a);
  return cudaGetLastError();
}
template <typename T> cudaError_t launch_permute(const PlaceArgs<T>& a, cudaStream_t s) {
  if (a.M == 0) return cudaSuccess;
  k_permute<T><<<place_grid(a.M), kPlaceThreads, 0, s>>>(a);
  return cudaGetLastError();
}
template <typename T> cudaError_t launch_place_unsorted(const PlaceArgs<T>& a, cudaStream_t s) {
  if (a.M == 0) return cudaSuccess;
  k_place_unsorted<T><<<place_grid(a.M), kPlaceThreads, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_place_narrow(const NarrowPlaceArgs& a, cudaStream_t s) {
  if (a.M == 0) return cudaSuccess;
  k_place_narrow<<<place_grid(a.M), kPlaceThreads, 0, s>>>(a);
  return cudaGetLastError();
}

template cudaError_t launch_bin_count<float>(const PlaceArgs<float>&, cudaStream_t);
template cudaError_t launch_bin_count<double>(const PlaceArgs<double>&, cudaStream_t);
template cudaError_t launch_permute<float>(const PlaceArgs<float>&, cudaStream_t);
template cudaError_t launch_permute<double>(const PlaceArgs<double>&, cudaStream_t);
template cudaError_t launch_place_unsorted<float>(const PlaceArgs<float>&, cudaStream_t);
template cudaError_t launch_place_unsorted<double>(const PlaceArgs<double>&, cudaStream_t);

// ---------------------------------------------------------------------------
// Re-binning from stored first taps.
template <typename T>
__device__ __forceinline__ int stored_bin(const RebinArgs<T>& a, int i) {
  int b = 0, mul = 1;
  for (int k = 0; k < 3; ++k) {
    if (k < a.dim) {
      b += mul * (a.src_i0[k][i] / a.bs[k]);
      mul *= a.nb[k];
    }
  }
  return b;
}

template <typename T>
__global__ void __launch_bounds__(kPlaceThreads) k_rebin_count(RebinArgs<T> a) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long base = (long long)blockIdx.x * blockDim.x; base < a.M; base += stride) {
    const long long ii = base + threadIdx.x;
    const bool active = ii < a.M;
    const unsigned act = __ballot_sync(0xffffffffu, active);
    if (!active) continue;
    const int i = (int)ii;
    const int b = stored_bin(a, i);
    const int r = agg_rank(act, b, &a.count[b]);
    if (a.bank.cls_count) {
      const int i0[3] = {a.src_i0[0][i], a.dim > 1 ? a.src_i0[1][i] : 0, a.dim > 2 ? a.src_i0[2][i] : 0};
      const int key = b * a.bank.ncls + order_class(a.bank, a.bs, a.dim, i0);
      a.rank[i] = agg_rank(act, key, a.bank.cls_count + key);
    } else {
      a.rank[i] = r;
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(kPlaceThreads) k_rebin_permute(RebinArgs<T> a) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long base = (long long)blockIdx.x * blockDim.x; base < a.M; base += stride) {
    const long long ii = base + threadIdx.x;
    const bool active = ii < a.M;
    const unsigned act = __ballot_sync(0xffffffffu, active);
    if (!active) continue;
    const int i = (int)ii;
    const int b = stored_bin(a, i);
    int pos = a.start[b] + a.rank[i];
    if (a.bank.cls_count) {
      const int i0[3] = {a.src_i0[0][i], a.dim > 1 ? a.src_i0[1][i] : 0, a.dim > 2 ? a.src_i0[2][i] : 0};
      const int c = order_class(a.bank, a.bs, a.dim, i0);
      pos = a.bank.cell_order ? cell_position(a.bank, a.start, act, b, c, a.rank[i])
                              : ordered_pos(a.bank, a.start, b, c, a.rank[i]);
    }
    a.idx[pos] = a.src_idx[i];
    for (int k = 0; k < 3; ++k) {
      if (k < a.dim) {
        a.i0[k][pos] = a.src_i0[k][i];
        a.d[k][pos] = a.src_d[k][i];
      }
    }
  }
}

template <typename T> cudaError_t launch_rebin_count(const RebinArgs<T>& a, cudaStream_t s) {
  if (a.M == 0) return cudaSuccess;
  k_rebin_count<T><<<place_grid(a.M), kPlaceThreads, 0, s>>>(a);
  return cudaGetLastError();
}
template <typename T> cudaError_t launch_rebin_permute(const RebinArgs<T>& a, cudaStream_t s) {
  if (a.M == 0) return cudaSuccess;
  k_rebin_permute<T><<<place_grid(a.M), kPlaceThreads, 0, s>>>(a);
  return cudaGetLastError();
}
template cudaError_t launch_rebin_count<float>(const RebinArgs<float>&, cudaStream_t);
template cudaError_t launch_rebin_count<double>(const RebinArgs<double>&, cudaStream_t);
template cudaError_t launch_rebin_permute<float>(const RebinArgs<float>&, cudaStream_t);
template cudaError_t launch_rebin_permute<double>(const RebinArgs<double>&, cudaStream_t);

// ---------------------------------------------------------------------------
// Occupancy counts for the selector's features.
struct FeatureArgs {
  const int* i0[3];
  int fb[3], nb[3];
  int dim, M;
  int* counts;
};

__global__ void k_feature_count(FeatureArgs a) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.M; i += gridDim.x * blockDim.x) {
    int b = 0, mul = 1;
    for (int k = 0; k < 3; ++k) {
      if (k < a.dim) {
        b += mul * (a.i0[k][i] / a.fb[k]);
        mul *= a.nb[k];
      }
    }
    atomicAdd(&a.counts[b], 1);
  }
}

cudaError_t launch_feature_count(int dim, int M, const int* const i0[3], const int fb[3],
                                 const int nb[3], int* counts, cudaStream_t s) {
  if (M == 0) return cudaSuccess;
  FeatureArgs a;
  for (int k = 0; k < 3; ++k) {
    a.i0[k] = i0[k];
    a.fb[k] = fb[k];
    a.nb[k] = nb[k];
  }
  a.dim = dim;
  a.M = M;
  a.counts = counts;
  k_feature_count<<<place_grid(M), kPlaceThreads, 0, s>>>(a);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Exclusive scan: 1024 threads x 4 items per block; block totals are scanned
// by one block (up to 4096 blocks, i.e. 16.7M entries), then added back.
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;
constexpr int kScanMaxBlocks = 4096;

__device__ __forceinline__ int scan_load(const int* in, int i, int n, int mode, int div) {
  if (i >= n) return 0;
  int v = in[i];
  if (mode == 2) return v >= div ? v : 0;  // counts of at least div only
  return mode == 1 ? (v + div - 1) / div : v;
}

// Block-wide exclusive scan of one value per thread; returns the block total.
__device__ __forceinline__ int block_exclusive_scan(int v, int& excl) {
  __shared__ int warp_tot[kScanThreads / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int n = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += n;
  }
  if (lane == 31) warp_tot[w] = incl;
  __syncthreads();
  if (w == 0) {
    int t = lane < (int)(blockDim.x >> 5) ? warp_tot[lane] : 0;
    int ti = t;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int n = __shfl_up_sync(0xffffffffu, ti, o);
      if (lane >= o) ti += n;
    }
    warp_tot[lane] = ti - t;  // exclusive warp offsets
  }
  __syncthreads();
  excl = warp_tot[w] + incl - v;
  __shared__ int tot;
  if (threadIdx.x == blockDim.x - 1) tot = excl + v;  // inclusive sum of the last thread
  __syncthreads();
  const int total = tot;
  __syncthreads();
  return total;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_partial(const int* in, int n, int mode, int div,
                                                              int* partial) {
  const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  int s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) s += scan_load(in, base + k, n, mode, div);
  int excl;
  int total = block_exclusive_scan(s, excl);
  if (threadIdx.x == 0) partial[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_partials(int* partial, int nblocks) {
  // one block: exclusive scan of nblocks (<= 4096) partial sums in place
  int v[kScanItems];
  int s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    int i = threadIdx.x * kScanItems + k;
    v[k] = i < nblocks ? partial[i] : 0;
    s += v[k];
  }
  int excl;
  block_exclusive_scan(s, excl);
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    int i = threadIdx.x * kScanItems + k;
    if (i < nblocks) partial[i] = excl;
    excl += v[k];
  }
}

__global__ void __launch_bounds__(kScanThreads) k_scan_final(const int* in, int n, int mode, int div,
                                                            const int* partial, int* out) {
  const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  int v[kScanItems];
  int s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    v[k] = scan_load(in, base + k, n, mode, div);
    s += v[k];
  }
  int excl;
  int total = block_exclusive_scan(s, excl);
  excl += partial[blockIdx.x];
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    if (base + k < n) out[base + k] = excl;
    excl += v[k];
  }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) out[n] = partial[blockIdx.x] + total;
}

int scan_tmp_ints(int n) {
  int nb = (n + kScanTile - 1) / kScanTile;
  return nb < 1 ? 1 : nb;
}

cudaError_t launch_scan(const int* in, int* out, int n, int mode, int div, int* tmp, cudaStream_t s) {
  if (n <= 0) return cudaMemsetAsync(out, 0, sizeof(int), s);
  int nb = scan_tmp_ints(n);
  if (nb > kScanMaxBlocks) return cudaErrorInvalidValue;
  k_scan_partial<<<nb, kScanThreads, 0, s>>>(in, n, mode, div, tmp);
  k_scan_partials<<<1, kScanThreads, 0, s>>>(tmp, nb);
  k_scan_final<<<nb, kScanThreads, 0, s>>>(in, n, mode, div, tmp, out);
  return cudaGetLastError();
}

__global__ void k_classify_subproblems(SubClassArgs a) {
  for (int sidx = blockIdx.x * blockDim.x + threadIdx.x; sidx < a.nsub; sidx += gridDim.x * blockDim.x) {
    const int b = a.sub_to_bin[sidx];
    const int p0 = a.start[b] + (sidx - a.sub_start[b]) * a.maxsub;
    const int lx = a.i0[0][p0] % a.bs[0];
    const int ly = a.dim > 1 ? a.i0[1][p0] % a.bs[1] : 0;
    const int lz = a.dim > 2 ? a.i0[2][p0] % a.bs[2] : 0;
    const int c = lx + a.bs[0] * (ly + a.bs[1] * lz);
    a.dense[sidx] = a.cls_count[(long long)b * a.ncls + c] >= a.dense_min ? 1 : 0;
    if (a.ndense) {
      const int js = sidx - a.sub_start[b];
      const int np = min(a.maxsub, a.count[b] - js * a.maxsub);
      const int nd = a.cls_start[(long long)(b + 1) * a.ncls] - a.cls_start[(long long)b * a.ncls];
      a.ndense[sidx] = max(0, min(np, nd - js * a.maxsub));
    }
  }
}

cudaError_t launch_classify_subproblems(const SubClassArgs& a, cudaStream_t s) {
  if (a.nsub <= 0) return cudaSuccess;
  int blocks = (a.nsub + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  k_classify_subproblems<<<blocks, 256, 0, s>>>(a);
  return cudaGetLastError();
}

__global__ void k_sub_to_bin(const int* sub_start, int nbins, int nsub, int* sub_to_bin) {
  for (int sidx = blockIdx.x * blockDim.x + threadIdx.x; sidx < nsub; sidx += gridDim.x * blockDim.x) {
    // largest b with sub_start[b] <= sidx
    int lo = 0, hi = nbins;  // invariant: sub_start[lo] <= sidx < sub_start[hi]
    while (hi - lo > 1) {
      int mid = (lo + hi) >> 1;
      if (sub_start[mid] <= sidx) lo = mid;
      else hi = mid;
    }
    sub_to_bin[sidx] = lo;
  }
}

cudaError_t launch_sub_to_bin(const int* sub_start, int nbins, int nsub, int* sub_to_bin, cudaStream_t s) {
  if (nsub <= 0) return cudaSuccess;
  k_sub_to_bin<<<place_grid(nsub), kPlaceThreads, 0, s>>>(sub_start, nbins, nsub, sub_to_bin);
  return cudaGetLastError();
}

struct SubHdrArgs {
  const int *sub_start, *start, *count;
  int nbins, nsub, maxsub;
  int bs[3], nb[3];
  int* sub_to_bin;
  SubHdr* hdr;
};

// The same bin search as k_sub_to_bin, then the subproblem's point range
// (subproblem js of bin b: points start[b] + js maxsub, at most maxsub of
// them) and its tile origin (the bin's first cell).
__global__ void k_sub_headers(SubHdrArgs a) {
  for (int sidx = blockIdx.x * blockDim.x + threadIdx.x; sidx < a.nsub; sidx += gridDim.x * blockDim.x) {
    int lo = 0, hi = a.nbins;
    while (hi - lo > 1) {
      int mid = (lo + hi) >> 1;
      if (a.sub_start[mid] <= sidx) lo = mid;
      else hi = mid;
    }
    const int b = lo;
    a.sub_to_bin[sidx] = b;
    const int js = sidx - a.sub_start[b];
    SubHdr h;
    h.p0 = a.start[b] + js * a.maxsub;
    h.np = min(a.maxsub, a.count[b] - js * a.maxsub);
    h.ox = (b % a.nb[0]) * a.bs[0];
    h.oy = ((b / a.nb[0]) % a.nb[1]) * a.bs[1];
    h.oz = (b / (a.nb[0] * a.nb[1])) * a.bs[2];
    h.pad0 = h.pad1 = h.pad2 = 0;
    a.hdr[sidx] = h;
  }
}

cudaError_t launch_sub_headers(const int* sub_start, const int* start, const int* count, int nbins,
                               int nsub, int maxsub, const int bs[3], const int nb[3], int* sub_to_bin,
                               SubHdr* hdr, cudaStream_t s) {
  if (nsub <= 0) return cudaSuccess;
  SubHdrArgs a;
  a.sub_start = sub_start;
  a.start = start;
  a.count = count;
  a.nbins = nbins;
  a.nsub = nsub;
  a.maxsub = maxsub;
  for (int k = 0; k < 3; ++k) {
    a.bs[k] = bs[k];
    a.nb[k] = nb[k];
  }
  a.sub_to_bin = sub_to_bin;
  a.hdr = hdr;
  k_sub_headers<<<place_grid(nsub), kPlaceThreads, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace cfg
