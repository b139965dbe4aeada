// noalloc.cu -- an allocation-free 2D FP32 spreading entry point.
//
// Some callers cannot allocate device memory when they need a transform:
// code that runs inside a framework which owns all device memory (custom
// operators of array libraries, other libraries' memory pools), real-time
// loops that must not enter the driver's allocator, and host code that runs
// where a cudaMalloc would synchronise the device or fail outright under a
// memory budget.  For them cufinufftf_spread2d_noalloc performs the type-1
// spreading stage -- bin sort of the points and shared-memory subproblem
// spreading onto a caller-provided fine grid -- without any allocation: the
// sort's scratch (bin counts and starts, the subproblem map, the sorted
// points) lives in one fixed device array declared below, of kNaScratchBytes
// bytes, which every GPU that loads this library holds until the process
// exits.
//
// Rules a caller must know (they are repeated in include/cufinufft.h):
//   * at most kNaMaxPoints points and kNaMaxBins 32x32 bins (a fine grid up
//     to 2048 x 2048); larger requests return CUFINUFFT_ERR_ARG;
//   * the scratch array is shared by every call in the process on that
//     device and keeps the previous call's contents; this call clears what
//     must start at zero (the bin counts and the output grid), but calls
//     whose GPU work overlaps -- on different streams or host threads --
//     race on it and must be serialised by the caller;
//   * the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress, once per device, with that device current), so
//     make that first call before any stream capture begins.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/cufinufft.h"
#include "kernels.h"
#include "planner.h"
#include "spreadinterp.cuh"

namespace cfg {
namespace {

constexpr int kNaMaxPoints = 1 << 17;  // 131072 nonuniform points
constexpr int kNaBin = 32;              // bin edge (cells), as the 2D default
constexpr int kNaMaxBins = 4096;        // (2048 / 32)^2
constexpr int kNaMaxSub = 1024;         // points per subproblem
constexpr int kNaMaxSubprobs = kNaMaxBins + kNaMaxPoints / kNaMaxSub + 1;
constexpr int kNaMaxDevices = 64;

constexpr size_t align256(size_t n) { return (n + 255) & ~size_t(255); }
constexpr size_t kNaBinBytes = align256(sizeof(int) * (kNaMaxBins + 1));
constexpr size_t kNaSubBytes = align256(sizeof(int) * kNaMaxSubprobs);
constexpr size_t kNaPtBytes = align256(sizeof(int) * kNaMaxPoints);
// count, start, sub_start, scan tmp | sub_to_bin | idx, rank, i0x, i0y, dx, dy
constexpr size_t kNaScratchBytes = 4 * kNaBinBytes + kNaSubBytes + 6 * kNaPtBytes;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaScratchBytes];

std::mutex g_na_mutex;
void* g_na_base[kNaMaxDevices] = {};

// Device address of the scratch array on the current device (looked up once
// per device; the host-side name is only a stand-in for the symbol).  The
// address is cached for the life of the process: a device reset after the
// first call would reload the module and leave the cached address stale, so
// resets are not supported once the entry point has been used.
cudaError_t scratch_base(int dev, unsigned char** out) {
  if (dev < 0 || dev >= kNaMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_na_mutex);
  if (g_na_base[dev] == nullptr) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_na_base[dev] = p;
  }
  *out = static_cast<unsigned char*>(g_na_base[dev]);
  return cudaSuccess;
}

AxisMap<float> na_axis(int nf, int ns) {
  AxisMap<float> a;
  const double S = (double)nf / (2.0 * M_PI);
  a.s_hi = (float)S;
  a.s_lo = (float)(S - (double)a.s_hi);
  a.o_lo = (float)(1.5 * nf);
  a.o_mid = (float)(0.5 * nf);
  a.o_hi = (float)(-0.5 * nf);
  a.half_int = ns / 2;
  a.half_frac = (ns % 2) ? 0.5f : 0.0f;
  a.nf = nf;
  return a;
}

// Subproblem -> bin map with the subproblem total read on the device (the
// grid covers the upper bound kNaMaxSubprobs).
__global__ void k_na_sub_to_bin(const int* sub_start, int nbins, int* sub_to_bin) {
  const int nsub = sub_start[nbins];
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nsub; s += gridDim.x * blockDim.x) {
    int lo = 0, hi = nbins;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (sub_start[mid] <= s) lo = mid;
      else hi = mid;
    }
    sub_to_bin[s] = lo;
  }
}

// The warp-cooperative shared-memory spread (k_spread_sm_wc) specialised to
// 2D FP32, launched over the upper bound of subproblems: blocks past the
// device-side total return at once.
template <int NS>
__global__ void __launch_bounds__(kSpreadThreads)
k_na_spread2d(SpreadArgs<float> a, const int* nsub_dev) {
  if ((int)blockIdx.x >= *nsub_dev) return;
  constexpr int L = lanes_per_point<NS>();
  constexpr int PPW = 32 / L;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* tile = reinterpret_cast<float2*>(smem_raw);
  const SubTile st = sub_tile<2, NS>(a.bins, blockIdx.x);
  tile_zero<float>(tile, st.ntile);
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
    const int ly = a.pts.i0[1][p] - st.oy;
    const float kx = kernel_tap<float, NS, horner_degree<float>(NS)>(a.pts.d[0][p], jj, a.kc);
    const float ky = kernel_tap<float, NS, horner_degree<float>(NS)>(a.pts.d[1][p], jj, a.kc);
    const float2 v = a.c_in[a.pts.idx[p]];
    const float vr = v.x * kx, vi = v.y * kx;
    float2* row0 = tile + ly * st.TX + lx + jj;
#pragma unroll
    for (int dy = 0; dy < NS; ++dy) {
      const float kyv = __shfl_sync(0xffffffffu, ky, g * L + dy);
      if (tap && valid) smem_add(row0 + dy * st.TX, vr * kyv, vi * kyv);
    }
  }
  __syncthreads();
  tile_flush<float>(tile, a.fw, st, a.g);
}

template <int NS>
cudaError_t na_launch(const SpreadArgs<float>& a, const int* nsub_dev, int nsub_max,
                      cudaStream_t s) {
  const size_t smem = tile_cells(2, NS, a.bins.bs) * sizeof(float2);
  k_na_spread2d<NS><<<nsub_max, kSpreadThreads, smem, s>>>(a, nsub_dev);
  return cudaGetLastError();
}

cudaError_t na_dispatch(int ns, const SpreadArgs<float>& a, const int* nsub_dev, int nsub_max,
                        cudaStream_t s) {
  switch (ns) {
    case 2: return na_launch<2>(a, nsub_dev, nsub_max, s);
    case 3: return na_launch<3>(a, nsub_dev, nsub_max, s);
    case 4: return na_launch<4>(a, nsub_dev, nsub_max, s);
    case 5: return na_launch<5>(a, nsub_dev, nsub_max, s);
    case 6: return na_launch<6>(a, nsub_dev, nsub_max, s);
    case 7: return na_launch<7>(a, nsub_dev, nsub_max, s);
    case 8: return na_launch<8>(a, nsub_dev, nsub_max, s);
    case 9: return na_launch<9>(a, nsub_dev, nsub_max, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace
}  // namespace cfg

extern "C" int cufinufftf_spread2d_noalloc(int M, const float* x, const float* y,
                                           const cuFloatComplex* c, int nf1, int nf2, float tol,
                                           cuFloatComplex* fw, cudaStream_t stream) {
  using namespace cfg;
  if (M < 0 || nf1 < 1 || nf2 < 1 || fw == nullptr) return CUFINUFFT_ERR_ARG;
  if (M > 0 && (x == nullptr || y == nullptr || c == nullptr)) return CUFINUFFT_ERR_ARG;
  SpreaderParams sp;
  const int ier = setup_spreader((double)tol, 2.0, 0, true, &sp);
  if (ier > 1) return ier;
  if (sp.ns > 9) return CUFINUFFT_ERR_ARG;
  const int nb0 = (nf1 + kNaBin - 1) / kNaBin, nb1 = (nf2 + kNaBin - 1) / kNaBin;
  const long long nbins = (long long)nb0 * nb1;
  if (M > kNaMaxPoints || nbins > kNaMaxBins) {
    fprintf(stderr,
            "cufinufftf_spread2d_noalloc: request exceeds the fixed scratch (M=%d of at most %d "
            "points, %lld of at most %d bins of 32x32 cells)\n",
            M, kNaMaxPoints, nbins, kNaMaxBins);
    return CUFINUFFT_ERR_ARG;
  }
  if (nf1 < 2 * sp.ns || nf2 < 2 * sp.ns) return CUFINUFFT_ERR_ARG;

  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return CUFINUFFT_ERR_CUDA;
  unsigned char* base = nullptr;
  cudaError_t e = scratch_base(dev, &base);
  if (e != cudaSuccess) {
    fprintf(stderr, "cufinufftf_spread2d_noalloc: cudaGetSymbolAddress failed: %s\n",
            cudaGetErrorString(e));
    return CUFINUFFT_ERR_CUDA;
  }
  int* count = reinterpret_cast<int*>(base);
  int* start = reinterpret_cast<int*>(base + kNaBinBytes);
  int* sub_start = reinterpret_cast<int*>(base + 2 * kNaBinBytes);
  int* scan_tmp = reinterpret_cast<int*>(base + 3 * kNaBinBytes);
  int* sub_to_bin = reinterpret_cast<int*>(base + 4 * kNaBinBytes);
  unsigned char* pts = base + 4 * kNaBinBytes + kNaSubBytes;
  int* idx = reinterpret_cast<int*>(pts);
  int* rank = reinterpret_cast<int*>(pts + kNaPtBytes);
  int* i0x = reinterpret_cast<int*>(pts + 2 * kNaPtBytes);
  int* i0y = reinterpret_cast<int*>(pts + 3 * kNaPtBytes);
  float* dx = reinterpret_cast<float*>(pts + 4 * kNaPtBytes);
  float* dy = reinterpret_cast<float*>(pts + 5 * kNaPtBytes);

  // what must start at zero: the output grid and the bin counts
  e = cudaMemsetAsync(fw, 0, sizeof(cuFloatComplex) * (size_t)nf1 * nf2, stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(count, 0, sizeof(int) * (size_t)nbins, stream);
  if (e != cudaSuccess) return CUFINUFFT_ERR_CUDA;
  if (M == 0) return 0;

  PlaceArgs<float> pa;
  memset(&pa, 0, sizeof(pa));  // also plain bin order: pa.bank.cls_count = nullptr
  pa.x[0] = x;
  pa.x[1] = y;
  pa.x[2] = nullptr;
  pa.ax[0] = na_axis(nf1, sp.ns);
  pa.ax[1] = na_axis(nf2, sp.ns);
  pa.ax[2] = na_axis(1, sp.ns);
  pa.dim = 2;
  pa.M = M;
  pa.bs[0] = kNaBin;
  pa.bs[1] = kNaBin;
  pa.bs[2] = 1;
  pa.nb[0] = nb0;
  pa.nb[1] = nb1;
  pa.nb[2] = 1;
  pa.idx = idx;
  pa.i0[0] = i0x;
  pa.i0[1] = i0y;
  pa.i0[2] = nullptr;
  pa.d[0] = dx;
  pa.d[1] = dy;
  pa.d[2] = nullptr;
  pa.count = count;
  pa.rank = rank;
  pa.start = start;
  e = launch_bin_count<float>(pa, stream);
  if (e == cudaSuccess) e = launch_scan(count, start, (int)nbins, 0, 1, scan_tmp, stream);
  if (e == cudaSuccess) e = launch_permute<float>(pa, stream);
  if (e == cudaSuccess) e = launch_scan(count, sub_start, (int)nbins, 1, kNaMaxSub, scan_tmp, stream);
  const int nsub_max = (int)nbins + (M + kNaMaxSub - 1) / kNaMaxSub;
  if (e == cudaSuccess) {
    k_na_sub_to_bin<<<(nsub_max + 255) / 256, 256, 0, stream>>>(sub_start, (int)nbins, sub_to_bin);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) return CUFINUFFT_ERR_CUDA;

  SpreadArgs<float> a;
  memset(&a, 0, sizeof(a));
  a.pts.idx = idx;
  a.pts.i0[0] = i0x;
  a.pts.i0[1] = i0y;
  a.pts.d[0] = dx;
  a.pts.d[1] = dy;
  a.pts.M = M;
  a.bins.bs[0] = kNaBin;
  a.bins.bs[1] = kNaBin;
  a.bins.bs[2] = 1;
  a.bins.nb[0] = nb0;
  a.bins.nb[1] = nb1;
  a.bins.nb[2] = 1;
  a.bins.nbins = (int)nbins;
  a.bins.count = count;
  a.bins.start = start;
  a.bins.sub_start = sub_start;
  a.bins.sub_to_bin = sub_to_bin;
  a.bins.nsub = nsub_max;
  a.bins.maxsub = kNaMaxSub;
  a.kc.beta = (float)sp.beta;
  a.kc.c = (float)sp.c;
  a.kc.e_beta = (float)std::exp(sp.beta);
  a.kc.bl2e = (float)(sp.beta * 1.44269504088896340736);
  a.kc.horner = 0;
  a.kc.coef_g = nullptr;
  a.g.nf[0] = nf1;
  a.g.nf[1] = nf2;
  a.g.nf[2] = 1;
  a.g.Nf = (long long)nf1 * nf2;
  a.c_in = reinterpret_cast<const float2*>(c);
  a.fw = reinterpret_cast<float2*>(fw);
  a.ntr = 1;
  a.M = M;
  e = na_dispatch(sp.ns, a, sub_start + nbins, nsub_max, stream);
  return e == cudaSuccess ? 0 : CUFINUFFT_ERR_CUDA;
}
