// plan.h -- the plan object shared by the C ABI (api.cu) and the
// multi-plan batch (batch.cu), with small helpers both use.
#pragma once

#include <cufft.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/cufinufft.h"
#include "kernels.h"
#include "planner.h"

namespace cfg {

template <typename T> struct Plan {
  using C = cplx_t<T>;
  int type = 0, dim = 0;
  int N[3] = {1, 1, 1};
  int nf[3] = {1, 1, 1};
  int ntransf = 1, maxbatch = 1, iflag = 1;
  cufinufft_opts opts;
  SpreaderParams sp{};
  int width_rule = 0;  // 0: the reference's kernel width, 1: the tolerance-meeting width
  int method = 0;  // method run: 1 (NU-point driven) or 2 (subproblem); 0 = invalid
                   // (layout method 5 = method 2 with cell_order, see set_layout)
  int variant = 0; // kernel family: 0 default, 1 one thread per point, 2 warp-cooperative
  bool auto_method = false;  // gpu_method 0: chosen by the library
  float* sel_buf = nullptr;  // selector network parameters and scratch (device)
  int sort = 1;
  int bs[3] = {1, 1, 1}, nb[3] = {1, 1, 1};
  int nbins = 1;
  int device = 0;
  int M = 0, nsub = 0;
  bool planned = false, pts_set = false;
  bool spread_only = false;  // gpu_spreadinterponly: fk is the fine grid, no FFT/deconvolution
  cudaStream_t own = nullptr, stream = nullptr;
  cufftHandle fft = 0, fft_rem = 0;
  bool have_fft = false, have_fft_rem = false;
  // pruned line FFTs (fftpass.cu) instead of cuFFT: per-axis twiddle tables
  // exp(iflag 2 pi i m / nf_d) and radix sequences
  bool line_fft = false;
  bool half_fft = false;  // pruned power-of-two passes (halffft.cu), tables in tw
  // FP64 2D grids: double-float FFT (fft_df.cu) instead of cuFFT's Z2Z
  bool df_fft = false;
  int df_fft_ok = 0;            // set at makeplan: precision, tol and switch allow it
  double2* df_tmp = nullptr;    // maxbatch grids of scratch
  float4* df_tw[2] = {nullptr, nullptr};  // twiddles per axis (float pairs)
  C* tw[3] = {nullptr, nullptr, nullptr};
  std::vector<int> rad[3];
  int rem = 0;
  C* fw = nullptr;
  C* fw2 = nullptr;  // type 2 with cuFFT: FFT output (fw keeps zero padding between executes)
  T* fac[3] = {nullptr, nullptr, nullptr};
  std::vector<T> horner;  // fitted kernel polynomials (kerevalmeth 1), [k][j]
  T* horner_d = nullptr;  // device copy of the same
  // sorted points and bin tables
  int* idx = nullptr;
  int* i0[3] = {nullptr, nullptr, nullptr};
  T* d[3] = {nullptr, nullptr, nullptr};
  int* rank = nullptr;
  size_t capM = 0;
  int* count = nullptr;
  int* start = nullptr;
  int* sub_start = nullptr;
  int* scan_tmp = nullptr;
  int* sub_to_bin = nullptr;
  SubHdr* sub_hdr = nullptr;  // [cap_sub] subproblem headers
  size_t cap_sub = 0;
  int* cls_count = nullptr;  // per (bin, class) counts for method 2 ordering
  size_t cap_cls = 0;
  bool cell_order = false;   // method 2 spreading over cell-ordered points (cell-run kernel)
  int* cls_start = nullptr;  // scanned (bin, cell) counts (cell order)
  int* cls_tmp = nullptr;    // scan scratch for cls_start
  size_t cap_cls_start = 0;
  int* sparse_count = nullptr;  // per-bin counter of the points on sparse cells
  size_t cap_sparse = 0;
  unsigned char* sub_dense = nullptr;  // per subproblem: starts on a dense cell (cell order)
  size_t cap_sub_dense = 0;
  int* sub_ndense = nullptr;  // cell order: leading dense points per subproblem
  // FP64 plans whose tolerance allows it run the spread/interp, FFT and
  // deconvolution chain in FP32: `lo` is that FP32 plan (null otherwise).
  // This side folds and rescales the points in FP64 (n_* arrays: caller
  // order, input of lo's sort) and converts c / fk (c32, fk32).
  Plan<float>* lo = nullptr;
  int* n_idx = nullptr;
  int* n_i0[3] = {nullptr, nullptr, nullptr};
  float* n_d[3] = {nullptr, nullptr, nullptr};
  size_t n_cap = 0;
  cplx_t<float>* c32 = nullptr;
  size_t c32_cap = 0;
  cplx_t<float>* fk32 = nullptr;
  // type 3: a spread-only plan onto the rescaled grid and an inner type-2
  // plan over that grid, the extents of sources and targets, phases
  Plan<T>* t3_spread = nullptr;
  Plan<T>* t3_inner = nullptr;
  double t3_tol = 0;
  double t3_C[3] = {0, 0, 0}, t3_D[3] = {0, 0, 0}, t3_gam[3] = {1, 1, 1}, t3_h[3] = {1, 1, 1};
  int t3_N = 0;                       // targets
  T* t3_xp[3] = {nullptr, nullptr, nullptr};   // rescaled sources (scratch of setpts)
  T* t3_tau[3] = {nullptr, nullptr, nullptr};  // inner type-2 frequencies (scratch of setpts)
  cplx_t<T>* t3_pre = nullptr;        // [M] prephase
  cplx_t<T>* t3_post = nullptr;       // [N] phase over phihat
  cplx_t<T>* t3_c = nullptr;          // [ntransf M] prephased strengths
  cplx_t<T>* t3_grid = nullptr;       // [ntransf nf] spread grid
  size_t t3_capM = 0, t3_capN = 0, t3_capG = 0;
  double* t3_part = nullptr;          // min/max partials (device)
  int* h_total = nullptr;  // pinned readback of the subproblem count
  // interpolation tile-wait status (SpreadArgs::status): host-mapped, two ints
  int* h_status = nullptr;
  int* d_status = nullptr;
  int tma_wait_test = 0;   // CUFINUFFT_TMA_WAIT_TEST=1 at makeplan
  int fp64_df = 0;         // FP64 type 2: double-float subproblem interpolation
  // execute as a CUDA graph (timing off): captured for one pair of caller
  // arrays and one plan state (`version` counts setpts / set_layout)
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  const void* g_c = nullptr;
  const void* g_fk = nullptr;
  unsigned version = 0, g_version = 0;
  // stage timing (extension): events recorded around each stage of execute
  bool timing = false;
  std::vector<cudaEvent_t> ev_pool;   // free events
  std::vector<cudaEvent_t> ev_live;   // groups of 4 per batch, not yet read
  double stage_ms[3] = {0, 0, 0};     // spread|interp, fft, deconv|amplify
  long long stage_batches = 0;
};

// Restores the caller's current device on scope exit.
struct DeviceGuard {
  int prev = -1;
  bool ok = false;
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    ok = cudaSetDevice(dev) == cudaSuccess;
  }
  ~DeviceGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

#define CFG_CUDA(call)                                             \
  do {                                                             \
    cudaError_t e_ = (call);                                       \
    if (e_ != cudaSuccess) {                                       \
      fprintf(stderr, "cufinufft: %s failed: %s\n", #call, cudaGetErrorString(e_)); \
      return e_ == cudaErrorMemoryAllocation ? CUFINUFFT_ERR_ALLOC : CUFINUFFT_ERR_CUDA; \
    }                                                              \
  } while (0)

#define CFG_CUFFT(call)                                            \
  do {                                                             \
    cufftResult r_ = (call);                                       \
    if (r_ != CUFFT_SUCCESS) {                                     \
      fprintf(stderr, "cufinufft: %s failed: cufftResult %d\n", #call, (int)r_); \
      return r_ == CUFFT_ALLOC_FAILED ? CUFINUFFT_ERR_ALLOC : CUFINUFFT_ERR_CUFFT; \
    }                                                              \
  } while (0)

template <typename T> constexpr bool is_single() { return sizeof(T) == 4; }

template <typename T> cufftType fft_type();
template <> inline cufftType fft_type<float>() { return CUFFT_C2C; }
template <> inline cufftType fft_type<double>() { return CUFFT_Z2Z; }

inline cufftResult fft_exec(cufftHandle h, float2* data, int dir) {
  return cufftExecC2C(h, (cufftComplex*)data, (cufftComplex*)data, dir);
}
inline cufftResult fft_exec(cufftHandle h, double2* data, int dir) {
  return cufftExecZ2Z(h, (cufftDoubleComplex*)data, (cufftDoubleComplex*)data, dir);
}
inline cufftResult fft_exec(cufftHandle h, float2* in, float2* out, int dir) {
  return cufftExecC2C(h, (cufftComplex*)in, (cufftComplex*)out, dir);
}
inline cufftResult fft_exec(cufftHandle h, double2* in, double2* out, int dir) {
  return cufftExecZ2Z(h, (cufftDoubleComplex*)in, (cufftDoubleComplex*)out, dir);
}

template <typename T> inline long long grid_cells(const Plan<T>* p) {
  return (long long)p->nf[0] * p->nf[1] * p->nf[2];
}

template <typename T>
inline AxisMap<T> axis_map(int nf, int ns) {
  AxisMap<T> a;
  const double S = (double)nf / (2.0 * M_PI);
  a.s_hi = (T)S;
  a.s_lo = (T)(S - (double)a.s_hi);
  a.o_lo = (T)(1.5 * nf);
  a.o_mid = (T)(0.5 * nf);
  a.o_hi = (T)(-0.5 * nf);
  a.half_int = ns / 2;
  a.half_frac = (ns % 2) ? T(0.5) : T(0);
  a.nf = nf;
  return a;
}

template <typename T>
inline SpreadArgs<T> spread_args(Plan<T>* p) {
  SpreadArgs<T> a;
  std::memset(&a, 0, sizeof(a));
  a.pts.idx = p->idx;
  for (int k = 0; k < 3; ++k) {
    a.pts.i0[k] = p->i0[k];
    a.pts.d[k] = p->d[k];
    a.bins.bs[k] = p->bs[k];
    a.bins.nb[k] = p->nb[k];
    a.g.nf[k] = p->nf[k];
  }
  a.pts.M = p->M;
  a.bins.nbins = p->nbins;
  a.bins.count = p->count;
  a.bins.start = p->start;
  a.bins.sub_start = p->sub_start;
  a.bins.sub_to_bin = p->sub_to_bin;
  a.bins.hdr = p->sub_hdr;
  a.bins.nsub = p->nsub;
  a.bins.maxsub = p->opts.gpu_maxsubprobsize;
  a.kc.beta = (T)p->sp.beta;
  a.kc.c = (T)p->sp.c;
  a.kc.e_beta = (T)std::exp(p->sp.beta);
  a.kc.bl2e = (T)(p->sp.beta * 1.44269504088896340736);
  a.kc.horner = p->horner.empty() ? 0 : 1;
  a.kc.coef_g = p->horner_d;
  for (size_t k = 0; k < p->horner.size() && k < (size_t)(kMaxHornerRows * kMaxNS); ++k) {
    a.kc.coef[k] = p->horner[k];
    if constexpr (sizeof(T) == 8) {
      // scaled by 2^-E, E = round(beta log2 e): kernel values ~1, see df_scale_exp
      const double v = std::ldexp(p->horner[k], -(int)std::lround(p->sp.beta * 1.44269504088896340736));
      a.kc.df.hi[k] = (float)v;
      a.kc.df.lo[k] = (float)(v - (double)a.kc.df.hi[k]);
    }
  }
  a.g.Nf = grid_cells(p);
  a.M = p->M;
  a.variant = p->variant;
  a.run = (p->cell_order && p->type == 1 && p->method == 2) ? 1 : 0;
  a.sub_dense = a.run ? p->sub_dense : nullptr;
  a.sub_ndense = a.run ? p->sub_ndense : nullptr;
  a.status = p->d_status;
  a.tma_wait_test = p->tma_wait_test;
  a.fp64_df = p->fp64_df;
  return a;
}

// A plan's whole execute, and moving its work (cuFFT plans included) to
// another stream (api.cu; used by the batch).
template <typename T>
int execute_plan(Plan<T>* p, cplx_t<T>* c, cplx_t<T>* fk);
template <typename T>
int plan_use_stream(Plan<T>* p, cudaStream_t s);

template <typename T>
inline cudaError_t run_spread(Plan<T>* p, const SpreadArgs<T>& a) {
  switch (p->dim) {
    case 1: return spread_dim<T, 1>(p->method, p->sp.ns, a, p->stream);
    case 2: return spread_dim<T, 2>(p->method, p->sp.ns, a, p->stream);
    default: return spread_dim<T, 3>(p->method, p->sp.ns, a, p->stream);
  }
}

template <typename T>
inline cudaError_t run_interp(Plan<T>* p, const SpreadArgs<T>& a) {
  switch (p->dim) {
    case 1: return interp_dim<T, 1>(p->method, p->sp.ns, a, p->stream);
    case 2: return interp_dim<T, 2>(p->method, p->sp.ns, a, p->stream);
    default: return interp_dim<T, 3>(p->method, p->sp.ns, a, p->stream);
  }
}

}  // namespace cfg

struct cufinufft_plan_s {
  cfg::Plan<double> p;
};
struct cufinufftf_plan_s {
  cfg::Plan<float> p;
};
