// api.cu -- the C ABI (include/cufinufft.h): plan, setpts, execute, destroy.
//
// Stage structure follows the reference (src/cufinufft.cu:78-637 and the
// per-dimension drivers src/{1d,2d,3d}/cufinufft*d.cu): makeplan sizes the
// fine grid, builds the cuFFT plan and the kernel's Fourier-series factors;
// setpts bin-sorts the points; execute loops over batches of maxbatchsize
// transforms doing spread -> FFT -> deconvolve (type 1) or amplify -> FFT ->
// interp (type 2).  All device work is queued on one stream per plan; no
// call inside execute synchronises the host.
#include <cufft.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <initializer_list>
#include <type_traits>
#include <new>
#include <vector>

#include "plan.h"
#include "selector_weights.h"

static_assert(sizeof(cfg::kSelParams) == sizeof(float) * CUFINUFFT_MLP_PARAMS,
              "selector weights do not match the network shape");

namespace cfg {

// Defaults, restating CUFINUFFT_DEFAULT_OPTS (src/cufinufft.cu:639-730).
int default_opts(int type, int dim, cufinufft_opts* opts) {
  if (opts == nullptr) return CUFINUFFT_ERR_ARG;
  opts->upsampfac = 2.0;
  opts->gpu_nstreams = 0;
  opts->gpu_sort = 1;
  opts->gpu_maxsubprobsize = 1024;
  opts->gpu_obinsizex = -1;
  opts->gpu_obinsizey = -1;
  opts->gpu_obinsizez = -1;
  opts->gpu_binsizex = -1;
  opts->gpu_binsizey = -1;
  opts->gpu_binsizez = -1;
  opts->gpu_spreadinterponly = 0;
  opts->gpu_kerevalmeth = 0;
  opts->gpu_device_id = 0;
  if (dim < 1 || dim > 3) return CUFINUFFT_ERR_ARG;
  // type 3 spreads as type 1 does (the reference reserves type 3 and
  // returns 1 here)
  if (type == 1 || type == 3) opts->gpu_method = 2;
  else if (type == 2) opts->gpu_method = 1;
  else return CUFINUFFT_ERR_GENERIC;
  return 0;
}

// Bin sizes, restating SETUP_BINSIZE (src/cufinufft.cu:17-73): a value < 0
// means "choose"; 1D 1024, 2D 32x32, 3D 16x16x2, 3D method 4 obin 8^3.
static void setup_binsize(int dim, cufinufft_opts* o) {
  if (dim == 1) {
    if (o->gpu_binsizex < 0) o->gpu_binsizex = 1024;
    o->gpu_binsizey = 1;
    o->gpu_binsizez = 1;
  } else if (dim == 2) {
    if (o->gpu_binsizex < 0) o->gpu_binsizex = 32;
    if (o->gpu_binsizey < 0) o->gpu_binsizey = 32;
    o->gpu_binsizez = 1;
  } else {
    if (o->gpu_method == 4) {
      if (o->gpu_obinsizex < 0) o->gpu_obinsizex = 8;
      if (o->gpu_obinsizey < 0) o->gpu_obinsizey = 8;
      if (o->gpu_obinsizez < 0) o->gpu_obinsizez = 8;
      if (o->gpu_binsizex < 0) o->gpu_binsizex = 4;
      if (o->gpu_binsizey < 0) o->gpu_binsizey = 4;
      if (o->gpu_binsizez < 0) o->gpu_binsizez = 4;
    } else {
      if (o->gpu_binsizex < 0) o->gpu_binsizex = 16;
      if (o->gpu_binsizey < 0) o->gpu_binsizey = 16;
      if (o->gpu_binsizez < 0) o->gpu_binsizez = 2;
    }
  }
}

template <typename T> static void free_points(Plan<T>* p) {
  cudaFree(p->idx);
  cudaFree(p->rank);
  p->idx = p->rank = nullptr;
  for (int k = 0; k < 3; ++k) {
    cudaFree(p->i0[k]);
    cudaFree(p->d[k]);
    p->i0[k] = nullptr;
    p->d[k] = nullptr;
  }
  p->capM = 0;
}

template <typename T> static void drop_graph(Plan<T>* p) {
  if (p->gexec) cudaGraphExecDestroy(p->gexec);
  if (p->graph) cudaGraphDestroy(p->graph);
  p->gexec = nullptr;
  p->graph = nullptr;
}

template <typename T> static void release(Plan<T>* p) {
  if (p->lo) {
    release(p->lo);
    delete p->lo;
    p->lo = nullptr;
  }
  Plan<T>** const t3[2] = {&p->t3_spread, &p->t3_inner};
  for (Plan<T>** q : t3) {
    if (*q) {
      release(*q);
      delete *q;
      *q = nullptr;
    }
  }
  for (int k = 0; k < 3; ++k) {
    cudaFree(p->t3_xp[k]);
    cudaFree(p->t3_tau[k]);
    p->t3_xp[k] = p->t3_tau[k] = nullptr;
  }
  cudaFree(p->t3_pre);
  cudaFree(p->t3_post);
  cudaFree(p->t3_c);
  cudaFree(p->t3_grid);
  cudaFree(p->t3_part);
  p->t3_pre = p->t3_post = p->t3_c = p->t3_grid = nullptr;
  p->t3_part = nullptr;
  p->t3_capM = p->t3_capN = p->t3_capG = 0;
  cudaFree(p->n_idx);
  p->n_idx = nullptr;
  for (int k = 0; k < 3; ++k) {
    cudaFree(p->n_i0[k]);
    cudaFree(p->n_d[k]);
    p->n_i0[k] = nullptr;
    p->n_d[k] = nullptr;
  }
  p->n_cap = 0;
  cudaFree(p->c32);
  p->c32 = nullptr;
  p->c32_cap = 0;
  cudaFree(p->fk32);
  p->fk32 = nullptr;
  drop_graph(p);
  if (p->have_fft) cufftDestroy(p->fft);
  if (p->have_fft_rem) cufftDestroy(p->fft_rem);
  p->have_fft = p->have_fft_rem = false;
  cudaFree(p->fw);
  p->fw = nullptr;
  cudaFree(p->fw2);
  p->fw2 = nullptr;
  for (int k = 0; k < 3; ++k) {
    cudaFree(p->fac[k]);
    p->fac[k] = nullptr;
    cudaFree(p->tw[k]);
    p->tw[k] = nullptr;
    p->rad[k].clear();
  }
  p->line_fft = false;
  p->half_fft = false;
  p->df_fft = false;
  cudaFree(p->df_tmp);
  p->df_tmp = nullptr;
  for (int k = 0; k < 2; ++k) {
    cudaFree(p->df_tw[k]);
    p->df_tw[k] = nullptr;
  }
  p->horner.clear();
  cudaFree(p->sel_buf);
  p->sel_buf = nullptr;
  cudaFree(p->horner_d);
  p->horner_d = nullptr;
  free_points(p);
  cudaFree(p->count);
  cudaFree(p->start);
  cudaFree(p->sub_start);
  cudaFree(p->scan_tmp);
  cudaFree(p->sub_to_bin);
  cudaFree(p->sub_hdr);
  p->sub_hdr = nullptr;
  p->count = p->start = p->sub_start = p->scan_tmp = p->sub_to_bin = nullptr;
  p->cap_sub = 0;
  cudaFree(p->cls_count);
  p->cls_count = nullptr;
  p->cap_cls = 0;
  cudaFree(p->cls_start);
  cudaFree(p->cls_tmp);
  p->cls_start = p->cls_tmp = nullptr;
  p->cap_cls_start = 0;
  cudaFree(p->sparse_count);
  p->sparse_count = nullptr;
  p->cap_sparse = 0;
  cudaFree(p->sub_dense);
  cudaFree(p->sub_ndense);
  p->sub_dense = nullptr;
  p->sub_ndense = nullptr;
  p->cap_sub_dense = 0;
  if (p->h_total) cudaFreeHost(p->h_total);
  p->h_total = nullptr;
  if (p->h_status) cudaFreeHost(p->h_status);
  p->h_status = nullptr;
  p->d_status = nullptr;
  for (cudaEvent_t e : p->ev_pool) cudaEventDestroy(e);
  for (cudaEvent_t e : p->ev_live) cudaEventDestroy(e);
  p->ev_pool.clear();
  p->ev_live.clear();
  if (p->own) cudaStreamDestroy(p->own);
  p->own = p->stream = nullptr;
  p->planned = p->pts_set = false;
}

template <typename T>
static int make_fft(Plan<T>* p, int batch, cufftHandle* h) {
  int n[3], dist = (int)grid_cells(p);
  for (int k = 0; k < p->dim; ++k) n[k] = p->nf[p->dim - 1 - k];  // slowest first
  CFG_CUFFT(cufftPlanMany(h, p->dim, n, n, 1, dist, n, 1, dist, fft_type<T>(), batch));
  CFG_CUFFT(cufftSetStream(*h, p->stream));
  return 0;
}

// ---------------------------------------------------------------------------
// Pruned line FFTs (fftpass.cu): with CUFINUFFT_FFT=line, used when every
// axis length is 2,3,5-smooth and fits one block's shared memory (8192 FP32
// / 4096 FP64 points); otherwise the whole-grid cuFFT path runs.

// Radices (8, 4, 2, 5, 3) whose product is L; empty if L has another factor.
static std::vector<int> radix_plan(int L) {
  std::vector<int> r;
  if (L < 2) return r;
  for (int R : {8, 4, 2, 5, 3})
    while (L % R == 0) {
      r.push_back(R);
      L /= R;
    }
  if (L != 1) r.clear();
  return r;
}

template <typename T>
static bool use_line_fft(const Plan<T>* p) {
  const char* v = std::getenv("CUFINUFFT_FFT");
  if (v == nullptr || std::strcmp(v, "line") != 0) return false;
  for (int k = 0; k < p->dim; ++k) {
    const std::vector<int> r = radix_plan(p->nf[k]);
    if (p->nf[k] > line_fft_cap<T>() || r.empty() || r.size() > 24) return false;
  }
  return true;
}

// Pruned power-of-two passes (halffft.cu): every axis nf a power of two in
// [256, 2048] with at most nf/2 modes (always so at upsampfac 2); selected
// by CUFINUFFT_FFT=half.
template <typename T>
static bool use_half_fft(const Plan<T>* p) {
  const char* v = std::getenv("CUFINUFFT_FFT");
  if (!v || std::strcmp(v, "half") != 0) return false;
  for (int k = 0; k < p->dim; ++k)
    if (!half_fft_size_ok(p->nf[k]) || 2 * p->N[k] > p->nf[k]) return false;
  return true;
}

// Double-float FFT (fft_df.cu) for FP64 plans of dimension 2 whose fine
// grid sides are powers of two <= 4096, when the tol gate allows it and no
// other FFT form was asked for.
template <typename T>
static bool use_df_fft(const Plan<T>* p) {
  if (sizeof(T) != 8 || !p->df_fft_ok || p->dim != 2 || (p->type != 1 && p->type != 2)) return false;
  if (std::getenv("CUFINUFFT_FFT")) return false;  // line / half forms asked for
  return fft_df_size_ok(p->nf[0]) && fft_df_size_ok(p->nf[1]);
}

// Its scratch grids and, per axis, W^k = exp(iflag 2 pi i k / nf), k < nf/2,
// computed in extended precision and split into float pairs.
template <typename T>
static int make_df_fft(Plan<T>* p) {
  const long double two_pi = 6.283185307179586476925286766559005768L;
  const size_t Nf = (size_t)p->nf[0] * p->nf[1];
  CFG_CUDA(cudaMalloc(&p->df_tmp, sizeof(double2) * Nf * p->maxbatch));
  for (int k = 0; k < 2; ++k) {
    const int n = p->nf[k];
    std::vector<float4> h((size_t)n / 2);
    for (int m = 0; m < n / 2; ++m) {
      const long double a = two_pi * (long double)m / (long double)n * (p->iflag >= 0 ? 1 : -1);
      const double re = (double)cosl(a), im = (double)sinl(a);
      const float rh = (float)re, ih = (float)im;
      h[m] = make_float4(rh, (float)(re - (double)rh), ih, (float)(im - (double)ih));
    }
    CFG_CUDA(cudaMalloc(&p->df_tw[k], sizeof(float4) * h.size()));
    CFG_CUDA(cudaMemcpyAsync(p->df_tw[k], h.data(), sizeof(float4) * h.size(), cudaMemcpyHostToDevice,
                             p->stream));
  }
  CFG_CUDA(cudaStreamSynchronize(p->stream));
  return 0;
}

// 2D transform of B grids in -> out through the scratch: rows along x, a
// transpose, rows along y, a transpose back.  in may equal out (type 1).
template <typename T>
static cudaError_t df_fft_exec(Plan<T>* p, const cplx_t<T>* in, cplx_t<T>* out, int B) {
  if constexpr (sizeof(T) == 8) {
    const int nx = p->nf[0], ny = p->nf[1];
    cudaError_t e = launch_fft_df_rows(in, p->df_tmp, nx, (long long)B * ny, p->df_tw[0], p->stream);
    if (e == cudaSuccess) e = launch_transpose_d2(p->df_tmp, out, ny, nx, B, p->stream);
    if (e == cudaSuccess) e = launch_fft_df_rows(out, p->df_tmp, ny, (long long)B * nx, p->df_tw[1], p->stream);
    if (e == cudaSuccess) e = launch_transpose_d2(p->df_tmp, out, nx, ny, B, p->stream);
    return e;
  } else {
    (void)p; (void)in; (void)out; (void)B;
    return cudaErrorInvalidValue;
  }
}

// Twiddle tables W^m = exp(iflag 2 pi i m / nf_d), m < nf_d, per axis, in
// extended precision on the host.
template <typename T>
static int make_twiddles(Plan<T>* p) {
  const long double two_pi = 6.283185307179586476925286766559005768L;
  for (int k = 0; k < p->dim; ++k) {
    const int L = p->nf[k];
    std::vector<cplx_t<T>> h((size_t)L);
    for (int m = 0; m < L; ++m) {
      const long double ang = two_pi * (long double)m / (long double)L;
      h[m].x = (T)(double)cosl(ang);
      h[m].y = (T)(double)((long double)p->iflag * sinl(ang));
    }
    CFG_CUDA(cudaMalloc(&p->tw[k], sizeof(cplx_t<T>) * (size_t)L));
    CFG_CUDA(cudaMemcpy(p->tw[k], h.data(), sizeof(cplx_t<T>) * (size_t)L, cudaMemcpyHostToDevice));
  }
  return 0;
}

// The passes of one batch of B transforms (see halffft.cu): type 2 modes fk
// -> x pass (amplification fused) -> y -> z -> grid fw2, intermediates in
// fw; type 1 grid fw -> z -> y -> x pass (deconvolution fused) -> modes fk,
// intermediates in fw2.
template <typename T>
static std::vector<HalfPass<T>> half_passes(const Plan<T>* p, cplx_t<T>* fk, int B) {
  const long long L0 = p->nf[0], L1 = p->nf[1], L2 = p->nf[2];
  const int N0 = p->N[0], N1 = p->N[1], N2 = p->N[2];
  const long long Nm = (long long)N0 * N1 * N2, Nf = L0 * L1 * L2;
  auto base = [&](int kind, int axis) {
    HalfPass<T> a;
    std::memset(&a, 0, sizeof(a));
    a.kind = kind;
    a.Mp = half_fft_mp(p->nf[axis]);
    a.F = p->nf[axis] / a.Mp;
    a.Fb = std::min(a.F, 4);
    a.dir = p->iflag;
    a.N = p->N[axis];
    a.tw = p->tw[axis];
    a.ntr = B;
    a.nouter = 1;
    a.Na = 1;
    return a;
  };
  std::vector<HalfPass<T>> v;
  if (p->type == 2) {
    cplx_t<T>* t1 = p->fw;
    cplx_t<T>* t2 = p->fw + (size_t)B * N2 * N1 * L0;
    HalfPass<T> x = base(kHalfT2Rows, 0);
    x.in = fk;
    x.in_tr = Nm;
    x.in_row = N0;
    x.nlines = N1 * N2;
    x.fac = p->fac[0];
    x.fac_a = p->dim > 1 ? p->fac[1] : nullptr;
    x.fac_b = p->dim > 2 ? p->fac[2] : nullptr;
    x.Na = N1;
    x.out = p->dim == 1 ? p->fw2 : t1;
    x.out_tr = p->dim == 1 ? Nf : (long long)N2 * N1 * L0;
    x.out_row = L0;
    v.push_back(x);
    if (p->dim >= 2) {
      HalfPass<T> y = base(kHalfT2Cols, 1);
      y.in = t1;
      y.in_tr = (long long)N2 * N1 * L0;
      y.in_row = L0;
      y.in_plane = (long long)N1 * L0;
      y.ncols = (int)L0;
      y.nouter = p->dim == 3 ? N2 : 1;
      y.out = p->dim == 2 ? p->fw2 : t2;
      y.out_tr = p->dim == 2 ? Nf : (long long)N2 * L1 * L0;
      y.out_row = L0;
      y.out_plane = L1 * L0;
      y.pitch = half_col_pitch<T>(N1, y.Mp);
      v.push_back(y);
    }
    if (p->dim == 3) {
      HalfPass<T> z = base(kHalfT2Cols, 2);
      z.in = t2;
      z.in_tr = (long long)N2 * L1 * L0;
      z.in_row = L1 * L0;
      z.ncols = (int)(L1 * L0);
      z.out = p->fw2;
      z.out_tr = Nf;
      z.out_row = L1 * L0;
      z.pitch = half_col_pitch<T>(N2, z.Mp);
      v.push_back(z);
    }
    return v;
  }
  cplx_t<T>* s2 = p->fw2;
  cplx_t<T>* s1 = p->dim == 3 ? p->fw2 + (size_t)B * N2 * L1 * L0 : p->fw2;
  if (p->dim == 3) {
    HalfPass<T> z = base(kHalfT1Cols, 2);
    z.in = p->fw;
    z.in_tr = Nf;
    z.in_row = L1 * L0;
    z.ncols = (int)(L1 * L0);
    z.out = s2;
    z.out_tr = (long long)N2 * L1 * L0;
    z.out_row = L1 * L0;
    z.pitch = half_col_pitch<T>(z.Mp, z.Mp);
    v.push_back(z);
  }
  if (p->dim >= 2) {
    HalfPass<T> y = base(kHalfT1Cols, 1);
    y.in = p->dim == 3 ? s2 : p->fw;
    y.in_tr = p->dim == 3 ? (long long)N2 * L1 * L0 : Nf;
    y.in_row = L0;
    y.in_plane = L1 * L0;
    y.ncols = (int)L0;
    y.nouter = p->dim == 3 ? N2 : 1;
    y.out = s1;
    y.out_tr = (long long)N2 * N1 * L0;
    y.out_row = L0;
    y.out_plane = (long long)N1 * L0;
    y.pitch = half_col_pitch<T>(y.Mp, y.Mp);
    v.push_back(y);
  }
  HalfPass<T> x = base(kHalfT1Rows, 0);
  x.in = p->dim == 1 ? p->fw : s1;
  x.in_tr = p->dim == 1 ? Nf : (long long)N2 * N1 * L0;
  x.in_row = L0;
  x.nlines = N1 * N2;
  x.out = fk;
  x.out_tr = Nm;
  x.out_row = N0;
  x.fac = p->fac[0];
  x.fac_a = p->dim > 1 ? p->fac[1] : nullptr;
  x.fac_b = p->dim > 2 ? p->fac[2] : nullptr;
  x.Na = N1;
  v.push_back(x);
  return v;
}

template <typename T>
static int make_line_fft(Plan<T>* p) {
  const long double two_pi = 6.283185307179586476925286766559005768L;
  for (int k = 0; k < p->dim; ++k) {
    const int L = p->nf[k];
    p->rad[k] = radix_plan(L);
    std::vector<cplx_t<T>> h((size_t)L);
    for (int m = 0; m < L; ++m) {
      const long double ang = two_pi * (long double)m / (long double)L;
      h[m].x = (T)(double)cosl(ang);
      h[m].y = (T)(double)((long double)p->iflag * sinl(ang));
    }
    CFG_CUDA(cudaMalloc(&p->tw[k], sizeof(cplx_t<T>) * (size_t)L));
    CFG_CUDA(cudaMemcpy(p->tw[k], h.data(), sizeof(cplx_t<T>) * (size_t)L, cudaMemcpyHostToDevice));
  }
  CFG_CUDA(line_fft_prepare<T>());
  p->line_fft = true;
  return 0;
}

// Lines per block: a power of two with G * L at most half the cap (two
// padded buffers of ~34 KB, three blocks per SM); longer lines run one per
// block.
//
// Power-of-two lines of at least 16 points take the register-resident kernel:
// block = G * L / 16 threads, G * L <= 4096 FP32 / 2048 FP64 points.  Along
// x (contiguous lines) G is lowered (down to 64 threads) while that leaves
// fewer than ~6 blocks per SM.  Along y and z a block's G lines are G
// adjacent elements of each grid row it reads, so G is never lowered, and
// lines longer than 1024 FP32 / 512 FP64 points may take twice the points
// (G = 4 / 2: 32-byte row segments).
template <typename T>
static LineArgs<T> line_base(const Plan<T>* p, int axis, int B, int nlines) {
  LineArgs<T> a;
  std::memset(&a, 0, sizeof(a));
  a.L = p->nf[axis];
  a.dir = p->iflag;
  const int base_elems = line_fft_p2_elems<T>();
  const int p2_elems = (axis > 0 && a.L > base_elems / 4) ? 2 * base_elems : base_elems;
  if (a.L >= 16 && (a.L & (a.L - 1)) == 0 && a.L <= p2_elems) {
    int G = p2_elems / a.L;
    const long long want = 152LL * 6;
    while (axis == 0 && G > 1 && G * a.L / 16 > 64 && (long long)((nlines + G - 1) / G) * B < want)
      G /= 2;
    int lg = 0;
    while ((1 << lg) < G) ++lg;
    a.p2 = 1;
    a.G = G;
    a.log2G = lg;
    a.nlines = nlines;
    a.ntr = B;
    a.tw = p->tw[axis];
    return a;
  }
  const int cap = line_fft_cap<T>() / 2;
  int G = 1, lg = 0;
  while (G < 256 && G < nlines && 2 * G * a.L <= cap) {
    G *= 2;
    ++lg;
  }
  a.G = G;
  a.log2G = lg;
  a.nlines = nlines;
  a.ntr = B;
  a.nrad = (int)p->rad[axis].size();
  for (int s = 0; s < a.nrad; ++s) a.rad[s] = p->rad[axis][s];
  a.tw = p->tw[axis];
  return a;
}

static LineSide line_side(long long st, long long sa, long long sb, long long sp, int pmode, int Np) {
  LineSide s;
  std::memset(&s, 0, sizeof(s));
  s.st = st;
  s.sa = sa;
  s.sb = sb;
  s.sp = sp;
  s.pmode = pmode;
  s.Np = Np;
  return s;
}
static void corner_a(LineSide* s, int N, int nf) {
  s->acorner = 1;
  s->Na = N;
  s->nfa = nf;
}
static void corner_b(LineSide* s, int N, int nf) {
  s->bcorner = 1;
  s->Nb = N;
  s->nfb = nf;
}

// The axis passes of one batch of B transforms, in order.  Type 2: modes fk
// -> grid fw, the first pass fused with the amplification.  Type 1: grid fw
// -> modes fk, the last pass fused with the deconvolution.
template <typename T>
static std::vector<LineArgs<T>> line_passes(const Plan<T>* p, cplx_t<T>* fk, int B) {
  const long long Nf = grid_cells(p);
  const long long Nm = (long long)p->N[0] * p->N[1] * p->N[2];
  const int n0 = p->nf[0], n1 = p->nf[1], n2 = p->nf[2];
  const int N0 = p->N[0], N1 = p->N[1], N2 = p->N[2];
  const long long n01 = (long long)n0 * n1, N01 = (long long)N0 * N1;
  cplx_t<T>* fw = p->fw;
  std::vector<LineArgs<T>> v;
  LineArgs<T> a;
  if (p->type == 2) {
    if (p->dim == 1) {
      a = line_base(p, 0, B, 1);
      a.A = 1;
      a.in = fk;
      a.out = fw;
      a.si = line_side(Nm, 0, 0, 1, 1, N0);
      a.so = line_side(Nf, 0, 0, 1, 0, 0);
      a.fp = p->fac[0];
      v.push_back(a);
    } else if (p->dim == 2) {
      a = line_base(p, 1, B, N0);  // y over the mode columns
      a.A = N0;
      a.in = fk;
      a.out = fw;
      a.si = line_side(Nm, 1, 0, N0, 1, N1);
      a.so = line_side(Nf, 1, 0, n0, 0, 0);
      corner_a(&a.so, N0, n0);
      a.fa = p->fac[0];
      a.fp = p->fac[1];
      v.push_back(a);
      a = line_base(p, 0, B, n1);  // x over every row
      a.A = n1;
      a.in = fw;
      a.out = fw;
      a.si = line_side(Nf, n0, 0, 1, 2, N0);
      a.so = line_side(Nf, n0, 0, 1, 0, 0);
      v.push_back(a);
    } else {
      a = line_base(p, 2, B, (int)N01);  // z over the (x, y) mode columns
      a.A = N0;
      a.in = fk;
      a.out = fw;
      a.si = line_side(Nm, 1, N0, N01, 1, N2);
      a.so = line_side(Nf, 1, n0, n01, 0, 0);
      corner_a(&a.so, N0, n0);
      corner_b(&a.so, N1, n1);
      a.fa = p->fac[0];
      a.fb = p->fac[1];
      a.fp = p->fac[2];
      v.push_back(a);
      a = line_base(p, 1, B, N0 * n2);  // y over (x mode column, every z)
      a.A = N0;
      a.in = fw;
      a.out = fw;
      a.si = line_side(Nf, 1, n01, n0, 2, N1);
      corner_a(&a.si, N0, n0);
      a.so = line_side(Nf, 1, n01, n0, 0, 0);
      corner_a(&a.so, N0, n0);
      v.push_back(a);
      a = line_base(p, 0, B, n1 * n2);  // x over every (y, z) row
      a.A = n1;
      a.in = fw;
      a.out = fw;
      a.si = line_side(Nf, n0, n01, 1, 2, N0);
      a.so = line_side(Nf, n0, n01, 1, 0, 0);
      v.push_back(a);
    }
  } else {
    if (p->dim == 1) {
      a = line_base(p, 0, B, 1);
      a.A = 1;
      a.in = fw;
      a.out = fk;
      a.si = line_side(Nf, 0, 0, 1, 0, 0);
      a.so = line_side(Nm, 0, 0, 1, 1, N0);
      a.fp = p->fac[0];
      a.fac_on_out = 1;
      v.push_back(a);
    } else if (p->dim == 2) {
      a = line_base(p, 0, B, n1);  // x over every row, keep the x modes
      a.A = n1;
      a.in = fw;
      a.out = fw;
      a.si = line_side(Nf, n0, 0, 1, 0, 0);
      a.so = line_side(Nf, n0, 0, 1, 2, N0);
      v.push_back(a);
      a = line_base(p, 1, B, N0);  // y over the x mode columns -> fk
      a.A = N0;
      a.in = fw;
      a.out = fk;
      a.si = line_side(Nf, 1, 0, n0, 0, 0);
      corner_a(&a.si, N0, n0);
      a.so = line_side(Nm, 1, 0, N0, 1, N1);
      a.fa = p->fac[0];
      a.fp = p->fac[1];
      a.fac_on_out = 1;
      v.push_back(a);
    } else {
      a = line_base(p, 0, B, n1 * n2);  // x over every (y, z) row
      a.A = n1;
      a.in = fw;
      a.out = fw;
      a.si = line_side(Nf, n0, n01, 1, 0, 0);
      a.so = line_side(Nf, n0, n01, 1, 2, N0);
      v.push_back(a);
      a = line_base(p, 1, B, N0 * n2);  // y over (x mode column, every z)
      a.A = N0;
      a.in = fw;
      a.out = fw;
      a.si = line_side(Nf, 1, n01, n0, 0, 0);
      corner_a(&a.si, N0, n0);
      a.so = line_side(Nf, 1, n01, n0, 2, N1);
      corner_a(&a.so, N0, n0);
      v.push_back(a);
      a = line_base(p, 2, B, (int)N01);  // z over the (x, y) mode columns -> fk
      a.A = N0;
      a.in = fw;
      a.out = fk;
      a.si = line_side(Nf, 1, n0, n01, 0, 0);
      corner_a(&a.si, N0, n0);
      corner_b(&a.si, N1, n1);
      a.so = line_side(Nm, 1, N0, N01, 1, N2);
      a.fa = p->fac[0];
      a.fb = p->fac[1];
      a.fp = p->fac[2];
      a.fac_on_out = 1;
      v.push_back(a);
    }
  }
  return v;
}

static int max_smem_optin(int device);

// Kernel-width rule of the next makeplan calls on this thread (-1: from
// CUFINUFFT_WIDTH_RULE, "tol" or "1" for the tolerance-meeting rule, else
// the reference's).
static thread_local int t_width_rule = -1;

static int width_rule_now() {
  if (t_width_rule >= 0) return t_width_rule;
  const char* v = std::getenv("CUFINUFFT_WIDTH_RULE");
  if (v && (std::strcmp(v, "tol") == 0 || std::strcmp(v, "1") == 0)) return 1;
  return 0;
}

static int set_width_rule(int rule, int* previous) {
  if (rule < -1 || rule > 1) return CUFINUFFT_ERR_ARG;
  if (previous) *previous = t_width_rule;
  t_width_rule = rule;
  return 0;
}

// sp_fixed: the kernel (width and shape) chosen by an FP64 plan for its FP32
// chain, instead of this precision's rule.
template <typename T>
static int makeplan_impl(Plan<T>* p, int type, int dim, const int* nmodes, int iflag, int ntransf,
                         double tol, int maxbatchsize, const cufinufft_opts* opts,
                         const SpreaderParams* sp_fixed = nullptr) {
  p->type = type;
  p->dim = dim;
  p->width_rule = width_rule_now();
  if (const char* v = std::getenv("CUFINUFFT_KERNEL_VARIANT")) {
    const int k = std::atoi(v);
    p->variant = (k == 1 || k == 2) ? k : 0;
  }
  if (opts) p->opts = *opts;
  else default_opts(type, dim, &p->opts);
  int ier = setup_spreader(tol, p->opts.upsampfac, p->opts.gpu_kerevalmeth, is_single<T>(), &p->sp,
                           p->width_rule, dim);
  if (ier > 1) return ier;
  if (sp_fixed) p->sp = *sp_fixed;
  for (int k = 0; k < dim; ++k) p->N[k] = nmodes[k];
  setup_binsize(dim, &p->opts);

  // method actually run (src/2d/spread2d_wrapper.cu:99-164,
  // src/3d/spread3d_wrapper.cu:101-160, src/*/interp*_wrapper.cu):
  int m = p->opts.gpu_method;
  if (m == 0) {
    // extension: gpu_method 0 lets the library choose (the reference rejects
    // 0).  Measured on GB300: spreading is fastest NU-point driven into the
    // grid (vector reductions in L2); interpolation from shared-memory tiles
    // in 2D/3D.
    m = (type == 1 || dim == 1) ? 1 : 2;
    p->opts.gpu_method = m;
    p->opts.gpu_sort = 1;
    p->auto_method = true;
  }
  p->sort = p->opts.gpu_sort;
  int bins_from_obin = 0;
  if (type == 1) {
    if (m == 1 || m == 2) p->method = m;
    else if (m == 3 && dim == 2) {
      // the reference's method 3 sorts points by cell inside bins for
      // clustered 2D data (src/2d/spread2d_wrapper_paul.cu); here it is the
      // cell-run spread over cell-ordered points
      p->method = 2;
      p->cell_order = true;
    }
    else if (m == 4 && dim == 3) { p->method = 2; bins_from_obin = 1; }
    else p->method = 0;
  } else {
    if (m == 1) p->method = 1;
    else if (m == 2 && dim > 1) p->method = 2;
    else p->method = 0;
  }
  if (p->method == 2) p->sort = 1;

  const int obin[3] = {p->opts.gpu_obinsizex, p->opts.gpu_obinsizey, p->opts.gpu_obinsizez};
  p->spread_only = p->opts.gpu_spreadinterponly != 0;
  for (int k = 0; k < dim; ++k) {
    if (bins_from_obin && obin[k] <= 0) return CUFINUFFT_ERR_ARG;
    if (p->spread_only) {
      // spread/interpolation only: nmodes is the caller's grid itself; it
      // must hold a kernel's support twice (as set_nf_type12's grids do),
      // and for method 4 whole output bins
      if (p->N[k] < 2 * p->sp.ns) return CUFINUFFT_ERR_ARG;
      if (bins_from_obin && p->N[k] % obin[k] != 0) return CUFINUFFT_ERR_ARG;
      p->nf[k] = p->N[k];
    } else {
      p->nf[k] = set_nf_type12(p->N[k], p->opts.upsampfac, p->sp.ns, m, bins_from_obin ? obin[k] : 1);
    }
  }
  const int bsz[3] = {p->opts.gpu_binsizex, p->opts.gpu_binsizey, p->opts.gpu_binsizez};
  for (int k = 0; k < 3; ++k) {
    if (k < dim) {
      int b = bins_from_obin ? obin[k] : bsz[k];
      if (b <= 0) return CUFINUFFT_ERR_GENERIC;  // reference: "invalid binsize"
      if (b > p->nf[k]) b = p->nf[k];
      p->bs[k] = b;
      p->nb[k] = (p->nf[k] + b - 1) / b;
    } else {
      p->bs[k] = 1;
      p->nb[k] = 1;
    }
  }
  long long nbins = (long long)p->nb[0] * p->nb[1] * p->nb[2];
  if (nbins > (1LL << 24)) return CUFINUFFT_ERR_ARG;
  p->nbins = (int)nbins;
  if (p->cell_order && (!cell_order_fits(p, p->bs, nbins) ||
                        run_smem_bytes(p, p->bs) > (size_t)max_smem_optin(p->device)))
    p->cell_order = false;  // too many (bin, cell) keys or taps: plain method 2
  if (p->method == 2 && p->opts.gpu_maxsubprobsize <= 0) return CUFINUFFT_ERR_ARG;

  p->iflag = iflag >= 0 ? 1 : -1;
  p->ntransf = ntransf;
  if (type == 2) tma_encoder();  // first lookup outside any capture of execute
  if (maxbatchsize == 0) maxbatchsize = std::min(ntransf, 8);
  p->maxbatch = std::min(maxbatchsize, ntransf);
  p->rem = ntransf % p->maxbatch;

  CFG_CUDA(cudaStreamCreate(&p->own));  // blocking: ordered after the legacy default stream
  p->stream = p->own;
  CFG_CUDA(cudaMallocHost(&p->h_total, sizeof(int)));
  if (type == 2) {
    CFG_CUDA(cudaHostAlloc(&p->h_status, 2 * sizeof(int), cudaHostAllocMapped));
    p->h_status[0] = p->h_status[1] = 0;
    CFG_CUDA(cudaHostGetDevicePointer(&p->d_status, p->h_status, 0));
    if (const char* v = std::getenv("CUFINUFFT_TMA_WAIT_TEST")) p->tma_wait_test = v[0] == '1';
    if constexpr (sizeof(T) == 8) {
      // double-float interpolation: ~2^-46 relative, below every tol >= 1e-13;
      // CUFINUFFT_FP64_DF=0 keeps FP64 instructions, =1 takes it at any tol
      const char* v = std::getenv("CUFINUFFT_FP64_DF");
      p->fp64_df = v && v[0] == '0' ? 0 : (v && v[0] == '1' ? 1 : (tol >= 1e-13 ? 1 : 0));
    }
  }
  if constexpr (sizeof(T) == 8) {
    // double-float FFT of 2D power-of-two grids (types 1 and 2), under the
    // same tol gate; CUFINUFFT_FP64_DF_FFT=0 keeps cuFFT's Z2Z
    const char* v = std::getenv("CUFINUFFT_FP64_DF_FFT");
    const char* w = std::getenv("CUFINUFFT_FP64_DF");
    const bool gate = w && w[0] == '0' ? false : (w && w[0] == '1' ? true : tol >= 1e-13);
    p->df_fft_ok = (v && v[0] == '0') ? 0 : (gate ? 1 : 0);
  }

  const long long Nf = grid_cells(p);
  CFG_CUDA(cudaMalloc(&p->count, sizeof(int) * (size_t)p->nbins));
  CFG_CUDA(cudaMalloc(&p->start, sizeof(int) * ((size_t)p->nbins + 1)));
  CFG_CUDA(cudaMalloc(&p->sub_start, sizeof(int) * ((size_t)p->nbins + 1)));
  CFG_CUDA(cudaMalloc(&p->scan_tmp, sizeof(int) * (size_t)scan_tmp_ints(p->nbins)));
  if (p->spread_only) {
    // no grid, FFT or kernel Fourier series: execute spreads into / reads
    // from the caller's fk
    if (p->opts.gpu_kerevalmeth == 1) {
      const int deg = horner_degree<T>(p->sp.ns);
      std::vector<double> cd = horner_fit(p->sp, deg);
      p->horner.assign(cd.begin(), cd.end());
      CFG_CUDA(cudaMalloc(&p->horner_d, sizeof(T) * p->horner.size()));
      CFG_CUDA(cudaMemcpyAsync(p->horner_d, p->horner.data(), sizeof(T) * p->horner.size(),
                               cudaMemcpyHostToDevice, p->stream));
    }
    CFG_CUDA(cudaStreamSynchronize(p->stream));
    p->planned = true;
    return 0;
  }
  CFG_CUDA(cudaMalloc(&p->fw, sizeof(cplx_t<T>) * (size_t)Nf * p->maxbatch));
  for (int k = 0; k < dim; ++k) CFG_CUDA(cudaMalloc(&p->fac[k], sizeof(T) * (size_t)p->N[k]));

  int e = 0;
  if (use_df_fft(p)) {
    // double-float FFT: no cuFFT plan; scratch for the passes, twiddles per axis
    e = make_df_fft(p);
    if (e) return e;
    if (type == 2) {
      // as with cuFFT: fw holds only the amplified modes over zero padding,
      // the transform writes fw2, interpolation reads fw2
      CFG_CUDA(cudaMalloc(&p->fw2, sizeof(cplx_t<T>) * (size_t)Nf * p->maxbatch));
      CFG_CUDA(cudaMemsetAsync(p->fw, 0, sizeof(cplx_t<T>) * (size_t)Nf * p->maxbatch, p->stream));
    }
    p->df_fft = true;
  } else if (use_half_fft(p)) {
    // pruned power-of-two passes: no cuFFT plan; type 2 grid in fw2
    // (intermediates in fw), type 1 intermediates in fw2
    e = make_twiddles(p);
    if (e) return e;
    CFG_CUDA(cudaMalloc(&p->fw2, sizeof(cplx_t<T>) * (size_t)Nf * p->maxbatch));
    p->half_fft = true;
  } else if (use_line_fft(p)) {
    e = make_line_fft(p);
    if (e) return e;
  } else {
    if (type == 2) {
      // out-of-place FFT: fw holds only the amplified modes over padding
      // zeroed once here, the FFT writes fw2, interpolation reads fw2
      CFG_CUDA(cudaMalloc(&p->fw2, sizeof(cplx_t<T>) * (size_t)Nf * p->maxbatch));
      CFG_CUDA(cudaMemsetAsync(p->fw, 0, sizeof(cplx_t<T>) * (size_t)Nf * p->maxbatch, p->stream));
    }
    e = make_fft(p, p->maxbatch, &p->fft);
    if (e) return e;
    p->have_fft = true;
    if (p->rem) {
      e = make_fft(p, p->rem, &p->fft_rem);
      if (e) return e;
      p->have_fft_rem = true;
    }
  }

  FseriesNodes nodes;
  fseries_nodes(p->sp, &nodes);
  CFG_CUDA(launch_fseries<T>(nodes, dim, p->nf, p->N, p->fac[0], p->fac[1], p->fac[2], p->stream));

  if (p->opts.gpu_kerevalmeth == 1) {
    const int deg = horner_degree<T>(p->sp.ns);
    std::vector<double> cd = horner_fit(p->sp, deg);
    p->horner.assign(cd.begin(), cd.end());
    CFG_CUDA(cudaMalloc(&p->horner_d, sizeof(T) * p->horner.size()));
    CFG_CUDA(cudaMemcpyAsync(p->horner_d, p->horner.data(), sizeof(T) * p->horner.size(),
                             cudaMemcpyHostToDevice, p->stream));
  }
  CFG_CUDA(cudaStreamSynchronize(p->stream));
  p->planned = true;
  return 0;
}

template <typename T>
static int ensure_points(Plan<T>* p, int M) {
  if ((size_t)M <= p->capM && p->idx) return 0;
  free_points(p);
  size_t n = (size_t)std::max(M, 1);
  CFG_CUDA(cudaMalloc(&p->idx, sizeof(int) * n));
  CFG_CUDA(cudaMalloc(&p->rank, sizeof(int) * n));
  for (int k = 0; k < p->dim; ++k) {
    CFG_CUDA(cudaMalloc(&p->i0[k], sizeof(int) * n));
    CFG_CUDA(cudaMalloc(&p->d[k], sizeof(T) * n));
  }
  p->capM = n;
  return 0;
}

template <typename T>
static int select_layout(Plan<T>* p);

// Bank-class order inside bins for method 2 (BankOrder in kernels.h): the
// per (bin, class) counters, zeroed on the plan stream.  Plain bin order for
// method 1, when the counters would exceed 2^24 ints, or with
// CUFINUFFT_BANK_ORDER=0.
// Cell order (cell = true): counters per (bin, cell) and their scan, for
// the cell-run spread; the caller checks cell_order_fits first.
template <typename T>
static bool cell_order_fits(const Plan<T>* p, const int bs[3], long long nbins) {
  long long cells = 1;
  for (int k = 0; k < p->dim; ++k) cells *= bs[k];
  long long taps = 1;
  for (int k = 0; k < p->dim; ++k) taps *= p->sp.ns;
  return p->type == 1 && taps <= 512 && nbins * cells <= (1LL << 24);
}

// Shared memory of the cell-run spread (run_bytes in spreadinterp.cuh).
template <typename T>
static size_t run_smem_bytes(const Plan<T>* p, const int bs[3]) {
  return tile_cells(p->dim, p->sp.ns, bs) * 2 * sizeof(T) +
         (size_t)(256 / 32) * 32 * (size_t)(p->dim * p->sp.ns) * sizeof(T) +
         (size_t)(256 / 32) * 32 * sizeof(cplx_t<T>);
}

template <typename T>
static int bank_order(Plan<T>* p, int method, const int bs[3], int nbins, BankOrder* o,
                      bool cell = false) {
  std::memset(o, 0, sizeof(*o));
  if (method != 2) return 0;
  if (cell) {
    int cells = 1;
    for (int k = 0; k < p->dim; ++k) cells *= bs[k];
    const size_t n = (size_t)nbins * cells;
    if (n > p->cap_cls) {
      cudaFree(p->cls_count);
      p->cls_count = nullptr;
      p->cap_cls = 0;
      CFG_CUDA(cudaMalloc(&p->cls_count, sizeof(int) * n));
      p->cap_cls = n;
    }
    if (n > p->cap_cls_start) {
      cudaFree(p->cls_start);
      cudaFree(p->cls_tmp);
      p->cls_start = p->cls_tmp = nullptr;
      p->cap_cls_start = 0;
      CFG_CUDA(cudaMalloc(&p->cls_start, sizeof(int) * (n + 1)));
      CFG_CUDA(cudaMalloc(&p->cls_tmp, sizeof(int) * (size_t)scan_tmp_ints((int)n)));
      p->cap_cls_start = n;
    }
    if ((size_t)nbins > p->cap_sparse) {
      cudaFree(p->sparse_count);
      p->sparse_count = nullptr;
      p->cap_sparse = 0;
      CFG_CUDA(cudaMalloc(&p->sparse_count, sizeof(int) * (size_t)nbins));
      p->cap_sparse = nbins;
    }
    CFG_CUDA(cudaMemsetAsync(p->cls_count, 0, sizeof(int) * n, p->stream));
    CFG_CUDA(cudaMemsetAsync(p->sparse_count, 0, sizeof(int) * (size_t)nbins, p->stream));
    o->cls_count = p->cls_count;
    o->ncls = cells;
    o->cell_order = 1;
    o->cls_start = p->cls_start;
    o->sparse_count = p->sparse_count;
    o->dense_min = dense_run(p->dim);
    return 0;
  }
  // only the one-thread-per-point tile kernels gain: interpolation by default,
  // spreading only when forced to that variant (the warp-cooperative spread,
  // measured on clustered 3D points, is slower with this order)
  const bool per_point = p->type == 2 ? p->variant != 2 : p->variant == 1;
  if (!per_point) return 0;
  if (const char* v = std::getenv("CUFINUFFT_BANK_ORDER"))
    if (std::strcmp(v, "0") == 0) return 0;  // plain bin order (for comparisons)
  const int ncls = 128 / (int)sizeof(cplx_t<T>);
  const size_t n = (size_t)nbins * ncls;
  if (n > ((size_t)1 << 24)) return 0;
  if (n > p->cap_cls) {
    cudaFree(p->cls_count);
    p->cls_count = nullptr;
    p->cap_cls = 0;
    CFG_CUDA(cudaMalloc(&p->cls_count, sizeof(int) * n));
    p->cap_cls = n;
  }
  CFG_CUDA(cudaMemsetAsync(p->cls_count, 0, sizeof(int) * n, p->stream));
  o->cls_count = p->cls_count;
  o->ncls = ncls;
  // the tile row length the interpolation kernel will index with: FP32 tiles
  // moved by bulk copies widen odd rows by one cell (bulk_tile_x), so the
  // classes must be taken modulo that pitch, or consecutive points of a bin
  // stop falling in distinct banks
  int tx = bs[0] + p->sp.ns - 1;
  if (is_single<T>() && p->type == 2 && (bs[0] & 1) == 0 && (tx & 1)) {
    const char* v = std::getenv("CUFINUFFT_TMA");
    if (!(v && v[0] == '0') && tma_encoder() != nullptr) tx += 1;
  }
  o->tx = tx;
  o->ty = p->dim > 1 ? bs[1] + p->sp.ns - 1 : 1;
  return 0;
}

template <typename T>
static int build_subproblems(Plan<T>* p);

static int setpts_chain(Plan<double>* p, int M, const double* x, const double* y, const double* z);
static int execute_chain(Plan<double>* p, double2* c, double2* fk);
template <typename T>
static int execute_t3(Plan<T>* p, cplx_t<T>* c, cplx_t<T>* fk);

template <typename T>
static int setpts_impl(Plan<T>* p, int M, const T* x, const T* y, const T* z) {
  if constexpr (std::is_same<T, double>::value) {
    if (p->lo) return setpts_chain(p, M, x, y, z);
  }
  if (!p->planned) return CUFINUFFT_ERR_GENERIC;
  if (M < 0) return CUFINUFFT_ERR_ARG;
  const T* xs[3] = {x, y, z};
  for (int k = 0; k < p->dim; ++k)
    if (M > 0 && xs[k] == nullptr) return CUFINUFFT_ERR_ARG;
  p->pts_set = false;
  ++p->version;  // point arrays may be reallocated below
  int e = ensure_points(p, M);
  if (e) return e;
  p->M = M;
  p->nsub = 0;
  PlaceArgs<T> a;
  std::memset(&a, 0, sizeof(a));
  for (int k = 0; k < 3; ++k) {
    a.x[k] = k < p->dim ? xs[k] : nullptr;
    a.ax[k] = axis_map<T>(p->nf[k], p->sp.ns);
    a.bs[k] = p->bs[k];
    a.nb[k] = p->nb[k];
    a.i0[k] = p->i0[k];
    a.d[k] = p->d[k];
  }
  a.dim = p->dim;
  a.M = M;
  a.idx = p->idx;
  a.count = p->count;
  a.rank = p->rank;
  a.start = p->start;
  if (p->method == 1 && p->sort == 0) {
    CFG_CUDA(launch_place_unsorted<T>(a, p->stream));
  } else {
    CFG_CUDA(cudaMemsetAsync(p->count, 0, sizeof(int) * (size_t)p->nbins, p->stream));
    e = bank_order(p, p->method, p->bs, p->nbins, &a.bank, p->cell_order);
    if (e) return e;
    CFG_CUDA(launch_bin_count<T>(a, p->stream));
    CFG_CUDA(launch_scan(p->count, p->start, p->nbins, 0, 1, p->scan_tmp, p->stream));
    if (a.bank.cell_order)
      CFG_CUDA(launch_scan(p->cls_count, p->cls_start, p->nbins * a.bank.ncls, 2, dense_run(p->dim), p->cls_tmp,
                           p->stream));
    CFG_CUDA(launch_permute<T>(a, p->stream));
    if (p->method == 2) {
      e = build_subproblems(p);
      if (e) return e;
    }
  }
  CFG_CUDA(cudaGetLastError());
  p->pts_set = true;
  return select_layout(p);
}

static int max_smem_optin(int device) {
  int v = 0;
  if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, device) != cudaSuccess) return 48 * 1024;
  return v;
}

template <typename T>
static cudaEvent_t take_event(Plan<T>* p) {
  cudaEvent_t e = nullptr;
  if (!p->ev_pool.empty()) {
    e = p->ev_pool.back();
    p->ev_pool.pop_back();
  } else if (cudaEventCreate(&e) != cudaSuccess) {
    return nullptr;
  }
  p->ev_live.push_back(e);
  return e;
}

template <typename T>
static void mark(Plan<T>* p, cudaEvent_t e) {
  if (e) cudaEventRecord(e, p->stream);
}

// Waits for the recorded batches and folds their stage times into stage_ms.
template <typename T>
static int collect_times(Plan<T>* p) {
  const size_t n = p->ev_live.size() / 4 * 4;
  for (size_t i = 0; i < n; i += 4) {
    cudaEvent_t* e = &p->ev_live[i];
    CFG_CUDA(cudaEventSynchronize(e[3]));
    float a = 0, b = 0, c = 0;
    CFG_CUDA(cudaEventElapsedTime(&a, e[0], e[1]));
    CFG_CUDA(cudaEventElapsedTime(&b, e[1], e[2]));
    CFG_CUDA(cudaEventElapsedTime(&c, e[2], e[3]));
    // event order: type 1 = [memset+spread | fft | deconv], type 2 =
    // [amplify | fft | interp]
    if (p->type == 1) {
      p->stage_ms[0] += a;
      p->stage_ms[2] += c;
    } else {
      p->stage_ms[2] += a;
      p->stage_ms[0] += c;
    }
    p->stage_ms[1] += b;
    p->stage_batches += 1;
  }
  for (size_t i = 0; i < n; ++i) p->ev_pool.push_back(p->ev_live[i]);
  p->ev_live.erase(p->ev_live.begin(), p->ev_live.begin() + n);
  return 0;
}

template <typename T>
static int execute_direct(Plan<T>* p, cplx_t<T>* c, cplx_t<T>* fk) {
  if (!p->planned) return CUFINUFFT_ERR_GENERIC;
  if (p->type != 1 && p->type != 2) return CUFINUFFT_ERR_GENERIC;
  if (p->method == 0) return CUFINUFFT_ERR_METHOD;
  if (!p->pts_set) return CUFINUFFT_ERR_GENERIC;
  if (p->M > 0 && c == nullptr) return CUFINUFFT_ERR_ARG;
  if (fk == nullptr) return CUFINUFFT_ERR_ARG;
  if (p->method == 2) {
    size_t bytes = tile_cells(p->dim, p->sp.ns, p->bs) * sizeof(cplx_t<T>);
    if (bytes > (size_t)max_smem_optin(p->device)) return CUFINUFFT_ERR_SHMEM;
  }
  const long long Nf = grid_cells(p);
  const long long Nm = (long long)p->N[0] * p->N[1] * p->N[2];
  SpreadArgs<T> a = spread_args(p);
  for (int b0 = 0; b0 < p->ntransf; b0 += p->maxbatch) {
    const int B = std::min(p->maxbatch, p->ntransf - b0);
    cufftHandle h = (B == p->maxbatch) ? p->fft : p->fft_rem;
    a.ntr = B;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    if (p->timing)
      for (int k = 0; k < 4; ++k) ev[k] = take_event(p);
    mark(p, ev[0]);
    if (p->spread_only) {
      // the caller's fk is the fine grid (nf = nmodes): spread into it or
      // interpolate from it, no FFT and no deconvolution
      mark(p, ev[1]);
      mark(p, ev[2]);
      if (p->type == 1) {
        a.c_in = c + (size_t)b0 * p->M;
        a.fw = fk + (size_t)b0 * Nf;
        CFG_CUDA(cudaMemsetAsync(a.fw, 0, sizeof(cplx_t<T>) * (size_t)Nf * B, p->stream));
        CFG_CUDA(run_spread(p, a));
      } else {
        a.fw_in = fk + (size_t)b0 * Nf;
        a.c_out = c + (size_t)b0 * p->M;
        CFG_CUDA(run_interp(p, a));
      }
      mark(p, ev[3]);
      continue;
    }
    if (p->type == 1) {
      a.c_in = c + (size_t)b0 * p->M;
      a.fw = p->fw;
      CFG_CUDA(cudaMemsetAsync(p->fw, 0, sizeof(cplx_t<T>) * (size_t)Nf * B, p->stream));
      CFG_CUDA(run_spread(p, a));
      mark(p, ev[1]);
      if (p->half_fft) {
        const std::vector<HalfPass<T>> passes = half_passes(p, fk + (size_t)b0 * Nm, B);
        for (size_t i = 0; i < passes.size(); ++i) {
          if (i + 1 == passes.size()) mark(p, ev[2]);  // last pass: deconvolution fused
          CFG_CUDA(launch_half_pass<T>(passes[i], p->stream));
        }
      } else if (p->line_fft) {
        const std::vector<LineArgs<T>> passes = line_passes(p, fk + (size_t)b0 * Nm, B);
        for (size_t i = 0; i < passes.size(); ++i) {
          if (i + 1 == passes.size()) mark(p, ev[2]);  // last pass: deconvolution fused
          CFG_CUDA(launch_line_fft<T>(passes[i], p->stream));
        }
      } else {
        if (p->df_fft) CFG_CUDA(df_fft_exec(p, p->fw, p->fw, B));
        else CFG_CUFFT(fft_exec(h, p->fw, p->iflag));
        mark(p, ev[2]);
        CFG_CUDA(launch_deconvolve<T>(p->dim, p->nf, p->N, p->fw, fk + (size_t)b0 * Nm, p->fac[0],
                                      p->fac[1], p->fac[2], B, p->stream));
      }
    } else {
      if (p->half_fft) {
        const std::vector<HalfPass<T>> passes = half_passes(p, fk + (size_t)b0 * Nm, B);
        for (size_t i = 0; i < passes.size(); ++i) {
          CFG_CUDA(launch_half_pass<T>(passes[i], p->stream));
          if (i == 0) mark(p, ev[1]);  // first pass: amplification fused
        }
        mark(p, ev[2]);
      } else if (p->line_fft) {
        const std::vector<LineArgs<T>> passes = line_passes(p, fk + (size_t)b0 * Nm, B);
        for (size_t i = 0; i < passes.size(); ++i) {
          CFG_CUDA(launch_line_fft<T>(passes[i], p->stream));
          if (i == 0) mark(p, ev[1]);  // first pass: amplification fused
        }
        mark(p, ev[2]);
      } else {
        CFG_CUDA(launch_amplify_modes<T>(p->dim, p->nf, p->N, p->fw, fk + (size_t)b0 * Nm, p->fac[0],
                                         p->fac[1], p->fac[2], B, p->stream));
        mark(p, ev[1]);
        if (p->df_fft) CFG_CUDA(df_fft_exec(p, p->fw, p->fw2, B));
        else CFG_CUFFT(fft_exec(h, p->fw, p->fw2, p->iflag));
        mark(p, ev[2]);
      }
      a.fw_in = p->fw2 ? p->fw2 : p->fw;
      a.c_out = c + (size_t)b0 * p->M;
      CFG_CUDA(run_interp(p, a));
    }
    mark(p, ev[3]);
  }
  return 0;
}

void* tma_encoder() {
  static void* const fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();  // no encoder: interpolation tiles stay on the per-cell path
      f = nullptr;
    }
    return f;
  }();
  return fn;
}

// CUFINUFFT_GRAPH=0: every execute launches its kernels directly.
static bool graphs_enabled() {
  const char* v = std::getenv("CUFINUFFT_GRAPH");
  return !(v && v[0] == '0');
}

// execute: with stage timing off, the launch sequence is captured once as a
// CUDA graph (for these caller arrays and this plan state) and replayed, which
// removes most of the gaps between its kernels.  A plan stream that is already
// being captured (a batch recording this plan), or a capture that fails, runs
// the kernels directly.
// A tile wait of an earlier execute ran out (SpreadArgs::status): its result
// was still computed from the same values, but the stall is reported once,
// as a CUDA error of the next execute or stage-time read (the flag is
// cleared).
template <typename T>
static int take_status(Plan<T>* p) {
  if (!p->h_status) return 0;
  volatile int* s = p->h_status;
  if (s[0] == 0 && s[1] == 0) return 0;
  if (s[1]) fprintf(stderr, "cufinufft: an interpolation tile copy did not complete\n");
  else fprintf(stderr, "cufinufft: an interpolation tile wait ran out (tile loaded cell by cell)\n");
  s[0] = s[1] = 0;
  return CUFINUFFT_ERR_CUDA;
}

template <typename T>
static int execute_impl(Plan<T>* p, cplx_t<T>* c, cplx_t<T>* fk) {
  if constexpr (std::is_same<T, double>::value) {
    if (p->lo) return execute_chain(p, c, fk);
  }
  if (p->type == 3) return execute_t3(p, c, fk);
  if (const int e = take_status(p)) return e;
  if (p->timing || !p->planned || !graphs_enabled()) return execute_direct(p, c, fk);
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(p->stream, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
    cudaGetLastError();
    return execute_direct(p, c, fk);
  }
  if (p->gexec && p->g_c == c && p->g_fk == fk && p->g_version == p->version) {
    CFG_CUDA(cudaGraphLaunch(p->gexec, p->stream));
    return 0;
  }
  drop_graph(p);
  if (cudaStreamBeginCapture(p->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
    const int e = execute_direct(p, c, fk);
    cudaGraph_t g = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(p->stream, &g);
    if (e == 0 && ce == cudaSuccess && g != nullptr &&
        cudaGraphInstantiate(&p->gexec, g, 0) == cudaSuccess) {
      p->graph = g;
      p->g_c = c;
      p->g_fk = fk;
      p->g_version = p->version;
      CFG_CUDA(cudaGraphLaunch(p->gexec, p->stream));
      return 0;
    }
    if (g) cudaGraphDestroy(g);
    p->gexec = nullptr;
    cudaGetLastError();  // a failed capture leaves its error behind
    if (e) return e;     // the plan or the arguments are at fault, not the capture
  } else {
    cudaGetLastError();
  }
  return execute_direct(p, c, fk);
}

// ---------------------------------------------------------------------------
// The FP32 chain of FP64 plans.  An FP64 plan whose tolerance is at least
// kChainTol makes an FP32 plan `lo` with the FP64 plan's kernel (width from
// the FP64 rule, beta and c rounded to FP32, Fourier-series factors
// evaluated in FP64 for that kernel) and runs spreading/interpolation, the
// FFT and the deconvolution there.  The FP64 side keeps what needs FP64:
// folding and rescaling the points (first tap and tap offset computed in
// FP64, the offset in [0,1) then rounded to FP32) and the conversion of c
// and fk.  On GB300, whose FP64 units are a small fraction of its FP32
// throughput, this moves the FP64 plan to the FP32 plan's speed.  FP32
// rounding of the chain leaves ~2-4e-7 relative l2 on large grids (an FP32
// FFT of 256^2..2048^2 alone 1.5-1.8e-7), so the chain is taken from tol
// 1e-6 up, where that stays below tol; CUFINUFFT_FP64_CHAIN=1 keeps every
// FP64 plan in FP64 throughout, as the reference's FP64 build does.
constexpr double kChainTol = 1e-6;

static bool chain_wanted(int type, double tol, const cufinufft_opts* opts) {
  if (type != 1 && type != 2) return false;
  if (opts && opts->gpu_spreadinterponly) return false;
  if (!(tol >= kChainTol)) return false;
  const char* v = std::getenv("CUFINUFFT_FP64_CHAIN");
  return !(v && v[0] == '1');
}

// The FP64 plan's view of its chain (what info, the batch and the layout
// calls read).
static void sync_from_lo(Plan<double>* p) {
  const Plan<float>* q = p->lo;
  for (int k = 0; k < 3; ++k) {
    p->N[k] = q->N[k];
    p->nf[k] = q->nf[k];
    p->bs[k] = q->bs[k];
    p->nb[k] = q->nb[k];
  }
  p->ntransf = q->ntransf;
  p->maxbatch = q->maxbatch;
  p->iflag = q->iflag;
  p->rem = q->rem;
  p->opts = q->opts;
  p->method = q->method;
  p->variant = q->variant;
  p->auto_method = q->auto_method;
  p->sort = q->sort;
  p->nbins = q->nbins;
  p->M = q->M;
  p->nsub = q->nsub;
  p->cell_order = q->cell_order;
  p->line_fft = q->line_fft;
  p->half_fft = q->half_fft;
  p->spread_only = q->spread_only;
  p->planned = q->planned;
  p->pts_set = q->pts_set;
  p->stream = q->stream;
  p->timing = q->timing;
}

static int makeplan_chain(Plan<double>* p, int type, int dim, const int* nmodes, int iflag, int ntransf,
                          double tol, int maxbatchsize, const cufinufft_opts* opts) {
  p->type = type;
  p->dim = dim;
  p->width_rule = width_rule_now();
  if (opts) p->opts = *opts;
  else default_opts(type, dim, &p->opts);
  int ier = setup_spreader(tol, p->opts.upsampfac, p->opts.gpu_kerevalmeth, false, &p->sp, p->width_rule,
                           dim);
  if (ier > 1) return ier;
  SpreaderParams sp = p->sp;
  sp.beta = (double)(float)sp.beta;  // the FP32 kernel's shape, exactly
  sp.c = (double)(float)sp.c;
  p->lo = new (std::nothrow) Plan<float>();
  if (!p->lo) return CUFINUFFT_ERR_ALLOC;
  p->lo->device = p->device;
  ier = makeplan_impl<float>(p->lo, type, dim, nmodes, iflag, ntransf, tol, maxbatchsize, opts, &sp);
  if (ier) return ier;
  sync_from_lo(p);
  const long long Nm = (long long)p->N[0] * p->N[1] * p->N[2];
  CFG_CUDA(cudaMalloc(&p->fk32, sizeof(cplx_t<float>) * (size_t)(Nm * p->ntransf)));
  return 0;
}

// Sort of points already placed (first taps and FP32 offsets in caller
// order): the counting sort of setpts, fed from stored arrays instead of
// coordinates (the rebin kernels).
static int setpts_placed(Plan<float>* q, int M, const int* s_idx, int* const s_i0[3], float* const s_d[3]) {
  if (!q->planned) return CUFINUFFT_ERR_GENERIC;
  q->pts_set = false;
  ++q->version;
  int e = ensure_points(q, M);
  if (e) return e;
  q->M = M;
  q->nsub = 0;
  if (M > 0 && q->method == 1 && q->sort == 0) {
    CFG_CUDA(cudaMemcpyAsync(q->idx, s_idx, sizeof(int) * (size_t)M, cudaMemcpyDeviceToDevice, q->stream));
    for (int k = 0; k < q->dim; ++k) {
      CFG_CUDA(cudaMemcpyAsync(q->i0[k], s_i0[k], sizeof(int) * (size_t)M, cudaMemcpyDeviceToDevice,
                               q->stream));
      CFG_CUDA(cudaMemcpyAsync(q->d[k], s_d[k], sizeof(float) * (size_t)M, cudaMemcpyDeviceToDevice,
                               q->stream));
    }
  } else if (!(q->method == 1 && q->sort == 0)) {
    RebinArgs<float> a;
    std::memset(&a, 0, sizeof(a));
    a.dim = q->dim;
    a.M = M;
    for (int k = 0; k < 3; ++k) {
      a.bs[k] = q->bs[k];
      a.nb[k] = q->nb[k];
      a.src_i0[k] = k < q->dim ? s_i0[k] : nullptr;
      a.src_d[k] = k < q->dim ? s_d[k] : nullptr;
      a.i0[k] = q->i0[k];
      a.d[k] = q->d[k];
    }
    a.src_idx = s_idx;
    a.idx = q->idx;
    a.count = q->count;
    a.rank = q->rank;
    a.start = q->start;
    CFG_CUDA(cudaMemsetAsync(q->count, 0, sizeof(int) * (size_t)q->nbins, q->stream));
    e = bank_order(q, q->method, q->bs, q->nbins, &a.bank, q->cell_order);
    if (e) return e;
    CFG_CUDA(launch_rebin_count<float>(a, q->stream));
    CFG_CUDA(launch_scan(q->count, q->start, q->nbins, 0, 1, q->scan_tmp, q->stream));
    if (a.bank.cell_order)
      CFG_CUDA(launch_scan(q->cls_count, q->cls_start, q->nbins * a.bank.ncls, 2, dense_run(q->dim),
                           q->cls_tmp, q->stream));
    CFG_CUDA(launch_rebin_permute<float>(a, q->stream));
    if (q->method == 2) {
      e = build_subproblems(q);
      if (e) return e;
    }
  }
  CFG_CUDA(cudaGetLastError());
  q->pts_set = true;
  return select_layout(q);
}

static int setpts_chain(Plan<double>* p, int M, const double* x, const double* y, const double* z) {
  Plan<float>* q = p->lo;
  if (!q->planned) return CUFINUFFT_ERR_GENERIC;
  if (M < 0) return CUFINUFFT_ERR_ARG;
  const double* xs[3] = {x, y, z};
  for (int k = 0; k < p->dim; ++k)
    if (M > 0 && xs[k] == nullptr) return CUFINUFFT_ERR_ARG;
  ++p->version;
  p->pts_set = q->pts_set = false;
  if ((size_t)M > p->n_cap || p->n_idx == nullptr) {
    cudaFree(p->n_idx);
    p->n_idx = nullptr;
    for (int k = 0; k < 3; ++k) {
      cudaFree(p->n_i0[k]);
      cudaFree(p->n_d[k]);
      p->n_i0[k] = nullptr;
      p->n_d[k] = nullptr;
    }
    cudaFree(p->c32);
    p->c32 = nullptr;
    p->n_cap = p->c32_cap = 0;
    const size_t n = (size_t)std::max(M, 1);
    CFG_CUDA(cudaMalloc(&p->n_idx, sizeof(int) * n));
    for (int k = 0; k < p->dim; ++k) {
      CFG_CUDA(cudaMalloc(&p->n_i0[k], sizeof(int) * n));
      CFG_CUDA(cudaMalloc(&p->n_d[k], sizeof(float) * n));
    }
    CFG_CUDA(cudaMalloc(&p->c32, sizeof(cplx_t<float>) * n * (size_t)p->ntransf));
    p->n_cap = n;
    p->c32_cap = n * (size_t)p->ntransf;
  }
  NarrowPlaceArgs na;
  std::memset(&na, 0, sizeof(na));
  for (int k = 0; k < 3; ++k) {
    na.x[k] = k < p->dim ? xs[k] : nullptr;
    na.ax[k] = axis_map<double>(q->nf[k], q->sp.ns);
    na.i0[k] = p->n_i0[k];
    na.d[k] = p->n_d[k];
  }
  na.dim = p->dim;
  na.M = M;
  na.idx = p->n_idx;
  CFG_CUDA(launch_place_narrow(na, q->stream));
  const int e = setpts_placed(q, M, p->n_idx, p->n_i0, p->n_d);
  sync_from_lo(p);
  return e;
}

static int execute_chain(Plan<double>* p, double2* c, double2* fk) {
  Plan<float>* q = p->lo;
  if (!q->planned || !q->pts_set) return CUFINUFFT_ERR_GENERIC;
  if (q->M > 0 && c == nullptr) return CUFINUFFT_ERR_ARG;
  if (fk == nullptr) return CUFINUFFT_ERR_ARG;
  const long long nc = (long long)q->ntransf * q->M;
  const long long nk = (long long)q->ntransf * q->N[0] * q->N[1] * q->N[2];
  int e = 0;
  if (q->type == 1) {
    CFG_CUDA(launch_narrow_complex(c, p->c32, nc, q->stream));
    e = execute_impl(q, p->c32, p->fk32);
    if (e) return e;
    CFG_CUDA(launch_widen_complex(p->fk32, fk, nk, q->stream));
  } else {
    CFG_CUDA(launch_narrow_complex(fk, p->fk32, nk, q->stream));
    e = execute_impl(q, p->c32, p->fk32);
    if (e) return e;
    CFG_CUDA(launch_widen_complex(p->c32, c, nc, q->stream));
  }
  return 0;
}

// ---------------------------------------------------------------------------
// Type 3 (nonuniform points to nonuniform frequencies; type3.cu has the
// method).  makeplan keeps the parameters; setpts measures the extents of
// the points and frequencies, sizes the rescaled grid (nf >= 2 sigma S X /
// pi + ns + 1 per axis, with x' = (x - C)/gam in [-pi, pi) and gam = nf /
// (2 sigma S)), and makes a spread-only plan onto that grid and an inner
// type-2 plan over it (both with this plan's kernel); execute runs
// prephase -> spread -> type 2 -> phase / phihat.
template <typename T>
static int makeplan_t3(Plan<T>* p, int dim, int iflag, int ntransf, double tol, int maxbatchsize,
                       const cufinufft_opts* opts) {
  p->type = 3;
  p->dim = dim;
  p->width_rule = width_rule_now();
  if (opts) p->opts = *opts;
  else default_opts(3, dim, &p->opts);
  if (p->opts.gpu_spreadinterponly) return CUFINUFFT_ERR_ARG;
  int ier = setup_spreader(tol, p->opts.upsampfac, p->opts.gpu_kerevalmeth, is_single<T>(), &p->sp,
                           p->width_rule, dim);
  if (ier > 1) return ier;
  p->iflag = iflag >= 0 ? 1 : -1;
  p->ntransf = ntransf;
  if (maxbatchsize == 0) maxbatchsize = std::min(ntransf, 8);
  p->maxbatch = std::min(maxbatchsize, ntransf);
  p->t3_tol = tol;
  p->method = 2;
  CFG_CUDA(cudaStreamCreate(&p->own));
  p->stream = p->own;
  CFG_CUDA(cudaMalloc(&p->t3_part, sizeof(double) * 2 * (size_t)minmax_partials()));
  p->planned = true;
  return 0;
}

// Minimum and maximum of a[0..n) (device), on the plan stream.
template <typename T>
static int extent(Plan<T>* p, const T* a, long long n, double* lo, double* hi) {
  *lo = *hi = 0.0;
  if (n <= 0) return 0;
  int nb = 0;
  CFG_CUDA(launch_minmax<T>(a, n, p->t3_part, &nb, p->stream));
  std::vector<double> h(2 * (size_t)nb);
  CFG_CUDA(cudaMemcpyAsync(h.data(), p->t3_part, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, p->stream));
  CFG_CUDA(cudaStreamSynchronize(p->stream));
  double a0 = h[0], a1 = h[1];
  for (int b = 1; b < nb; ++b) {
    a0 = std::min(a0, h[2 * b]);
    a1 = std::max(a1, h[2 * b + 1]);
  }
  if (!std::isfinite(a0) || !std::isfinite(a1)) return CUFINUFFT_ERR_ARG;
  *lo = a0;
  *hi = a1;
  return 0;
}

template <typename T>
static int grow(T** buf, size_t* cap, size_t n) {
  if (n <= *cap && *buf) return 0;
  cudaFree(*buf);
  *buf = nullptr;
  *cap = 0;
  CFG_CUDA(cudaMalloc(buf, sizeof(T) * std::max<size_t>(n, 1)));
  *cap = n;
  return 0;
}

template <typename T>
static int setpts_t3(Plan<T>* p, int M, const T* x, const T* y, const T* z, int Nt, const T* s, const T* t,
                     const T* u) {
  if (!p->planned) return CUFINUFFT_ERR_GENERIC;
  if (M < 0 || Nt < 0) return CUFINUFFT_ERR_ARG;
  const T* xs[3] = {x, y, z};
  const T* ss[3] = {s, t, u};
  for (int k = 0; k < p->dim; ++k)
    if ((M > 0 && !xs[k]) || (Nt > 0 && !ss[k])) return CUFINUFFT_ERR_ARG;
  p->pts_set = false;
  ++p->version;
  const double sigma = p->opts.upsampfac;
  const int nss = p->sp.ns + 1;
  int nf[3] = {1, 1, 1};
  long long cells = 1;
  for (int k = 0; k < p->dim; ++k) {
    double xl, xh, sl, sh;
    int e = extent(p, xs[k], M, &xl, &xh);
    if (e) return e;
    e = extent(p, ss[k], Nt, &sl, &sh);
    if (e) return e;
    double X = 0.5 * (xh - xl), S = 0.5 * (sh - sl);
    p->t3_C[k] = 0.5 * (xh + xl);
    p->t3_D[k] = 0.5 * (sh + sl);
    if (X == 0.0) X = S == 0.0 ? 1.0 : 1.0 / S;
    if (S == 0.0) S = 1.0 / X;
    const double nfd = 2.0 * sigma * S * X / M_PI + nss;
    if (!(nfd < (double)(1 << 22))) return CUFINUFFT_ERR_ARG;  // the grid would not fit
    int n = std::max((int)nfd, 2 * nss);
    n = next235beven(n, 1);
    nf[k] = n;
    cells *= n;
    p->t3_h[k] = 2.0 * M_PI / n;
    p->t3_gam[k] = n / (2.0 * sigma * S);
  }
  if (cells > (1LL << 28)) return CUFINUFFT_ERR_ARG;
  p->M = M;
  p->t3_N = Nt;
  // spread-only plan onto the rescaled grid and the inner type-2 plan, made
  // again when the grid changes
  auto same = [&](const Plan<T>* q) {
    return q && q->nf[0] == nf[0] && q->nf[1] == nf[1] && q->nf[2] == nf[2];
  };
  if (!same(p->t3_spread) || !p->t3_inner || p->t3_inner->N[0] != nf[0] || p->t3_inner->N[1] != nf[1] ||
      p->t3_inner->N[2] != nf[2]) {
    Plan<T>** const t3[2] = {&p->t3_spread, &p->t3_inner};
  for (Plan<T>** q : t3) {
      if (*q) {
        release(*q);
        delete *q;
        *q = nullptr;
      }
    }
    p->t3_spread = new (std::nothrow) Plan<T>();
    p->t3_inner = new (std::nothrow) Plan<T>();
    if (!p->t3_spread || !p->t3_inner) return CUFINUFFT_ERR_ALLOC;
    p->t3_spread->device = p->t3_inner->device = p->device;
    cufinufft_opts o1 = p->opts;
    o1.gpu_spreadinterponly = 1;
    int e = makeplan_impl<T>(p->t3_spread, 1, p->dim, nf, p->iflag, p->ntransf, p->t3_tol, p->maxbatch, &o1,
                             &p->sp);
    if (e) return e;
    cufinufft_opts o2;
    default_opts(2, p->dim, &o2);
    o2.upsampfac = p->opts.upsampfac;
    o2.gpu_kerevalmeth = p->opts.gpu_kerevalmeth;
    o2.gpu_device_id = p->opts.gpu_device_id;
    o2.gpu_method = 0;  // the library's choice for the inner interpolation
    e = makeplan_impl<T>(p->t3_inner, 2, p->dim, nf, p->iflag, p->ntransf, p->t3_tol, p->maxbatch, &o2,
                         &p->sp);
    if (e) return e;
    plan_use_stream(p->t3_spread, p->stream);
    plan_use_stream(p->t3_inner, p->stream);
  }
  for (int k = 0; k < 3; ++k) p->nf[k] = nf[k];
  if ((size_t)M > p->t3_capM || !p->t3_pre) {
    for (int k = 0; k < 3; ++k) {
      cudaFree(p->t3_xp[k]);
      p->t3_xp[k] = nullptr;
    }
    cudaFree(p->t3_pre);
    cudaFree(p->t3_c);
    p->t3_pre = p->t3_c = nullptr;
    p->t3_capM = 0;
    const size_t n = (size_t)std::max(M, 1);
    for (int k = 0; k < p->dim; ++k) CFG_CUDA(cudaMalloc(&p->t3_xp[k], sizeof(T) * n));
    CFG_CUDA(cudaMalloc(&p->t3_pre, sizeof(cplx_t<T>) * n));
    CFG_CUDA(cudaMalloc(&p->t3_c, sizeof(cplx_t<T>) * n * (size_t)p->ntransf));
    p->t3_capM = n;
  }
  if ((size_t)Nt > p->t3_capN || !p->t3_post) {
    for (int k = 0; k < 3; ++k) {
      cudaFree(p->t3_tau[k]);
      p->t3_tau[k] = nullptr;
    }
    cudaFree(p->t3_post);
    p->t3_post = nullptr;
    p->t3_capN = 0;
    const size_t n = (size_t)std::max(Nt, 1);
    for (int k = 0; k < p->dim; ++k) CFG_CUDA(cudaMalloc(&p->t3_tau[k], sizeof(T) * n));
    CFG_CUDA(cudaMalloc(&p->t3_post, sizeof(cplx_t<T>) * n));
    p->t3_capN = n;
  }
  {
    const int e = grow(&p->t3_grid, &p->t3_capG, (size_t)cells * p->ntransf);
    if (e) return e;
  }
  Type3Phase<T> ph;
  std::memset(&ph, 0, sizeof(ph));
  ph.dim = p->dim;
  ph.sgn = p->iflag;
  for (int k = 0; k < p->dim; ++k) {
    ph.C[k] = p->t3_C[k];
    ph.D[k] = p->t3_D[k];
    ph.hg[k] = p->t3_h[k] * p->t3_gam[k];
    CFG_CUDA(launch_affine<T>(xs[k], M, p->t3_C[k], 1.0 / p->t3_gam[k], p->t3_xp[k], p->stream));
    CFG_CUDA(launch_affine<T>(ss[k], Nt, p->t3_D[k], ph.hg[k], p->t3_tau[k], p->stream));
  }
  for (int k = 0; k < p->dim; ++k) ph.x[k] = xs[k];
  CFG_CUDA(launch_prephase<T>(ph, M, p->t3_pre, p->stream));
  for (int k = 0; k < p->dim; ++k) ph.x[k] = ss[k];
  FseriesNodes nodes;
  fseries_nodes(p->sp, &nodes);
  CFG_CUDA(launch_postfactor<T>(ph, nodes, Nt, p->t3_post, p->stream));
  int e = setpts_impl(p->t3_spread, M, p->t3_xp[0], p->t3_xp[1], p->t3_xp[2]);
  if (e) return e;
  e = setpts_impl(p->t3_inner, Nt, p->t3_tau[0], p->t3_tau[1], p->t3_tau[2]);
  if (e) return e;
  // the caller's arrays may be released once setpts returns
  CFG_CUDA(cudaStreamSynchronize(p->stream));
  p->pts_set = true;
  return 0;
}

template <typename T>
static int execute_t3(Plan<T>* p, cplx_t<T>* c, cplx_t<T>* fk) {
  if (!p->planned || !p->pts_set) return CUFINUFFT_ERR_GENERIC;
  if ((p->M > 0 && !c) || (p->t3_N > 0 && !fk)) return CUFINUFFT_ERR_ARG;
  if (p->t3_N == 0) return 0;
  if (p->M == 0) {
    CFG_CUDA(cudaMemsetAsync(fk, 0, sizeof(cplx_t<T>) * (size_t)p->t3_N * p->ntransf, p->stream));
    return 0;
  }
  CFG_CUDA(launch_cmul_rows<T>(c, p->t3_pre, p->M, p->ntransf, p->t3_c, p->stream));
  int e = execute_impl(p->t3_spread, p->t3_c, p->t3_grid);
  if (e) return e;
  e = execute_impl(p->t3_inner, fk, p->t3_grid);
  if (e) return e;
  CFG_CUDA(launch_cmul_rows<T>(fk, p->t3_post, p->t3_N, p->ntransf, fk, p->stream));
  return 0;
}

// Entry points for the batch (batch.cu): a plan's whole execute, and moving
// a plan's work, cuFFT plans included, to another stream.
template <typename T>
int execute_plan(Plan<T>* p, cplx_t<T>* c, cplx_t<T>* fk) {
  if constexpr (std::is_same<T, double>::value) {
    if (p->lo) return execute_chain(p, c, fk);
  }
  return execute_direct(p, c, fk);
}
template <typename T>
int plan_use_stream(Plan<T>* p, cudaStream_t s) {
  if (p->lo) {
    const int e = plan_use_stream(p->lo, s);
    p->stream = s;
    return e;
  }
  Plan<T>* const t3[2] = {p->t3_spread, p->t3_inner};
  for (Plan<T>* q : t3)
    if (q) {
      const int e = plan_use_stream(q, s);
      if (e) return e;
    }
  p->stream = s;
  if (p->have_fft) CFG_CUFFT(cufftSetStream(p->fft, s));
  if (p->have_fft_rem) CFG_CUFFT(cufftSetStream(p->fft_rem, s));
  return 0;
}
template int execute_plan<float>(Plan<float>*, cplx_t<float>*, cplx_t<float>*);
template int execute_plan<double>(Plan<double>*, cplx_t<double>*, cplx_t<double>*);
template int plan_use_stream<float>(Plan<float>*, cudaStream_t);
template int plan_use_stream<double>(Plan<double>*, cudaStream_t);

template <typename T>
static void fill_info(const Plan<T>* p, cufinufft_plan_info* info) {
  std::memset(info, 0, sizeof(*info));
  info->type = p->type;
  info->dim = p->dim;
  info->ms = p->N[0];
  info->mt = p->N[1];
  info->mu = p->N[2];
  info->nf1 = p->nf[0];
  info->nf2 = p->nf[1];
  info->nf3 = p->nf[2];
  info->ns = p->sp.ns;
  info->M = p->M;
  info->ntransf = p->ntransf;
  info->maxbatchsize = p->maxbatch;
  info->method = p->method;
  info->sort = p->sort;
  info->binsizex = p->bs[0];
  info->binsizey = p->bs[1];
  info->binsizez = p->bs[2];
  info->nbins = p->nbins;
  info->nsubprob = p->nsub;
  info->kerevalmeth = p->opts.gpu_kerevalmeth;
  info->beta = p->sp.beta;
  info->es_c = p->sp.c;
  info->line_fft = p->line_fft ? 1 : 0;
  info->half_fft = p->half_fft ? 1 : 0;
  info->df_fft = p->df_fft ? 1 : 0;
  info->fp64_df = p->fp64_df && p->method == 2 ? 1 : 0;  // the subproblem interpolation only
  info->cell_order = p->cell_order ? 1 : 0;
  info->width_rule = p->width_rule;
}

// ---------------------------------------------------------------------------
// Layout changes and autotuning (extensions).

// Reallocate the bin tables for nbins bins.
template <typename T>
static int alloc_bins(Plan<T>* p, int nbins) {
  cudaFree(p->count);
  cudaFree(p->start);
  cudaFree(p->sub_start);
  cudaFree(p->scan_tmp);
  p->count = p->start = p->sub_start = p->scan_tmp = nullptr;
  CFG_CUDA(cudaMalloc(&p->count, sizeof(int) * (size_t)nbins));
  CFG_CUDA(cudaMalloc(&p->start, sizeof(int) * ((size_t)nbins + 1)));
  CFG_CUDA(cudaMalloc(&p->sub_start, sizeof(int) * ((size_t)nbins + 1)));
  CFG_CUDA(cudaMalloc(&p->scan_tmp, sizeof(int) * (size_t)scan_tmp_ints(nbins)));
  return 0;
}

// Subproblem tables of the current layout (method 2): one readback of the
// total, as in setpts.
template <typename T>
static int build_subproblems(Plan<T>* p) {
  p->nsub = 0;
  if (p->M == 0) return 0;
  const int ms = p->opts.gpu_maxsubprobsize;
  CFG_CUDA(launch_scan(p->count, p->sub_start, p->nbins, 1, ms, p->scan_tmp, p->stream));
  CFG_CUDA(cudaMemcpyAsync(p->h_total, p->sub_start + p->nbins, sizeof(int), cudaMemcpyDeviceToHost,
                           p->stream));
  CFG_CUDA(cudaStreamSynchronize(p->stream));
  const int nsub = *p->h_total;
  if ((size_t)nsub > p->cap_sub) {
    cudaFree(p->sub_to_bin);
    cudaFree(p->sub_hdr);
    p->sub_to_bin = nullptr;
    p->sub_hdr = nullptr;
    p->cap_sub = 0;
    CFG_CUDA(cudaMalloc(&p->sub_to_bin, sizeof(int) * (size_t)nsub));
    CFG_CUDA(cudaMalloc(&p->sub_hdr, sizeof(SubHdr) * (size_t)nsub));
    p->cap_sub = nsub;
  }
  CFG_CUDA(launch_sub_headers(p->sub_start, p->start, p->count, p->nbins, nsub, ms, p->bs, p->nb,
                              p->sub_to_bin, p->sub_hdr, p->stream));
  p->nsub = nsub;
  if (p->cell_order) {
    if ((size_t)nsub > p->cap_sub_dense) {
      cudaFree(p->sub_dense);
      cudaFree(p->sub_ndense);
      p->sub_dense = nullptr;
      p->sub_ndense = nullptr;
      p->cap_sub_dense = 0;
      CFG_CUDA(cudaMalloc(&p->sub_dense, (size_t)nsub));
      CFG_CUDA(cudaMalloc(&p->sub_ndense, sizeof(int) * (size_t)nsub));
      p->cap_sub_dense = nsub;
    }
    SubClassArgs c;
    std::memset(&c, 0, sizeof(c));
    c.sub_to_bin = p->sub_to_bin;
    c.sub_start = p->sub_start;
    c.start = p->start;
    c.cls_count = p->cls_count;
    for (int k = 0; k < 3; ++k) {
      c.i0[k] = p->i0[k];
      c.bs[k] = p->bs[k];
    }
    c.dim = p->dim;
    c.maxsub = ms;
    c.ncls = 1;
    for (int k = 0; k < p->dim; ++k) c.ncls *= p->bs[k];
    c.nsub = nsub;
    c.dense_min = dense_run(p->dim);
    c.dense = p->sub_dense;
    c.cls_start = p->cls_start;
    c.count = p->count;
    c.ndense = p->sub_ndense;
    CFG_CUDA(launch_classify_subproblems(c, p->stream));
  }
  return 0;
}

// Switch a plan with points set to another method / bin size / subproblem
// cap by re-sorting its stored points (the caller's coordinates are not
// needed).  Results are unchanged; only the work schedule moves.
template <typename T>
static int set_layout_impl(Plan<T>* p, int method, const int bsz[3], int maxsub) {
  if (!p->planned) return CUFINUFFT_ERR_GENERIC;
  if (p->type == 3) return CUFINUFFT_ERR_METHOD;  // type 3 lays out its inner plans itself
  ++p->version;  // the sorted arrays and bin tables are about to move
  // method 5: method 2 spreading over cell-ordered points (cell-run kernel)
  const bool cell = method == 5;
  if (cell) {
    if (p->type != 1) return CUFINUFFT_ERR_METHOD;
    method = 2;
  }
  if (method != 1 && method != 2) return CUFINUFFT_ERR_METHOD;
  if (method == 2 && p->type == 2 && p->dim == 1) return CUFINUFFT_ERR_METHOD;
  if (method == 2 && maxsub <= 0) return CUFINUFFT_ERR_ARG;
  int bs[3], nb[3];
  long long nbins = 1;
  for (int k = 0; k < 3; ++k) {
    if (k < p->dim) {
      if (bsz[k] <= 0) return CUFINUFFT_ERR_ARG;
      bs[k] = std::min(bsz[k], p->nf[k]);
      nb[k] = (p->nf[k] + bs[k] - 1) / bs[k];
    } else {
      bs[k] = 1;
      nb[k] = 1;
    }
    nbins *= nb[k];
  }
  if (nbins > (1LL << 24)) return CUFINUFFT_ERR_ARG;
  if (method == 2 && tile_cells(p->dim, p->sp.ns, bs) * sizeof(cplx_t<T>) >
                         (size_t)max_smem_optin(p->device))
    return CUFINUFFT_ERR_SHMEM;
  if (cell && !cell_order_fits(p, bs, nbins)) return CUFINUFFT_ERR_ARG;
  if (cell && run_smem_bytes(p, bs) > (size_t)max_smem_optin(p->device)) return CUFINUFFT_ERR_SHMEM;
  int e = alloc_bins(p, (int)nbins);
  if (e) return e;
  if (p->pts_set && p->M > 0) {
    // fresh arrays for the re-sorted points
    int* idx = nullptr;
    int* i0[3] = {nullptr, nullptr, nullptr};
    T* d[3] = {nullptr, nullptr, nullptr};
    CFG_CUDA(cudaMalloc(&idx, sizeof(int) * p->capM));
    for (int k = 0; k < p->dim; ++k) {
      CFG_CUDA(cudaMalloc(&i0[k], sizeof(int) * p->capM));
      CFG_CUDA(cudaMalloc(&d[k], sizeof(T) * p->capM));
    }
    RebinArgs<T> a;
    std::memset(&a, 0, sizeof(a));
    a.dim = p->dim;
    a.M = p->M;
    for (int k = 0; k < 3; ++k) {
      a.bs[k] = bs[k];
      a.nb[k] = nb[k];
      a.src_i0[k] = p->i0[k];
      a.src_d[k] = p->d[k];
      a.i0[k] = i0[k];
      a.d[k] = d[k];
    }
    a.src_idx = p->idx;
    a.idx = idx;
    a.count = p->count;
    a.rank = p->rank;
    a.start = p->start;
    e = bank_order(p, method, bs, (int)nbins, &a.bank, cell);
    if (e) return e;
    CFG_CUDA(cudaMemsetAsync(p->count, 0, sizeof(int) * (size_t)nbins, p->stream));
    CFG_CUDA(launch_rebin_count<T>(a, p->stream));
    CFG_CUDA(launch_scan(p->count, p->start, (int)nbins, 0, 1, p->scan_tmp, p->stream));
    if (a.bank.cell_order)
      CFG_CUDA(launch_scan(p->cls_count, p->cls_start, (int)nbins * a.bank.ncls, 2, dense_run(p->dim), p->cls_tmp,
                           p->stream));
    CFG_CUDA(launch_rebin_permute<T>(a, p->stream));
    CFG_CUDA(cudaStreamSynchronize(p->stream));
    cudaFree(p->idx);
    p->idx = idx;
    for (int k = 0; k < p->dim; ++k) {
      cudaFree(p->i0[k]);
      cudaFree(p->d[k]);
      p->i0[k] = i0[k];
      p->d[k] = d[k];
    }
  }
  p->method = method;
  p->cell_order = cell;
  p->sort = 1;
  p->opts.gpu_method = cell ? 5 : method;
  p->opts.gpu_sort = 1;
  for (int k = 0; k < 3; ++k) {
    p->bs[k] = bs[k];
    p->nb[k] = nb[k];
  }
  p->opts.gpu_binsizex = bs[0];
  p->opts.gpu_binsizey = bs[1];
  p->opts.gpu_binsizez = bs[2];
  if (method == 2) p->opts.gpu_maxsubprobsize = maxsub;
  p->nbins = (int)nbins;
  p->nsub = 0;
  if (method == 2 && p->pts_set) {
    e = build_subproblems(p);
    if (e) return e;
  }
  return 0;
}

// Device time (ms) of the plan's spread (type 1) or interp (type 2) stage for
// one batch, median of `reps` runs after one warm-up, on synthetic values.
template <typename T>
static int time_stage(Plan<T>* p, cplx_t<T>* scratch, cplx_t<T>* grid, int reps, float* ms) {
  SpreadArgs<T> a = spread_args(p);
  a.ntr = p->maxbatch;
  cudaEvent_t e0, e1;
  CFG_CUDA(cudaEventCreate(&e0));
  CFG_CUDA(cudaEventCreate(&e1));
  std::vector<float> t;
  for (int r = 0; r <= reps; ++r) {
    CFG_CUDA(cudaEventRecord(e0, p->stream));
    if (p->type == 1) {
      a.c_in = scratch;
      a.fw = grid;
      CFG_CUDA(run_spread(p, a));
    } else {
      a.fw_in = grid;
      a.c_out = scratch;
      CFG_CUDA(run_interp(p, a));
    }
    CFG_CUDA(cudaEventRecord(e1, p->stream));
    CFG_CUDA(cudaEventSynchronize(e1));
    float v = 0;
    CFG_CUDA(cudaEventElapsedTime(&v, e0, e1));
    if (r > 0) t.push_back(v);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  std::sort(t.begin(), t.end());
  *ms = t[t.size() / 2];
  return 0;
}

// The layout classes the autotuner times and the learned selector chooses
// among, in a fixed order: 0-2 method 1 with small / medium / large bins,
// 3-8 method 2 with small / medium / large bins x subproblem cap 256 / 1024,
// 9-11 method 5 (cell-run spread, type 1) with small / medium / large bins.
// Bin shapes per dimension: 1D 256 / 1024 / 4096; 2D 16^2 / 32^2 / 64^2;
// 3D 8x8x8 / 16x16x2 / 16x16x4 (clamped to the fine grid); for FP64 3D
// plans the large shape is 16x16xbz with the largest bz of 8, 6, 4 whose
// FP64 tile fits shared memory: at ns 11 a 16x16x8 bin holds ~16x the
// points of an 8^3 bin for 2x the tile, and interpolation on clustered 3D
// points at tol 1e-9 ran 24.5 ms (8^3) against 11.4 ms (16x16x8).  A class
// the plan cannot run (method 2 for 1D type 2, method 5 for type 2 or past
// its limits, a tile beyond shared memory) has ms = -2.
constexpr int kLayoutClasses = 12;

template <typename T>
static cufinufft_tune_entry layout_class(const Plan<T>* p, int cls) {
  static const int shapes[3][3][3] = {{{256, 1, 1}, {1024, 1, 1}, {4096, 1, 1}},
                                      {{16, 16, 1}, {32, 32, 1}, {64, 64, 1}},
                                      {{8, 8, 8}, {16, 16, 2}, {16, 16, 4}}};
  cufinufft_tune_entry e;
  e.method = cls < 3 ? 1 : (cls < 9 ? 2 : 5);
  const int shape = cls < 3 ? cls : (cls < 9 ? (cls - 3) / 2 : cls - 9);
  int sh[3] = {shapes[p->dim - 1][shape][0], shapes[p->dim - 1][shape][1], shapes[p->dim - 1][shape][2]};
  if (sizeof(T) == 8 && p->dim == 3 && shape == 2) {
    for (int bz : {8, 6, 4}) {
      const int b3[3] = {16, 16, bz};
      if (tile_cells(3, p->sp.ns, b3) * sizeof(cplx_t<T>) <= (size_t)max_smem_optin(p->device)) {
        sh[2] = bz;
        break;
      }
    }
  }
  e.binsizex = std::min(sh[0], p->nf[0]);
  e.binsizey = p->dim > 1 ? std::min(sh[1], p->nf[1]) : 1;
  e.binsizez = p->dim > 2 ? std::min(sh[2], p->nf[2]) : 1;
  e.maxsubprobsize = (cls < 3 || cls >= 9) ? 1024 : ((cls - 3) % 2 == 0 ? 256 : 1024);
  e.ms = -1.f;
  int bs[3] = {e.binsizex, e.binsizey, e.binsizez};
  if (e.method != 1 && p->type == 2 && p->dim == 1) e.ms = -2.f;
  if (e.method != 1 && tile_cells(p->dim, p->sp.ns, bs) * sizeof(cplx_t<T>) >
                           (size_t)max_smem_optin(p->device))
    e.ms = -2.f;
  if (e.method == 5) {
    long long nbins = 1;
    for (int k = 0; k < p->dim; ++k) nbins *= (p->nf[k] + bs[k] - 1) / bs[k];
    if (!cell_order_fits(p, bs, nbins) || run_smem_bytes(p, bs) > (size_t)max_smem_optin(p->device))
      e.ms = -2.f;
  }
  return e;
}

template <typename T>
static std::vector<cufinufft_tune_entry> tune_candidates(const Plan<T>* p) {
  std::vector<cufinufft_tune_entry> c;
  for (int k = 0; k < kLayoutClasses; ++k) c.push_back(layout_class(p, k));
  return c;
}

template <typename T>
static int autotune_impl(Plan<T>* p, cufinufft_tune_entry* out, int max_out, int* n_out) {
  if (p->type == 3) return CUFINUFFT_ERR_METHOD;
  if (!p->planned || !p->pts_set) return CUFINUFFT_ERR_GENERIC;
  std::vector<cufinufft_tune_entry> cand = tune_candidates(p);
  if (n_out) *n_out = 0;
  if (p->M == 0) return 0;
  cplx_t<T>* scratch = nullptr;
  CFG_CUDA(cudaMalloc(&scratch, sizeof(cplx_t<T>) * (size_t)p->M * p->maxbatch));
  // the grid the stage writes (type 1) or reads (type 2): the plan's own, or
  // a temporary one for a spread/interpolation-only plan (its grid is the
  // caller's); never the type-2 FFT input, whose padding must stay zero
  const size_t grid_bytes = sizeof(cplx_t<T>) * (size_t)grid_cells(p) * p->maxbatch;
  cplx_t<T>* grid = p->type == 1 ? p->fw : (p->fw2 ? p->fw2 : p->fw);
  cplx_t<T>* tmp_grid = nullptr;
  if (p->spread_only) {
    if (cudaMalloc(&tmp_grid, grid_bytes) != cudaSuccess) {
      cudaFree(scratch);
      return CUFINUFFT_ERR_ALLOC;
    }
    grid = tmp_grid;
  }
  // nonzero synthetic strengths/values (a zero tile would be skipped)
  CFG_CUDA(cudaMemsetAsync(scratch, 0x3f, sizeof(cplx_t<T>) * (size_t)p->M * p->maxbatch, p->stream));
  if (p->type == 2) CFG_CUDA(cudaMemsetAsync(grid, 0x3f, grid_bytes, p->stream));
  int best = -1;
  for (size_t i = 0; i < cand.size(); ++i) {
    if (cand[i].ms == -2.f) continue;  // not runnable for this plan
    int bs[3] = {cand[i].binsizex, cand[i].binsizey, cand[i].binsizez};
    int e = set_layout_impl(p, cand[i].method, bs, cand[i].maxsubprobsize);
    if (e) continue;
    if (p->type == 1) CFG_CUDA(cudaMemsetAsync(grid, 0, grid_bytes, p->stream));
    float ms = 0;
    e = time_stage(p, scratch, grid, 3, &ms);
    if (e) {
      cudaFree(scratch);
      cudaFree(tmp_grid);
      return e;
    }
    cand[i].ms = ms;
    if (best < 0 || ms < cand[best].ms) best = (int)i;
  }
  cudaFree(scratch);
  cudaFree(tmp_grid);
  if (best < 0) return CUFINUFFT_ERR_GENERIC;
  int bs[3] = {cand[best].binsizex, cand[best].binsizey, cand[best].binsizez};
  int e = set_layout_impl(p, cand[best].method, bs, cand[best].maxsubprobsize);
  if (e) return e;
  int n = 0;
  if (out) {
    // the chosen layout first, then every candidate tried
    out[n++] = cand[best];
    for (size_t i = 0; i < cand.size() && n < max_out; ++i) out[n++] = cand[i];
  }
  if (n_out) *n_out = n;
  return 0;
}

// ---------------------------------------------------------------------------
// Features and the learned selector.

template <typename T>
static int features_impl(Plan<T>* p, float* f) {
  if (p->type == 3) return CUFINUFFT_ERR_METHOD;
  if (!p->planned || !p->pts_set) return CUFINUFFT_ERR_GENERIC;
  int fb[3] = {1, 1, 1}, nb[3] = {1, 1, 1};
  long long nbins = 1;
  for (int k = 0; k < p->dim; ++k) {
    fb[k] = std::min(p->dim == 1 ? 64 : (p->dim == 2 ? 16 : 8), p->nf[k]);
    nb[k] = (p->nf[k] + fb[k] - 1) / fb[k];
    nbins *= nb[k];
  }
  std::vector<int> h((size_t)nbins, 0);
  if (p->M > 0) {
    int* counts = nullptr;
    CFG_CUDA(cudaMalloc(&counts, sizeof(int) * (size_t)nbins));
    CFG_CUDA(cudaMemsetAsync(counts, 0, sizeof(int) * (size_t)nbins, p->stream));
    const int* i0[3] = {p->i0[0], p->i0[1], p->i0[2]};
    cudaError_t e = launch_feature_count(p->dim, p->M, i0, fb, nb, counts, p->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(h.data(), counts, sizeof(int) * (size_t)nbins, cudaMemcpyDeviceToHost,
                          p->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(p->stream);
    cudaFree(counts);
    CFG_CUDA(e);
  }
  double sum = 0, sumsq = 0, mx = 0, occ = 0, sq_occ = 0;
  for (int c : h) {
    sum += c;
    sumsq += (double)c * c;
    if (c > mx) mx = c;
    if (c > 0) {
      occ += 1;
      sq_occ += (double)c * c;
    }
  }
  const double Nf = (double)grid_cells(p);
  const double Nm = (double)p->N[0] * p->N[1] * p->N[2];
  const double mean_all = sum / (double)nbins;
  const double mean_occ = occ > 0 ? sum / occ : 0.0;
  const double var_occ = occ > 0 ? std::max(0.0, sq_occ / occ - mean_occ * mean_occ) : 0.0;
  f[0] = (float)p->dim;
  f[1] = (float)p->type;
  f[2] = is_single<T>() ? 1.f : 0.f;
  f[3] = (float)p->sp.ns;
  f[4] = (float)std::log2((double)p->M + 1.0);
  f[5] = (float)std::log2(Nm);
  f[6] = (float)std::log2(Nf);
  f[7] = (float)std::log2(((double)p->M + 1.0) / Nf);
  f[8] = (float)std::log2((double)p->ntransf);
  f[9] = (float)(occ / (double)nbins);
  f[10] = (float)(mean_occ > 0 ? std::sqrt(var_occ) / mean_occ : 0.0);
  f[11] = (float)(mean_all > 0 ? std::log2(mx / mean_all) : 0.0);
  f[12] = (float)std::log2(mean_occ + 1.0);
  f[13] = (float)(sum > 0 ? std::log2((double)nbins * sumsq / (sum * sum)) : 0.0);
  return 0;
}

template <typename T>
static int apply_layout_class(Plan<T>* p, int cls);

// gpu_method 0 with a trained network: predict the twelve classes' relative
// times from the plan's features and switch to the fastest runnable one.
template <typename T>
static int select_layout(Plan<T>* p) {
  if (!kSelectorTrained || !p->auto_method || !p->pts_set || p->M == 0) return 0;
  float f[CUFINUFFT_MLP_FEATURES];
  int e = features_impl(p, f);
  if (e) return e;
  for (int k = 0; k < CUFINUFFT_MLP_FEATURES; ++k) f[k] = (f[k] - kSelMean[k]) / kSelStd[k];
  const int B = 1, Hd = CUFINUFFT_MLP_HIDDEN, K = CUFINUFFT_MLP_CLASSES;
  const size_t nfl = CUFINUFFT_MLP_PARAMS + CUFINUFFT_MLP_FEATURES + K + 2 * B * Hd;
  if (p->sel_buf == nullptr) {
    CFG_CUDA(cudaMalloc(&p->sel_buf, sizeof(float) * nfl));
    CFG_CUDA(cudaMemcpyAsync(p->sel_buf, kSelParams, sizeof(float) * CUFINUFFT_MLP_PARAMS,
                             cudaMemcpyHostToDevice, p->stream));
  }
  float* params = p->sel_buf;
  float* X = params + CUFINUFFT_MLP_PARAMS;
  float* Y = X + CUFINUFFT_MLP_FEATURES;
  float* work = Y + K;
  CFG_CUDA(cudaMemcpyAsync(X, f, sizeof(f), cudaMemcpyHostToDevice, p->stream));
  if (cufinufft_mlp_forward(params, X, B, Y, work, p->stream) != 0) return CUFINUFFT_ERR_CUDA;
  float y[CUFINUFFT_MLP_CLASSES];
  CFG_CUDA(cudaMemcpyAsync(y, Y, sizeof(y), cudaMemcpyDeviceToHost, p->stream));
  CFG_CUDA(cudaStreamSynchronize(p->stream));
  int best = -1;
  for (int k = 0; k < K; ++k) {
    cufinufft_tune_entry c = tune_candidates(p)[k];
    if (c.ms == -2.f) continue;
    if (best < 0 || y[k] < y[best]) best = k;
  }
  if (best < 0) return 0;
  return apply_layout_class(p, best);
}

template <typename T>
static int apply_layout_class(Plan<T>* p, int cls) {
  if (cls < 0 || cls >= kLayoutClasses) return CUFINUFFT_ERR_ARG;
  cufinufft_tune_entry c = tune_candidates(p)[cls];
  if (c.ms == -2.f) return CUFINUFFT_ERR_METHOD;
  int bs[3] = {c.binsizex, c.binsizey, c.binsizez};
  return set_layout_impl(p, c.method, bs, c.maxsubprobsize);
}

template <typename T, typename H>
static int makeplan_entry(int type, int dim, int* nmodes, int iflag, int ntransf, double tol,
                          int maxbatchsize, H** plan, cufinufft_opts* opts) {
  if (plan == nullptr) return CUFINUFFT_ERR_ARG;
  *plan = nullptr;
  if (dim < 1 || dim > 3 || nmodes == nullptr || ntransf < 1 || maxbatchsize < 0)
    return CUFINUFFT_ERR_ARG;
  for (int k = 0; k < dim; ++k)
    if (nmodes[k] < 1) return CUFINUFFT_ERR_ARG;
  H* h = new (std::nothrow) H();
  if (!h) return CUFINUFFT_ERR_ALLOC;
  *plan = h;
  Plan<T>* p = &h->p;
  p->device = opts ? opts->gpu_device_id : 0;
  if (type != 1 && type != 2 && type != 3) {
    p->type = type;
    p->dim = dim;
    return CUFINUFFT_ERR_GENERIC;
  }
  DeviceGuard g(p->device);
  if (!g.ok) return CUFINUFFT_ERR_CUDA;
  int ier;
  if (type == 3) {
    // implemented here; the reference returns 1 (src/cufinufft.cu:533-536)
    ier = makeplan_t3<T>(p, dim, iflag, ntransf, tol, maxbatchsize, opts);
    if (ier) release(p);
    return ier;
  }
  if constexpr (std::is_same<T, double>::value) {
    if (chain_wanted(type, tol, opts)) {
      ier = makeplan_chain(p, type, dim, nmodes, iflag, ntransf, tol, maxbatchsize, opts);
      if (ier) release(p);
      return ier;
    }
  }
  ier = makeplan_impl<T>(p, type, dim, nmodes, iflag, ntransf, tol, maxbatchsize, opts);
  if (ier) release(p);
  return ier;
}

}  // namespace cfg


using cfg::DeviceGuard;

template <typename H>
static int setpts_entry(H* h, int M, decltype(h->p.d[0]) x, decltype(h->p.d[0]) y,
                        decltype(h->p.d[0]) z, int N, decltype(h->p.d[0]) s, decltype(h->p.d[0]) t,
                        decltype(h->p.d[0]) u) {
  if (h == nullptr) return CUFINUFFT_ERR_GENERIC;
  DeviceGuard g(h->p.device);
  if (!g.ok) return CUFINUFFT_ERR_CUDA;
  if (h->p.type == 3) return cfg::setpts_t3(&h->p, M, x, y, z, N, s, t, u);
  return cfg::setpts_impl(&h->p, M, x, y, z);
}

template <typename H, typename C>
static int execute_entry(H* h, C* c, C* fk) {
  if (h == nullptr) return CUFINUFFT_ERR_GENERIC;
  DeviceGuard g(h->p.device);
  if (!g.ok) return CUFINUFFT_ERR_CUDA;
  return cfg::execute_impl(&h->p, c, fk);
}

template <typename H>
static int destroy_entry(H* h) {
  if (h == nullptr) return 1;  // reference: cannot destroy a NULL plan
  {
    DeviceGuard g(h->p.device);
    cfg::release(&h->p);
  }
  delete h;
  return 0;
}

// The plan that does the work: an FP64 plan's FP32 chain when it has one.
static cfg::Plan<float>* chain_of(cufinufft_plan h) { return h->p.lo; }
static cfg::Plan<float>* chain_of(cufinufftf_plan) { return nullptr; }
static void after_chain_call(cufinufft_plan h) {
  if (h->p.lo) cfg::sync_from_lo(&h->p);
}
static void after_chain_call(cufinufftf_plan) {}

template <typename P>
static int stage_times_impl(P* p, double* ms, long long* batches, int reset) {
  int e = cfg::collect_times(p);
  if (e) return e;
  e = cfg::take_status(p);
  if (e) return e;
  for (int k = 0; k < 3; ++k) ms[k] = p->stage_ms[k];
  if (batches) *batches = p->stage_batches;
  if (reset) {
    for (int k = 0; k < 3; ++k) p->stage_ms[k] = 0;
    p->stage_batches = 0;
  }
  return 0;
}

template <typename H>
static int stage_times_entry(H* h, double* ms, long long* batches, int reset) {
  if (!h || !ms) return CUFINUFFT_ERR_GENERIC;
  DeviceGuard g(h->p.device);
  if (cfg::Plan<float>* q = chain_of(h)) return stage_times_impl(q, ms, batches, reset);
  return stage_times_impl(&h->p, ms, batches, reset);
}

template <typename H>
static int set_layout_entry(H* h, int method, int bx, int by, int bz, int maxsub) {
  if (!h) return CUFINUFFT_ERR_GENERIC;
  DeviceGuard g(h->p.device);
  int bs[3] = {bx, by, bz};
  if (cfg::Plan<float>* q = chain_of(h)) {
    ++h->p.version;
    const int e = cfg::set_layout_impl(q, method, bs, maxsub);
    after_chain_call(h);
    return e;
  }
  return cfg::set_layout_impl(&h->p, method, bs, maxsub);
}
template <typename H>
static int autotune_entry(H* h, cufinufft_tune_entry* out, int max_out, int* n_out) {
  if (!h) return CUFINUFFT_ERR_GENERIC;
  DeviceGuard g(h->p.device);
  if (cfg::Plan<float>* q = chain_of(h)) {
    ++h->p.version;
    const int e = cfg::autotune_impl(q, out, max_out, n_out);
    after_chain_call(h);
    return e;
  }
  return cfg::autotune_impl(&h->p, out, max_out, n_out);
}

template <typename H>
static int set_stream_entry(H* h, cudaStream_t stream) {
  if (!h || !h->p.planned) return CUFINUFFT_ERR_GENERIC;
  auto set = [stream](auto* p) {
    p->stream = stream ? stream : p->own;
    if (p->have_fft && cufftSetStream(p->fft, p->stream) != CUFFT_SUCCESS) return CUFINUFFT_ERR_CUFFT;
    if (p->have_fft_rem && cufftSetStream(p->fft_rem, p->stream) != CUFFT_SUCCESS) return CUFINUFFT_ERR_CUFFT;
    return 0;
  };
  if (cfg::Plan<float>* q = chain_of(h)) {
    const int e = set(q);
    after_chain_call(h);
    return e;
  }
  return set(&h->p);
}

template <typename H>
static int set_timing_entry(H* h, int on) {
  if (!h) return CUFINUFFT_ERR_GENERIC;
  h->p.timing = on != 0;
  if (cfg::Plan<float>* q = chain_of(h)) q->timing = on != 0;
  return 0;
}

extern "C" {

int cufinufft_default_opts(int type, int dim, cufinufft_opts* opts) {
  return cfg::default_opts(type, dim, opts);
}
int cufinufftf_default_opts(int type, int dim, cufinufft_opts* opts) {
  return cfg::default_opts(type, dim, opts);
}

int cufinufft_makeplan(int type, int dim, int* nmodes, int iflag, int ntransf, double tol,
                       int maxbatchsize, cufinufft_plan* plan, cufinufft_opts* opts) {
  return cfg::makeplan_entry<double>(type, dim, nmodes, iflag, ntransf, tol, maxbatchsize, plan,
                                     opts);
}
int cufinufftf_makeplan(int type, int dim, int* nmodes, int iflag, int ntransf, float tol,
                        int maxbatchsize, cufinufftf_plan* plan, cufinufft_opts* opts) {
  return cfg::makeplan_entry<float>(type, dim, nmodes, iflag, ntransf, (double)tol, maxbatchsize,
                                    plan, opts);
}

int cufinufft_setpts(int M, double* x, double* y, double* z, int N, double* s, double* t, double* u,
                     cufinufft_plan plan) {
  return setpts_entry(plan, M, x, y, z, N, s, t, u);
}
int cufinufftf_setpts(int M, float* x, float* y, float* z, int N, float* s, float* t, float* u,
                      cufinufftf_plan plan) {
  return setpts_entry(plan, M, x, y, z, N, s, t, u);
}

int cufinufft_execute(cuDoubleComplex* c, cuDoubleComplex* fk, cufinufft_plan plan) {
  return execute_entry(plan, reinterpret_cast<double2*>(c), reinterpret_cast<double2*>(fk));
}
int cufinufftf_execute(cuFloatComplex* c, cuFloatComplex* fk, cufinufftf_plan plan) {
  return execute_entry(plan, reinterpret_cast<float2*>(c), reinterpret_cast<float2*>(fk));
}

int cufinufft_destroy(cufinufft_plan plan) { return destroy_entry(plan); }
int cufinufftf_destroy(cufinufftf_plan plan) { return destroy_entry(plan); }

int cufinufft_set_stream(cufinufft_plan plan, cudaStream_t stream) {
  return set_stream_entry(plan, stream);
}
int cufinufftf_set_stream(cufinufftf_plan plan, cudaStream_t stream) {
  return set_stream_entry(plan, stream);
}

int cufinufft_set_timing(cufinufft_plan plan, int on) { return set_timing_entry(plan, on); }
int cufinufftf_set_timing(cufinufftf_plan plan, int on) { return set_timing_entry(plan, on); }

int cufinufft_stage_times(cufinufft_plan plan, double* ms, long long* batches, int reset) {
  return stage_times_entry(plan, ms, batches, reset);
}
int cufinufftf_stage_times(cufinufftf_plan plan, double* ms, long long* batches, int reset) {
  return stage_times_entry(plan, ms, batches, reset);
}

int cufinufft_set_layout(cufinufft_plan plan, int method, int bx, int by, int bz, int maxsub) {
  return set_layout_entry(plan, method, bx, by, bz, maxsub);
}
int cufinufftf_set_layout(cufinufftf_plan plan, int method, int bx, int by, int bz, int maxsub) {
  return set_layout_entry(plan, method, bx, by, bz, maxsub);
}
int cufinufft_autotune(cufinufft_plan plan, cufinufft_tune_entry* out, int max_out, int* n_out) {
  return autotune_entry(plan, out, max_out, n_out);
}
int cufinufftf_autotune(cufinufftf_plan plan, cufinufft_tune_entry* out, int max_out, int* n_out) {
  return autotune_entry(plan, out, max_out, n_out);
}

int cufinufft_features(cufinufft_plan plan, float* features) {
  if (!plan || !features) return CUFINUFFT_ERR_GENERIC;
  DeviceGuard g(plan->p.device);
  if (plan->p.lo) return cfg::features_impl(plan->p.lo, features);
  return cfg::features_impl(&plan->p, features);
}
int cufinufftf_features(cufinufftf_plan plan, float* features) {
  if (!plan || !features) return CUFINUFFT_ERR_GENERIC;
  DeviceGuard g(plan->p.device);
  return cfg::features_impl(&plan->p, features);
}
int cufinufft_set_layout_class(cufinufft_plan plan, int cls) {
  if (!plan) return CUFINUFFT_ERR_GENERIC;
  DeviceGuard g(plan->p.device);
  if (plan->p.lo) {
    ++plan->p.version;
    const int e = cfg::apply_layout_class(plan->p.lo, cls);
    cfg::sync_from_lo(&plan->p);
    return e;
  }
  return cfg::apply_layout_class(&plan->p, cls);
}
int cufinufftf_set_layout_class(cufinufftf_plan plan, int cls) {
  if (!plan) return CUFINUFFT_ERR_GENERIC;
  DeviceGuard g(plan->p.device);
  return cfg::apply_layout_class(&plan->p, cls);
}

int cufinufft_set_width_rule(int rule, int* previous) { return cfg::set_width_rule(rule, previous); }

int cufinufft_get_info(cufinufft_plan plan, cufinufft_plan_info* info) {
  if (!plan || !info) return CUFINUFFT_ERR_GENERIC;
  if (plan->p.lo) {
    cfg::fill_info(plan->p.lo, info);
    info->beta = plan->p.sp.beta;  // the FP64 plan's kernel (the chain's is beta, c rounded to FP32)
    info->es_c = plan->p.sp.c;
    info->chain_fp32 = 1;
    return 0;
  }
  cfg::fill_info(&plan->p, info);
  return 0;
}
int cufinufftf_get_info(cufinufftf_plan plan, cufinufft_plan_info* info) {
  if (!plan || !info) return CUFINUFFT_ERR_GENERIC;
  cfg::fill_info(&plan->p, info);
  return 0;
}

}  // extern "C"
