/*
 * nufft_oracle.c -- CPU restatement of the cuFINUFFT v1.3 type-1/type-2 NUFFT
 * algorithm, in FP64.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle and the timed CPU
 * baseline.  Only tests/, __graft_entry__.smoke() and bench.py (its
 * cpu_baseline leg and its --impl reference arm) may load it.  The GPU product
 * path never links, calls or falls back to it.
 *
 * Every routine cites the reference routine it restates (paths are relative to
 * the cufinufft v1.3 source tree).  Complex arrays are interleaved (re, im)
 * doubles.  Grid layout: x fastest, then y, then z, then transform index.
 * Mode layout (fk): CMCL order, k_d = -N_d/2 .. (N_d-1)/2, k1 fastest.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_MAX_NSPREAD 16
#define ORC_MAX_NQUAD 100
#define ORC_PI 3.14159265358979323846
#define ORC_1_2PI 0.159154943091895336   /* contrib/utils.h:18 */

/* Error codes, contrib/utils.h:28-36. */
#define ORC_WARN_EPS_TOO_SMALL 1
#define ORC_ERR_UPSAMPFAC_TOO_SMALL 7
#define ORC_HORNER_WRONG_BETA 8

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void orc_set_num_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/* ------------------------------------------------------------------------ */
/* Spreader parameters: contrib/spreadinterp.cpp:6-67 (setup_spreader).
 * single != 0 reproduces the SINGLE build, where FLT=float: eps, the log10,
 * ES_c and beta are float quantities (contrib/utils_fp.h:34 EPSILON=6e-8),
 * otherwise FLT=double (EPSILON=1.1e-16, contrib/utils_fp.h:43). */
int orc_setup_spreader(double eps_in, double upsampfac, int kerevalmeth,
                       int single, int* ns_out, double* beta_out,
                       double* c_out) {
  if (upsampfac != 2.0) {
    if (kerevalmeth == 1) return ORC_HORNER_WRONG_BETA;
    if (upsampfac <= 1.0) return ORC_ERR_UPSAMPFAC_TOO_SMALL;
  }
  int ier = 0, ns;
  double beta, c;
  if (single) {
    float eps = (float)eps_in;
    const float epsmach = (float)6e-08;
    if (eps < epsmach) { eps = epsmach; ier = ORC_WARN_EPS_TOO_SMALL; }
    ns = (int)ceilf(-log10f(eps / 10.0f));
    if (upsampfac != 2.0) {
      float pif = (float)ORC_PI;
      float usf = (float)upsampfac;
      ns = (int)ceil(-logf(eps) / (pif * sqrtf(1.0f - 1.0f / usf)));
    }
    if (ns < 2) ns = 2;
    if (ns > ORC_MAX_NSPREAD) { ns = ORC_MAX_NSPREAD; ier = ORC_WARN_EPS_TOO_SMALL; }
    float cf = (float)(4.0 / (double)(float)(ns * ns));
    float bon = 2.30f;
    if (ns == 2) bon = 2.20f;
    if (ns == 3) bon = 2.26f;
    if (ns == 4) bon = 2.38f;
    if (upsampfac != 2.0) {
      float gamma = 0.97f, usf = (float)upsampfac;
      bon = gamma * (float)ORC_PI * (1.0f - 1.0f / (2.0f * usf));
    }
    float bf = bon * (float)ns;
    beta = bf;
    c = cf;
  } else {
    double eps = eps_in;
    const double epsmach = 1.1e-16;
    if (eps < epsmach) { eps = epsmach; ier = ORC_WARN_EPS_TOO_SMALL; }
    ns = (int)ceil(-log10(eps / 10.0));
    if (upsampfac != 2.0)
      ns = (int)ceil(-log(eps) / (ORC_PI * sqrt(1.0 - 1.0 / upsampfac)));
    if (ns < 2) ns = 2;
    if (ns > ORC_MAX_NSPREAD) { ns = ORC_MAX_NSPREAD; ier = ORC_WARN_EPS_TOO_SMALL; }
    c = 4.0 / (double)(ns * ns);
    double bon = 2.30;
    if (ns == 2) bon = 2.20;
    if (ns == 3) bon = 2.26;
    if (ns == 4) bon = 2.38;
    if (upsampfac != 2.0) bon = 0.97 * ORC_PI * (1.0 - 1.0 / (2.0 * upsampfac));
    beta = bon * (double)ns;
  }
  *ns_out = ns;
  *beta_out = beta;
  *c_out = c;
  return ier;
}

/* ES kernel, contrib/spreadinterp.cpp:69-81: exp(beta*sqrt(1-c x^2)) for
 * |x| < ns/2, else 0 (unnormalised; the deconvolution uses the same kernel). */
double orc_es_kernel(double x, int ns, double beta, double c) {
  if (fabs(x) >= 0.5 * ns) return 0.0;
  return exp(beta * sqrt(1.0 - c * x * x));
}

/* contrib/utils.cpp:3-22 (next235beven): smallest even integer >= n whose
 * prime factors are 2, 3, 5 only and which is a multiple of b. */
int orc_next235beven(int n, int b) {
  if (n <= 2) return 2;
  if (n % 2 == 1) n += 1;
  int nplus = n - 2, numdiv = 2;
  while (numdiv > 1 || nplus % b != 0) {
    nplus += 2;
    numdiv = nplus;
    while (numdiv % 2 == 0) numdiv /= 2;
    while (numdiv % 3 == 0) numdiv /= 3;
    while (numdiv % 5 == 0) numdiv /= 5;
  }
  return nplus;
}

/* contrib/common.cpp:24-37 (SET_NF_TYPE12): fine-grid size for ms modes. */
int orc_set_nf_type12(int ms, double upsampfac, int ns, int gpu_method, int bs) {
  long long nf = (long long)(upsampfac * (double)ms);
  if (nf < 2 * ns) nf = 2 * ns;
  if (nf < 2147483647LL) {
    if (gpu_method == 4) nf = orc_next235beven((int)nf, bs);
    else nf = orc_next235beven((int)nf, 1);
  }
  return (int)nf;
}

/* Gauss-Legendre rule on [-1,1] with n nodes by Newton iteration on the
 * three-term recurrence (a published textbook method; it replaces the
 * reference's legendre_compute_glr, contrib/legendre_rule_fast.c:15, which
 * is not restated).  Nodes are returned in decreasing order. */
void orc_gauss_legendre(int n, double* x, double* w) {
  for (int i = 0; i < n; ++i) {
    double z = cos(ORC_PI * (i + 0.75) / (n + 0.5));
    double dp = 1.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= n; ++k) {
        double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      double pn = (n == 1) ? z : p1;
      double pnm1 = (n == 1) ? 1.0 : p0;
      dp = n * (z * pn - pnm1) / (z * z - 1.0);
      double dz = pn / dp;
      z -= dz;
      if (fabs(dz) < 1e-16) {
        /* one more evaluation for the derivative at the converged node */
        p0 = 1.0; p1 = z;
        for (int k = 2; k <= n; ++k) {
          double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
          p0 = p1;
          p1 = p2;
        }
        pn = (n == 1) ? z : p1;
        pnm1 = (n == 1) ? 1.0 : p0;
        dp = n * (z * pn - pnm1) / (z * z - 1.0);
        break;
      }
    }
    x[i] = z;
    w[i] = 2.0 / ((1.0 - z * z) * dp * dp);
  }
}

/* Fourier-series samples of the ES kernel on the fine grid,
 * contrib/common.cpp:84-124 (onedim_fseries_kernel_precomp/_compute) and
 * src/common.cu:16-45 (FseriesKernelCompute):
 *   fwkerhalf[k] = sum_n 2 f_n cos(k * theta_n),  k = 0..nf/2,
 *   f_n = (ns/2) w_n phi(z_n),  theta_n = 2 pi (nf/2 - z_n)/nf,
 * with q = floor(2 + 1.5 ns) positive Gauss-Legendre nodes z_n on (0, ns/2). */
void orc_fseries(int nf, int ns, double beta, double c, double* fwkerhalf) {
  double J2 = ns / 2.0;
  int q = (int)(2 + 3.0 * J2);
  double z[2 * ORC_MAX_NQUAD], w[2 * ORC_MAX_NQUAD];
  double f[ORC_MAX_NQUAD], zz[ORC_MAX_NQUAD];
  orc_gauss_legendre(2 * q, z, w);
  for (int n = 0; n < q; ++n) {  /* the q positive nodes */
    zz[n] = z[n] * J2;
    f[n] = J2 * w[n] * orc_es_kernel(zz[n], ns, beta, c);
  }
  /* nf is even, so cos(k theta_n) = (-1)^k cos(2 pi k z_n / nf): the small
   * argument keeps the phase accurate to ~1e-15 rad for every k. */
  for (int k = 0; k <= nf / 2; ++k) {
    double s = 0.0;
    for (int n = 0; n < q; ++n)
      s += 2.0 * f[n] * cos(2.0 * ORC_PI * ((double)k * zz[n] / (double)nf));
    fwkerhalf[k] = (k % 2) ? -s : s;
  }
}

/* RESCALE macro with pirange=1, contrib/spreadinterp.h:36-38: maps
 * x in [-3pi,3pi) to [0,N) folding one period on each side. */
static inline double orc_rescale(double x, int N) {
  double sh = (x < -ORC_PI) ? 1.5 : (x >= ORC_PI ? -0.5 : 0.5);
  return (x * ORC_1_2PI + sh) * (double)N;
}

static inline int orc_wrap(int i, int n) {
  return i < 0 ? i + n : (i >= n ? i - n : i);
}

/* Kernel values along one dimension for the taps start..start+ns-1 of a
 * point at rescaled position xr; start = ceil(xr - ns/2).  Restates
 * eval_kernel_vec (src/cuspreadinterp.h:33-40).  The reference loops
 * xstart..xend, which is ns taps unless xr-ns/2 is an integer; the extra tap
 * then has kernel value 0, so ns taps carry the whole sum. */
static inline int orc_taps(double xr, int ns, double beta, double c,
                           double* ker) {
  int start = (int)ceil(xr - ns / 2.0);
  for (int j = 0; j < ns; ++j)
    ker[j] = orc_es_kernel((double)(start + j) - xr, ns, beta, c);
  return start;
}

/* Coloured bin schedule for a race-free parallel spread: bins of width bs
 * (bs >= ns) in each dimension; a point belongs to the bin of its first tap.
 * Colour per dimension: b%2, and colour 2 for the last bin when nbins is odd,
 * so bins that share a colour never touch the same fine-grid cell.  A bin
 * writes its own cells and the ns-1 cells after them (periodically), so a
 * last bin narrower than ns-1 cells would let the halo of the bin before it
 * wrap into bin 0; such a sliver is merged into the bin before it (the last
 * bin is then between bs and 2 bs - 1 cells wide).  This is
 * the CPU form of the subproblem method (src/2d/spreadinterp2d.cu:152-231):
 * points are grouped by bin and each group is added to the grid by one
 * thread. */
static inline int orc_colour(int b, int nb) {
  if (nb % 2 == 1 && b == nb - 1 && nb > 1) return 2;
  return b % 2;
}

/* Type-1 spread (spread_direction 1) of ntr transforms:
 * fw[t][cell] += c[t][j] * prod_d phi(cell_d - xr_d), restating
 * Spread_{1,2,3}d_NUptsdriven (src/2d/spreadinterp2d.cu:16-57,
 * src/3d/spreadinterp3d.cu:73-127, src/1d/spreadinterp1d.cu:16-44).
 * fw must be zeroed by the caller.  x/y/z are FP64 copies of the user's
 * coordinates in [-3pi,3pi). */
void orc_spread(int dim, int nf1, int nf2, int nf3, int M, const double* x,
                const double* y, const double* z, int ntr, const double* c,
                double* fw, int ns, double beta, double es_c) {
  int nf[3] = {nf1, dim > 1 ? nf2 : 1, dim > 2 ? nf3 : 1};
  int bs[3], nb[3];
  int bdef = dim == 1 ? 256 : (dim == 2 ? 32 : 16);
  for (int d = 0; d < 3; ++d) {
    bs[d] = d < dim ? (bdef < ns ? ns : bdef) : 1;
    if (d < dim && bs[d] > nf[d]) bs[d] = nf[d];
    nb[d] = (nf[d] + bs[d] - 1) / bs[d];
    if (nb[d] > 1 && nf[d] - (nb[d] - 1) * bs[d] < ns - 1) nb[d] -= 1;
  }
  long long nbins = (long long)nb[0] * nb[1] * nb[2];
  /* bin every point by its first tap */
  int* bin = (int*)malloc(sizeof(int) * (size_t)(M > 0 ? M : 1));
  long long* cnt = (long long*)calloc((size_t)nbins + 1, sizeof(long long));
  for (int j = 0; j < M; ++j) {
    const double* co[3] = {x, y, z};
    int bidx[3] = {0, 0, 0};
    for (int d = 0; d < dim; ++d) {
      double xr = orc_rescale(co[d][j], nf[d]);
      int s = (int)ceil(xr - ns / 2.0);
      s = ((s % nf[d]) + nf[d]) % nf[d];
      bidx[d] = s / bs[d] < nb[d] ? s / bs[d] : nb[d] - 1;
    }
    bin[j] = bidx[0] + nb[0] * (bidx[1] + nb[1] * bidx[2]);
    cnt[bin[j] + 1]++;
  }
  for (long long b = 0; b < nbins; ++b) cnt[b + 1] += cnt[b];
  int* order = (int*)malloc(sizeof(int) * (size_t)(M > 0 ? M : 1));
  long long* fill = (long long*)malloc(sizeof(long long) * (size_t)nbins);
  memcpy(fill, cnt, sizeof(long long) * (size_t)nbins);
  for (int j = 0; j < M; ++j) order[fill[bin[j]]++] = j;
  free(fill);
  size_t Nf = (size_t)nf[0] * nf[1] * nf[2];
  for (int colour = 0; colour < 27; ++colour) {
    int cz = colour / 9, cy = (colour / 3) % 3, cx = colour % 3;
    if ((dim < 3 && cz) || (dim < 2 && cy)) continue;
#pragma omp parallel for schedule(dynamic, 1)
    for (long long b = 0; b < nbins; ++b) {
      int bx = (int)(b % nb[0]), by = (int)((b / nb[0]) % nb[1]),
          bz = (int)(b / ((long long)nb[0] * nb[1]));
      if (orc_colour(bx, nb[0]) != cx || orc_colour(by, nb[1]) != cy ||
          orc_colour(bz, nb[2]) != cz)
        continue;
      double k1[ORC_MAX_NSPREAD], k2[ORC_MAX_NSPREAD], k3[ORC_MAX_NSPREAD];
      for (long long p = cnt[b]; p < cnt[b + 1]; ++p) {
        int j = order[p];
        int s1 = orc_taps(orc_rescale(x[j], nf[0]), ns, beta, es_c, k1);
        int s2 = 0, s3 = 0;
        int n2 = 1, n3 = 1;
        k2[0] = 1.0;
        k3[0] = 1.0;
        if (dim > 1) { s2 = orc_taps(orc_rescale(y[j], nf[1]), ns, beta, es_c, k2); n2 = ns; }
        if (dim > 2) { s3 = orc_taps(orc_rescale(z[j], nf[2]), ns, beta, es_c, k3); n3 = ns; }
        for (int t = 0; t < ntr; ++t) {
          double cr = c[2 * ((size_t)t * M + j)], ci = c[2 * ((size_t)t * M + j) + 1];
          double* g = fw + 2 * Nf * (size_t)t;
          for (int dz = 0; dz < n3; ++dz) {
            int iz = dim > 2 ? orc_wrap(s3 + dz, nf[2]) : 0;
            for (int dy = 0; dy < n2; ++dy) {
              int iy = dim > 1 ? orc_wrap(s2 + dy, nf[1]) : 0;
              double kyz = k2[dy] * k3[dz];
              size_t row = ((size_t)iz * nf[1] + iy) * nf[0];
              for (int dx = 0; dx < ns; ++dx) {
                int ix = orc_wrap(s1 + dx, nf[0]);
                double kv = k1[dx] * kyz;
                g[2 * (row + ix)] += cr * kv;
                g[2 * (row + ix) + 1] += ci * kv;
              }
            }
          }
        }
      }
    }
  }
  free(order);
  free(cnt);
  free(bin);
}

/* Type-2 interpolation: c[t][j] = sum_cells fw[t][cell] * prod_d
 * phi(cell_d - xr_d), restating Interp_{1,2,3}d_NUptsdriven
 * (src/2d/spreadinterp2d.cu:516-553, src/3d/spreadinterp3d.cu:654-703,
 * src/1d/spreadinterp1d.cu:233-258). */
void orc_interp(int dim, int nf1, int nf2, int nf3, int M, const double* x,
                const double* y, const double* z, int ntr, double* c,
                const double* fw, int ns, double beta, double es_c) {
  int nf[3] = {nf1, dim > 1 ? nf2 : 1, dim > 2 ? nf3 : 1};
  size_t Nf = (size_t)nf[0] * nf[1] * nf[2];
#pragma omp parallel for schedule(static)
  for (int j = 0; j < M; ++j) {
    double k1[ORC_MAX_NSPREAD], k2[ORC_MAX_NSPREAD], k3[ORC_MAX_NSPREAD];
    int s1 = orc_taps(orc_rescale(x[j], nf[0]), ns, beta, es_c, k1);
    int s2 = 0, s3 = 0, n2 = 1, n3 = 1;
    k2[0] = 1.0;
    k3[0] = 1.0;
    if (dim > 1) { s2 = orc_taps(orc_rescale(y[j], nf[1]), ns, beta, es_c, k2); n2 = ns; }
    if (dim > 2) { s3 = orc_taps(orc_rescale(z[j], nf[2]), ns, beta, es_c, k3); n3 = ns; }
    for (int t = 0; t < ntr; ++t) {
      const double* g = fw + 2 * Nf * (size_t)t;
      double ar = 0.0, ai = 0.0;
      for (int dz = 0; dz < n3; ++dz) {
        int iz = dim > 2 ? orc_wrap(s3 + dz, nf[2]) : 0;
        for (int dy = 0; dy < n2; ++dy) {
          int iy = dim > 1 ? orc_wrap(s2 + dy, nf[1]) : 0;
          double kyz = k2[dy] * k3[dz];
          size_t row = ((size_t)iz * nf[1] + iy) * nf[0];
          for (int dx = 0; dx < ns; ++dx) {
            int ix = orc_wrap(s1 + dx, nf[0]);
            double kv = k1[dx] * kyz;
            ar += g[2 * (row + ix)] * kv;
            ai += g[2 * (row + ix) + 1] * kv;
          }
        }
      }
      c[2 * ((size_t)t * M + j)] = ar;
      c[2 * ((size_t)t * M + j) + 1] = ai;
    }
  }
}

/* Deconvolution (type 1) and amplification (type 2), restating
 * Deconvolve_{1,2,3}d / Amplify_{1,2,3}d (src/deconvolve_wrapper.cu:14-121):
 * mode k_d (index i_d in 0..N_d-1, k_d = i_d - N_d/2) sits at fine-grid
 * index k_d mod nf_d and is divided by prod_d fwkerhalf_d[|k_d|].
 * dir 1: fk = fw / ker.  dir 2: fw = 0 everywhere, then fw[mode] = fk / ker. */
void orc_deconvolve(int dir, int dim, int ms, int mt, int mu, int nf1, int nf2,
                    int nf3, int ntr, double* fw, double* fk,
                    const double* ker1, const double* ker2,
                    const double* ker3) {
  int N[3] = {ms, dim > 1 ? mt : 1, dim > 2 ? mu : 1};
  int nf[3] = {nf1, dim > 1 ? nf2 : 1, dim > 2 ? nf3 : 1};
  size_t Nf = (size_t)nf[0] * nf[1] * nf[2];
  size_t Nm = (size_t)N[0] * N[1] * N[2];
  if (dir == 2) memset(fw, 0, sizeof(double) * 2 * Nf * (size_t)ntr);
#pragma omp parallel for schedule(static)
  for (long long m = 0; m < (long long)Nm; ++m) {
    int i1 = (int)(m % N[0]), i2 = (int)((m / N[0]) % N[1]),
        i3 = (int)(m / ((long long)N[0] * N[1]));
    int k1 = i1 - N[0] / 2, k2 = i2 - N[1] / 2, k3 = i3 - N[2] / 2;
    int w1 = k1 >= 0 ? k1 : nf[0] + k1;
    int w2 = k2 >= 0 ? k2 : nf[1] + k2;
    int w3 = k3 >= 0 ? k3 : nf[2] + k3;
    double kv = ker1[abs(k1)];
    if (dim > 1) kv *= ker2[abs(k2)];
    if (dim > 2) kv *= ker3[abs(k3)];
    size_t widx = ((size_t)w3 * nf[1] + w2) * nf[0] + w1;
    for (int t = 0; t < ntr; ++t) {
      double* g = fw + 2 * (Nf * (size_t)t + widx);
      double* f = fk + 2 * (Nm * (size_t)t + (size_t)m);
      if (dir == 1) { f[0] = g[0] / kv; f[1] = g[1] / kv; }
      else { g[0] = f[0] / kv; g[1] = f[1] / kv; }
    }
  }
}

/* FP64 direct sums (the accuracy oracle), restating contrib/dirft2d.cpp:7-64
 * (dirft2d1/dirft2d2) for any dimension, with each phase computed directly
 * as k.x (no winding) so that the sum is accurate to FP64 rounding.
 * Type 1 on a subset of modes:  f[m] = sum_j c[j] exp(i*sgn*(k(m).x_j)),
 *   modes[m] = flat CMCL index of the requested mode.
 * Type 2 on a subset of targets: c[m] = sum_k fk[k] exp(i*sgn*(k.x_{tg[m]})). */
void orc_dirft_type1(int dim, int ms, int mt, int mu, int M, const double* x,
                     const double* y, const double* z, const double* c,
                     int iflag, int nmodes, const long long* modes,
                     double* out) {
  int N[3] = {ms, dim > 1 ? mt : 1, dim > 2 ? mu : 1};
  double sgn = iflag >= 0 ? 1.0 : -1.0;
#pragma omp parallel for schedule(dynamic, 1)
  for (int m = 0; m < nmodes; ++m) {
    long long f = modes[m];
    double k1 = (double)(f % N[0]) - N[0] / 2;
    double k2 = (double)((f / N[0]) % N[1]) - N[1] / 2;
    double k3 = (double)(f / ((long long)N[0] * N[1])) - N[2] / 2;
    double ar = 0.0, ai = 0.0;
    for (int j = 0; j < M; ++j) {
      double ph = k1 * x[j];
      if (dim > 1) ph += k2 * y[j];
      if (dim > 2) ph += k3 * z[j];
      ph *= sgn;
      double cs = cos(ph), sn = sin(ph);
      ar += c[2 * j] * cs - c[2 * j + 1] * sn;
      ai += c[2 * j] * sn + c[2 * j + 1] * cs;
    }
    out[2 * m] = ar;
    out[2 * m + 1] = ai;
  }
}

void orc_dirft_type2(int dim, int ms, int mt, int mu, const double* x,
                     const double* y, const double* z, const double* fk,
                     int iflag, int ntargets, const long long* targets,
                     double* out) {
  int N[3] = {ms, dim > 1 ? mt : 1, dim > 2 ? mu : 1};
  long long Nm = (long long)N[0] * N[1] * N[2];
  double sgn = iflag >= 0 ? 1.0 : -1.0;
#pragma omp parallel for schedule(dynamic, 1)
  for (int m = 0; m < ntargets; ++m) {
    long long j = targets[m];
    double ar = 0.0, ai = 0.0;
    for (long long f = 0; f < Nm; ++f) {
      double k1 = (double)(f % N[0]) - N[0] / 2;
      double ph = k1 * x[j];
      if (dim > 1) ph += ((double)((f / N[0]) % N[1]) - N[1] / 2) * y[j];
      if (dim > 2) ph += ((double)(f / ((long long)N[0] * N[1])) - N[2] / 2) * z[j];
      ph *= sgn;
      double cs = cos(ph), sn = sin(ph);
      ar += fk[2 * f] * cs - fk[2 * f + 1] * sn;
      ai += fk[2 * f] * sn + fk[2 * f + 1] * cs;
    }
    out[2 * m] = ar;
    out[2 * m + 1] = ai;
  }
}

/* FP64 direct sum of the type-3 transform (nonuniform to nonuniform), the
 * accuracy reference for type 3: f[m] = sum_j c[j] exp(i*sgn*(s_k.x_j)) at
 * the targets k = targets[m].  The reference library reserves type 3 in its
 * interface (src/cufinufft.cu:533-536) without implementing it, so this sum
 * is the only check.  x/y/z: M source points; s/t/u: target frequencies. */
void orc_dirft_type3(int dim, int M, const double* x, const double* y,
                     const double* z, const double* c, const double* s,
                     const double* t, const double* u, int iflag,
                     int ntargets, const long long* targets, double* out) {
  double sgn = iflag >= 0 ? 1.0 : -1.0;
#pragma omp parallel for schedule(dynamic, 1)
  for (int m = 0; m < ntargets; ++m) {
    long long k = targets[m];
    double ar = 0.0, ai = 0.0;
    for (int j = 0; j < M; ++j) {
      double ph = s[k] * x[j];
      if (dim > 1) ph += t[k] * y[j];
      if (dim > 2) ph += u[k] * z[j];
      ph *= sgn;
      double cs = cos(ph), sn = sin(ph);
      ar += c[2 * j] * cs - c[2 * j + 1] * sn;
      ai += c[2 * j] * sn + c[2 * j + 1] * cs;
    }
    out[2 * m] = ar;
    out[2 * m + 1] = ai;
  }
}
