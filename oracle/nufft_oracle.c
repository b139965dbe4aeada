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

static inline int orc_wrap(int i, int n) {
  return i < 0 ? i + n : (i >= n ? i - n : i);
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

#define ORC_R double
#define ORC_SFX(n) n
#include "oracle_stages.inc"
#undef ORC_R
#undef ORC_SFX
#define ORC_R float
#define ORC_SFX(n) n##_f32
#include "oracle_stages.inc"
#undef ORC_R
#undef ORC_SFX

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
