// planner.cpp -- host-side plan arithmetic: kernel width and shape, fine-grid
// sizes, Gauss-Legendre quadrature for the kernel's Fourier series, and the
// piecewise-polynomial kernel fit.
#include "planner.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>

namespace cfg {

// Worst relative l2 error of the FP64 oracle against direct sums, divided by
// the reference's accuracy model for the width (10^(1-ns) at upsampfac 2,
// exp(-pi ns sqrt(1 - 1/upsampfac)) otherwise), over uniform random points,
// types 1 and 2, two mode shapes and three seeds per dimension; rows ns =
// 2..16, columns dim 1..3.  Printed by oracle/width_table.py.
static const double kWidthErr2[15][3] = {
    {0.6, 0.837, 0.97},   {0.696, 0.968, 1.24}, {1.58, 2.07, 2.79}, {0.725, 1.06, 1.72},
    {0.703, 1.04, 1.69},  {0.872, 1.21, 1.44},  {1.11, 1.48, 1.39}, {1.31, 1.86, 2.14},
    {1.48, 2.17, 3.45},   {1.46, 2.07, 3.74},   {1.54, 2.25, 3.54}, {1.78, 2.45, 2.65},
    {2.84, 3.02, 2.7},    {17.7, 3.98, 4.23},   {166, 14.6, 12}};
static const double kWidthErr125[15][3] = {
    {2.63, 3.61, 4},      {2.7, 3.88, 3.95},    {2.85, 4.56, 4.31}, {2.96, 3.52, 4.73},
    {2.23, 3.09, 4.56},   {1.81, 2.87, 3.29},   {2.21, 2.94, 2.12}, {2.77, 3.32, 2.21},
    {3.31, 4.27, 4.41},   {3.52, 4.42, 5.18},   {2.92, 6.16, 5.77}, {2.86, 5.57, 5.81},
    {2.47, 4.52, 3.76},   {2.87, 4.04, 1.83},   {3.82, 4.5, 1.32}};

double width_error_bound(int ns, int dim, double upsampfac) {
  if (ns < 2 || ns > kMaxNS || dim < 1 || dim > 3) return 1.0;
  const double model = upsampfac == 2.0 ? std::pow(10.0, 1 - ns)
                                        : std::exp(-M_PI * ns * std::sqrt(1.0 - 1.0 / upsampfac));
  const double r = (upsampfac == 2.0 ? kWidthErr2 : kWidthErr125)[ns - 2][dim - 1];
  return 1.25 * r * model;  // a quarter of margin over the worst case measured
}

int width_for_tol(double tol, int dim, double upsampfac, bool single, int* warn) {
  // the widest kernel the reference's own rule uses in this precision (its
  // width at the machine-precision floor, contrib/spreadinterp.cpp:35-49)
  SpreaderParams cap;
  setup_spreader(0.0, upsampfac, 0, single, &cap);
  for (int ns = 2; ns <= cap.ns; ++ns)
    if (width_error_bound(ns, dim, upsampfac) <= tol) return ns;
  if (warn) *warn = 1;
  return cap.ns;
}

int setup_spreader(double tol, double upsampfac, int kerevalmeth, bool single, SpreaderParams* sp,
                   int width_rule, int dim) {
  if (upsampfac != 2.0) {
    // HORNER_WRONG_BETA: the reference has no polynomial table for sigma !=
    // 2; the fitted polynomials here serve any sigma unless the reference's
    // refusal is asked for (CUFINUFFT_HORNER_SIGMA2_ONLY=1)
    if (kerevalmeth == 1) {
      const char* v = std::getenv("CUFINUFFT_HORNER_SIGMA2_ONLY");
      if (v && v[0] == '1') return 8;
    }
    if (upsampfac <= 1.0) return 7;   // ERR_UPSAMPFAC_TOO_SMALL
  }
  int ier = 0, ns;
  double beta, c;
  if (single) {
    // FP32 build: FLT = float throughout (contrib/utils_fp.h:34, EPSILON 6e-8)
    float eps = (float)tol;
    const float epsmach = (float)6e-08;
    if (eps < epsmach) { eps = epsmach; ier = 1; }
    ns = (int)std::ceil(-std::log10(eps / 10.0f));
    if (upsampfac != 2.0) {
      const float usf = (float)upsampfac, pif = (float)M_PI;
      ns = (int)std::ceil(-std::log(eps) / (pif * std::sqrt(1.0f - 1.0f / usf)));
    }
    if (ns < 2) ns = 2;
    if (ns > kMaxNS) { ns = kMaxNS; ier = 1; }
    if (width_rule == 1) ns = width_for_tol(tol, dim, upsampfac, true, &ier);
    const float cf = (float)(4.0 / (double)(float)(ns * ns));
    float bon = 2.30f;
    if (ns == 2) bon = 2.20f;
    if (ns == 3) bon = 2.26f;
    if (ns == 4) bon = 2.38f;
    if (upsampfac != 2.0) {
      const float usf = (float)upsampfac;
      bon = 0.97f * (float)M_PI * (1.0f - 1.0f / (2.0f * usf));
    }
    beta = (double)(bon * (float)ns);
    c = (double)cf;
  } else {
    double eps = tol;
    const double epsmach = 1.1e-16;
    if (eps < epsmach) { eps = epsmach; ier = 1; }
    ns = (int)std::ceil(-std::log10(eps / 10.0));
    if (upsampfac != 2.0) ns = (int)std::ceil(-std::log(eps) / (M_PI * std::sqrt(1.0 - 1.0 / upsampfac)));
    if (ns < 2) ns = 2;
    if (ns > kMaxNS) { ns = kMaxNS; ier = 1; }
    if (width_rule == 1) ns = width_for_tol(tol, dim, upsampfac, false, &ier);
    c = 4.0 / (double)(ns * ns);
    double bon = 2.30;
    if (ns == 2) bon = 2.20;
    if (ns == 3) bon = 2.26;
    if (ns == 4) bon = 2.38;
    if (upsampfac != 2.0) bon = 0.97 * M_PI * (1.0 - 1.0 / (2.0 * upsampfac));
    beta = bon * (double)ns;
  }
  sp->ns = ns;
  sp->beta = beta;
  sp->c = c;
  sp->upsampfac = upsampfac;
  return ier;
}

int next235beven(int n, int b) {
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

int set_nf_type12(int ms, double upsampfac, int ns, int gpu_method, int bs) {
  long long nf = (long long)(upsampfac * (double)ms);
  if (nf < 2 * ns) nf = 2 * ns;
  if (nf < 2147483647LL) nf = next235beven((int)nf, gpu_method == 4 ? bs : 1);
  return (int)nf;
}

void gauss_legendre(int n, double* x, double* w) {
  for (int i = 0; i < n; ++i) {
    double z = std::cos(M_PI * (i + 0.75) / (n + 0.5));
    double dp = 1.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= n; ++k) {
        double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      double pn = n == 1 ? z : p1, pm = n == 1 ? 1.0 : p0;
      dp = n * (z * pn - pm) / (z * z - 1.0);
      double dz = pn / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-16) {
        p0 = 1.0;
        p1 = z;
        for (int k = 2; k <= n; ++k) {
          double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
          p0 = p1;
          p1 = p2;
        }
        pn = n == 1 ? z : p1;
        pm = n == 1 ? 1.0 : p0;
        dp = n * (z * pn - pm) / (z * z - 1.0);
        break;
      }
    }
    x[i] = z;
    w[i] = 2.0 / ((1.0 - z * z) * dp * dp);
  }
}

double es_kernel(double x, const SpreaderParams& sp) {
  if (std::fabs(x) >= 0.5 * sp.ns) return 0.0;
  return std::exp(sp.beta * std::sqrt(1.0 - sp.c * x * x));
}

void fseries_nodes(const SpreaderParams& sp, FseriesNodes* out) {
  const double J2 = sp.ns / 2.0;
  const int q = (int)(2 + 3.0 * J2);
  std::vector<double> z(2 * q), w(2 * q);
  gauss_legendre(2 * q, z.data(), w.data());
  out->q = q;
  for (int n = 0; n < q; ++n) {
    out->z[n] = z[n] * J2;
    out->f[n] = J2 * w[n] * es_kernel(out->z[n], sp);
  }
}

std::vector<double> horner_fit(const SpreaderParams& sp, int degree) {
  const int ns = sp.ns, K = degree;
  std::vector<double> coef((size_t)(K + 1) * ns, 0.0);
  std::vector<long double> nodes(K + 1), vals(K + 1), cheb(K + 1), mono(K + 1);
  for (int m = 0; m <= K; ++m) nodes[m] = std::cos((long double)M_PI * (m + 0.5L) / (K + 1));
  for (int j = 0; j < ns; ++j) {
    for (int m = 0; m <= K; ++m) {
      long double d = (nodes[m] + 1.0L) / 2.0L;
      long double x = d - ns / 2.0L + j;
      long double z = sp.c * x * x;
      vals[m] = (std::fabs((double)x) < ns / 2.0) ? std::exp(sp.beta * std::sqrt(1.0L - z)) : 0.0L;
    }
    // Chebyshev coefficients of the interpolant at the Chebyshev points
    for (int k = 0; k <= K; ++k) {
      long double s = 0;
      for (int m = 0; m <= K; ++m)
        s += vals[m] * std::cos((long double)M_PI * k * (m + 0.5L) / (K + 1));
      cheb[k] = s * (k == 0 ? 1.0L : 2.0L) / (K + 1);
    }
    // Chebyshev -> monomial: T_0 = 1, T_1 = z, T_{k+1} = 2 z T_k - T_{k-1}
    std::vector<long double> tkm1(K + 1, 0), tk(K + 1, 0), tkp1(K + 1, 0);
    for (int i = 0; i <= K; ++i) mono[i] = 0;
    tkm1[0] = 1;  // T_0
    mono[0] += cheb[0];
    if (K >= 1) {
      tk[1] = 1;  // T_1
      mono[1] += cheb[1];
    }
    for (int k = 1; k < K; ++k) {
      for (int i = 0; i <= K; ++i) tkp1[i] = -tkm1[i] + (i > 0 ? 2 * tk[i - 1] : 0);
      for (int i = 0; i <= K; ++i) mono[i] += cheb[k + 1] * tkp1[i];
      tkm1 = tk;
      tk = tkp1;
    }
    // highest degree first: row r holds z^(K - r)
    for (int r = 0; r <= K; ++r) coef[(size_t)r * ns + j] = (double)mono[K - r];
  }
  return coef;
}

}  // namespace cfg
