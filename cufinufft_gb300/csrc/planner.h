// planner.h -- host-side plan arithmetic (no device code).
#pragma once

#include <vector>

#include "kernels.h"

namespace cfg {

struct SpreaderParams {
  int ns;
  double beta;     // ES_beta in plan precision, widened to double
  double c;        // ES_c in plan precision, widened to double
  double upsampfac;
};

// Kernel width and ES parameters from the tolerance, restating
// setup_spreader (contrib/spreadinterp.cpp:6-67) for the FP32 (single=true)
// or FP64 build.  Returns 0, the warning 1 (tolerance below machine epsilon
// or width clipped to 16), or the errors 7 / 8.
// width_rule 0 is the reference's width, ns = ceil(-log10(tol/10)) at
// upsampfac 2, which leaves errors of 1-4 tol (see width_error_bound);
// width_rule 1 takes the narrowest width whose measured error bound for
// `dim` meets tol (at most the reference's width at machine precision; the
// warning 1 when even that misses).  The kernel's shape (beta, c) follows
// the reference's formulas at the chosen width either way.
int setup_spreader(double tol, double upsampfac, int kerevalmeth, bool single, SpreaderParams* sp,
                   int width_rule = 0, int dim = 3);

// Upper bound on the relative l2 error of a transform of dimension dim at
// kernel width ns: the worst error the FP64 oracle left against direct sums
// at that width (uniform random points and data), plus 25% margin.
double width_error_bound(int ns, int dim, double upsampfac);
// The narrowest width in [2, cap] whose bound meets tol, cap being the
// reference rule's width at this precision's machine epsilon; sets *warn
// (when given) and returns cap if none does.
int width_for_tol(double tol, int dim, double upsampfac, bool single, int* warn);

// contrib/utils.cpp:3-22 and contrib/common.cpp:24-37.
int next235beven(int n, int b);
int set_nf_type12(int ms, double upsampfac, int ns, int gpu_method, int bs);

// n-point Gauss-Legendre rule on [-1,1] by Newton iteration on the Legendre
// three-term recurrence; nodes in decreasing order.
void gauss_legendre(int n, double* x, double* w);

// Quadrature nodes/values for the kernel's Fourier series
// (contrib/common.cpp:84-96): q = floor(2 + 1.5 ns) nodes z_n on (0, ns/2),
// f_n = (ns/2) w_n phi(z_n).
void fseries_nodes(const SpreaderParams& sp, FseriesNodes* out);

// ES kernel value phi(x) in FP64.
double es_kernel(double x, const SpreaderParams& sp);

// Piecewise-polynomial fit of the kernel (kerevalmeth 1): for tap j and
// offset d in [0,1), phi(d - ns/2 + j) ~ sum_k a_k z^(deg-k), z = 2d-1.
// Coefficients are returned row-major [k][j], highest degree first, fitted
// by Chebyshev interpolation in long double.
std::vector<double> horner_fit(const SpreaderParams& sp, int degree);

}  // namespace cfg
