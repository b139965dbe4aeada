// ref_shim.cpp -- C entry points around the reference's own host-side helper
// code (contrib/), compiled from the reference sources by oracle/Makefile into
// oracle/_ref/libref_contrib.so.
//
// TEST INFRASTRUCTURE ONLY: it exists to pin the oracle (nufft_oracle.c)
// against the reference's own arithmetic and to generate the golden fixtures
// under tests/golden/.  It is compiled twice, once with -DSINGLE (the
// reference's FP32 build) and once without (FP64); REF_SUFFIX names the
// exported symbols of each build.
#include <cuda_runtime.h>
#include <cufinufft_opts.h>
#include "spreadinterp.h"
#include "common.h"
#include "dirft.h"

#ifdef SINGLE
#define REF_FN(name) name##_f
#else
#define REF_FN(name) name##_d
#endif

extern "C" {

// contrib/spreadinterp.cpp:6 setup_spreader
int REF_FN(ref_setup_spreader)(double eps, double upsampfac, int kerevalmeth,
                               int* ns, double* beta, double* c) {
  SPREAD_OPTS o;
  int ier = setup_spreader(o, (FLT)eps, (FLT)upsampfac, kerevalmeth);
  *ns = o.nspread;
  *beta = (double)o.ES_beta;
  *c = (double)o.ES_c;
  return ier;
}

// contrib/common.cpp:24 SET_NF_TYPE12 (after setup_spreader for ns)
int REF_FN(ref_set_nf)(int ms, double tol, int gpu_method, int bs) {
  SPREAD_OPTS o;
  cufinufft_opts opts;
  opts.upsampfac = 2.0;
  opts.gpu_method = gpu_method;
  opts.gpu_kerevalmeth = 0;
  setup_spreader(o, (FLT)tol, (FLT)2.0, 0);
  int nf = 0;
  SET_NF_TYPE12(ms, opts, o, &nf, bs);
  return nf;
}

// contrib/common.cpp:39 onedim_fseries_kernel (host version of the fseries)
int REF_FN(ref_fseries)(int nf, double tol, double* out) {
  SPREAD_OPTS o;
  setup_spreader(o, (FLT)tol, (FLT)2.0, 0);
  FLT* tmp = new FLT[nf / 2 + 1];
  onedim_fseries_kernel(nf, tmp, o);
  for (int k = 0; k <= nf / 2; ++k) out[k] = (double)tmp[k];
  delete[] tmp;
  return o.nspread;
}

// contrib/spreadinterp.cpp:69 evaluate_kernel
double REF_FN(ref_evaluate_kernel)(double x, double tol) {
  SPREAD_OPTS o;
  setup_spreader(o, (FLT)tol, (FLT)2.0, 0);
  return (double)evaluate_kernel((FLT)x, o);
}

// contrib/dirft2d.cpp:7 / :41 dirft2d1 / dirft2d2 (interleaved complex I/O)
void REF_FN(ref_dirft2d1)(int nj, const double* x, const double* y,
                          const double* c, int iflag, int ms, int mt,
                          double* f) {
  FLT* xx = new FLT[nj];
  FLT* yy = new FLT[nj];
  CPX* cc = new CPX[nj];
  CPX* ff = new CPX[(size_t)ms * mt];
  for (int j = 0; j < nj; ++j) {
    xx[j] = (FLT)x[j];
    yy[j] = (FLT)y[j];
    cc[j] = CPX((FLT)c[2 * j], (FLT)c[2 * j + 1]);
  }
  dirft2d1(nj, xx, yy, cc, iflag, ms, mt, ff);
  for (size_t m = 0; m < (size_t)ms * mt; ++m) {
    f[2 * m] = (double)ff[m].real();
    f[2 * m + 1] = (double)ff[m].imag();
  }
  delete[] xx; delete[] yy; delete[] cc; delete[] ff;
}

void REF_FN(ref_dirft2d2)(int nj, const double* x, const double* y, double* c,
                          int iflag, int ms, int mt, const double* f) {
  FLT* xx = new FLT[nj];
  FLT* yy = new FLT[nj];
  CPX* cc = new CPX[nj];
  CPX* ff = new CPX[(size_t)ms * mt];
  for (int j = 0; j < nj; ++j) { xx[j] = (FLT)x[j]; yy[j] = (FLT)y[j]; }
  for (size_t m = 0; m < (size_t)ms * mt; ++m)
    ff[m] = CPX((FLT)f[2 * m], (FLT)f[2 * m + 1]);
  dirft2d2(nj, xx, yy, cc, iflag, ms, mt, ff);
  for (int j = 0; j < nj; ++j) {
    c[2 * j] = (double)cc[j].real();
    c[2 * j + 1] = (double)cc[j].imag();
  }
  delete[] xx; delete[] yy; delete[] cc; delete[] ff;
}

}  // extern "C"
