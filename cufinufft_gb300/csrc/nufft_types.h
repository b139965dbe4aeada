// nufft_types.h -- plain-data types shared by host code and kernels.
#pragma once

#include <cuComplex.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace cfg {

constexpr int kMaxNS = 16;      // widest kernel (reference MAX_NSPREAD)
constexpr int kMaxNQuad = 100;  // Gauss-Legendre nodes cap (MAX_NQUAD)

template <typename T> struct cplx;
template <> struct cplx<float> { using type = float2; };
template <> struct cplx<double> { using type = double2; };
template <typename T> using cplx_t = typename cplx<T>::type;

// Degree of the fitted piecewise polynomials (kerevalmeth 1).  FP32: ns + 2.
// FP64: the least degree at which the fit error (relative to the kernel's
// peak, over every tap interval) comes within 1.5x of its floor -- the
// kernel's own truncation level, ~exp(-beta) -- plus one as margin.  Measured
// with the fit's Chebyshev construction at upsampfac 2 (the upsampfac 1.25
// kernels need at most the same): the least degree is ns + 1 for ns <= 6,
// ns for 7-8, ns - 1 for 9-12, ns - 2 for 13-14 and ns - 3 for 15-16, so
// wide FP64 kernels evaluate 4 to 6 fewer Horner steps per value than with
// degree ns + 3.
template <typename T> constexpr int horner_degree(int ns) {
  constexpr int kDegF64[17] = {0, 0, 4, 5, 6, 7, 8, 8, 9, 9, 10, 11, 12, 12, 13, 13, 13};
  return sizeof(T) == 4 ? ns + 2 : kDegF64[ns < 2 ? 2 : (ns > 16 ? 16 : ns)];
}

// Constants that place one coordinate axis on the fine grid (see
// place_coord in device_common.cuh).  s_hi + s_lo = nf/(2 pi); o_* = nf *
// {1.5, 0.5, -0.5} for x < -pi, -pi <= x < pi, x >= pi; ns/2 = half_int +
// half_frac.
template <typename T> struct AxisMap {
  T s_hi, s_lo, o_lo, o_mid, o_hi, half_frac;
  int nf, half_int;
};

constexpr int kMaxHornerRows = kMaxNS + 4;  // degree <= ns + 3

// Kernel-evaluation constants: phi(x) = exp(beta*sqrt(1 - c x^2)), or, when
// horner != 0, the fitted polynomials: coef[k*ns + j] is the coefficient of
// z^(deg-k) for tap j.  The coefficients travel inside the kernel's
// parameter block, so the unrolled evaluation reads them straight from the
// constant bank.
// FP64 plans also carry the fitted polynomials as FP32 pairs (hi + lo, the
// double-float interpolation kernel evaluates them without FP64 units),
// scaled by 2^-E with E = round(beta log2 e) so that kernel values are ~1
// (the kernel's peak e^beta, and the grid's 1/e^(d beta) scale, would leave
// FP32's exponent range in 3D at wide kernels).
template <typename T> struct DFCoef {};
template <> struct DFCoef<double> {
  float hi[kMaxHornerRows * kMaxNS];
  float lo[kMaxHornerRows * kMaxNS];
};

template <typename T> struct KernelCoeffs {
  T beta, c;
  T e_beta, bl2e;                    // e^beta and beta log2(e) (FP32 kernel evaluation)
  int horner;
  const T* coef_g;                   // device copy, read by kernel_tap (runtime tap index)
  T coef[kMaxHornerRows * kMaxNS];
  DFCoef<T> df;
};

// Bin-sorted points in plan memory (written by setpts).
template <typename T> struct SortedPts {
  const int* idx;     // sorted position -> caller's point index
  const int* i0[3];   // first tap per axis, wrapped into [0, nf)
  const T* d[3];      // tap offset per axis in [0,1)
  int M;
};

// Fine-grid geometry and bin/subproblem tables.
struct GridGeom {
  int nf[3];
  long long Nf;       // nf1*nf2*nf3
};

// Per-subproblem header written at setpts: first sorted point, point
// count, tile origin (cells).  Two 16-byte words.
struct __align__(16) SubHdr {
  int p0, np, ox, oy;
  int oz, pad0, pad1, pad2;
};

struct BinTables {
  int bs[3];          // bin size (cells) per axis
  int nb[3];          // bins per axis
  int nbins;
  const int* count;       // points per bin            [nbins]
  const int* start;       // exclusive scan of count   [nbins+1]
  const int* sub_start;   // exclusive scan of subproblems per bin [nbins+1]
  const int* sub_to_bin;  // subproblem -> bin          [nsub]
  int nsub;
  int maxsub;             // points per subproblem cap
  const SubHdr* hdr;      // subproblem headers [nsub], or null (derived from the tables above)
};

// Everything a spread or interp launch needs.
template <typename T> struct SpreadArgs {
  SortedPts<T> pts;
  BinTables bins;
  KernelCoeffs<T> kc;
  GridGeom g;
  const cplx_t<T>* c_in;    // type 1 strengths (ntr*M)
  cplx_t<T>* c_out;         // type 2 output (ntr*M)
  cplx_t<T>* fw;            // fine grids (ntr*Nf), type 1 output
  const cplx_t<T>* fw_in;   // type 2 input grid
  int ntr;
  int M;
  int variant;              // kernel family: 0 default, 1 one thread per point, 2 warp-cooperative
  int run;                  // method 2 spreading over cell-ordered points (cell-run kernel)
  const unsigned char* sub_dense;  // run: subproblems that start on a dense cell
  const int* sub_ndense;           // run: leading points on dense cells per subproblem
  // Interpolation tile waits (bulk copies): status[0] is set when a wait ran
  // out and the tile was loaded cell by cell instead, status[1] when the copy
  // had still not landed after a second full wait.  Host-mapped memory the
  // next call on the plan reads; null: not recorded.
  int* status;
  int tma_wait_test;        // nonzero: every tile's first wait gives up at once (tests)
  int fp64_df;              // FP64: subproblem interpolation in double-float (k_interp_sm_df)
};

// Cells of one subproblem tile: the bin plus the ns-1 cells its points
// reach beyond it along each axis.
inline size_t tile_cells(int dim, int ns, const int bs[3]) {
  size_t n = (size_t)(bs[0] + ns - 1);
  if (dim > 1) n *= (size_t)(bs[1] + ns - 1);
  if (dim > 2) n *= (size_t)(bs[2] + ns - 1);
  return n;
}

}  // namespace cfg
