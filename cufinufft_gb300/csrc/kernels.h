// kernels.h -- host-callable launchers for every device stage.  Each returns
// the cudaError_t of its launch (cudaSuccess when nothing needed launching).
#pragma once

#include <cuda_runtime.h>

#include "nufft_types.h"

namespace cfg {

// si_<prec><dim>.cu
template <typename T, int DIM>
cudaError_t spread_dim(int method, int ns, const SpreadArgs<T>& a, cudaStream_t s);
template <typename T, int DIM>
cudaError_t interp_dim(int method, int ns, const SpreadArgs<T>& a, cudaStream_t s);

// setpts.cu -- bin sort of the nonuniform points.
// Order inside a bin for the shared-memory (method 2) kernels.  A point's
// bank class is the tile address of its first tap modulo ncls (16 for FP32
// complex, 8 for FP64: one 128-byte bank sweep); the sort places a bin's
// points round-robin over the classes, so any ncls consecutive points of a
// bin differ in class and a half-warp's tile accesses (first tap + the same
// offset for every point) fall in distinct banks.  cls_count == nullptr
// keeps plain bin order.
//
// cell_order = 1 instead groups a bin's points for the cell-run spread (class
// = cell index inside the bin, ncls = cells per bin): points on cells holding
// at least dense_min points first, sorted by cell, then the others in arbitrary
// order; cls_start is the exclusive scan of those dense counts over all
// (bin, cell) keys, sparse_count a per-bin counter for the others.
// Points on one cell that make it dense for the cell-run spread: a run must
// amortise the flush of ns^d tap sums, 36 in 2D at ns = 6, 343 in 3D at 7.
constexpr int dense_run(int dim) { return dim == 3 ? 16 : 8; }

struct BankOrder {
  int* cls_count;   // [nbins * ncls], zeroed before counting
  int ncls;         // power of two (bank classes) or cells per bin
  int tx, ty;       // tile row length and rows per plane (bin size + ns - 1)
  int cell_order;
  const int* cls_start;  // [nbins * ncls + 1] (cell_order only)
  int* sparse_count;     // [nbins], zeroed before permuting (cell_order only)
  int dense_min;         // dense_run(dim) (cell_order only)
};

template <typename T> struct PlaceArgs {
  const T* x[3];           // caller's coordinates (device)
  AxisMap<T> ax[3];
  int dim;
  int M;
  int bs[3];               // bin size per axis (cells)
  int nb[3];               // bins per axis
  // outputs
  int* idx;                // sorted position -> caller index
  int* i0[3];
  T* d[3];
  int* count;              // [nbins] (must be zeroed before bin_count)
  int* rank;               // [M] rank of the point inside its bin (or its class)
  const int* start;        // [nbins+1] exclusive scan of count
  BankOrder bank;
};
template <typename T> cudaError_t launch_bin_count(const PlaceArgs<T>& a, cudaStream_t s);
template <typename T> cudaError_t launch_permute(const PlaceArgs<T>& a, cudaStream_t s);
template <typename T> cudaError_t launch_place_unsorted(const PlaceArgs<T>& a, cudaStream_t s);

// FP64 coordinates placed in FP64 (fold, rescale, first tap) with the tap
// offset in [0,1) rounded to FP32, in caller order (idx[i] = i): the input
// of an FP32 chain's sort in an FP64 plan.
struct NarrowPlaceArgs {
  const double* x[3];
  AxisMap<double> ax[3];
  int dim, M;
  int* idx;
  int* i0[3];
  float* d[3];
};
cudaError_t launch_place_narrow(const NarrowPlaceArgs& a, cudaStream_t s);

// Complex FP64 <-> FP32 conversion of n values.
cudaError_t launch_narrow_complex(const double2* in, float2* out, long long n, cudaStream_t s);
cudaError_t launch_widen_complex(const float2* in, double2* out, long long n, cudaStream_t s);

// Re-binning of already placed points (no caller coordinates needed): the
// bin of a point depends only on its first taps i0, so a new bin layout is a
// counting sort of the stored arrays into fresh ones.
template <typename T> struct RebinArgs {
  int dim, M;
  int bs[3], nb[3];
  const int* src_idx;
  const int* src_i0[3];
  const T* src_d[3];
  int* idx;
  int* i0[3];
  T* d[3];
  int* count;      // [nbins], zeroed before rebin_count
  int* rank;       // [M]
  const int* start;
  BankOrder bank;
};
template <typename T> cudaError_t launch_rebin_count(const RebinArgs<T>& a, cudaStream_t s);
template <typename T> cudaError_t launch_rebin_permute(const RebinArgs<T>& a, cudaStream_t s);

// Point counts over fixed feature bins (fb cells per axis) from the stored
// first taps; counts must be zeroed.
cudaError_t launch_feature_count(int dim, int M, const int* const i0[3], const int fb[3],
                                 const int nb[3], int* counts, cudaStream_t s);

// Exclusive scan of n ints: out[0..n] (out[n] = total).  mode 0 scans the
// values, mode 1 scans ceil(v / div), mode 2 scans v where v >= div (else
// 0).  tmp needs scan_tmp_ints(n) ints.
int scan_tmp_ints(int n);
cudaError_t launch_scan(const int* in, int* out, int n, int mode, int div, int* tmp,
                        cudaStream_t s);
// sub_to_bin[s] = the bin b with sub_start[b] <= s < sub_start[b+1].
// Cell order: flag the subproblems whose first point lies on a dense cell
// (those go to the cell-run kernel, the others to the warp-cooperative one).
struct SubClassArgs {
  const int* sub_to_bin;
  const int* sub_start;
  const int* start;
  const int* i0[3];
  const int* cls_count;
  int bs[3];
  int dim, maxsub, ncls, nsub, dense_min;
  unsigned char* dense;
  // optional: per subproblem, its leading points on dense cells (a bin's
  // dense cells come first), from the scanned dense counts and bin counts
  const int* cls_start;
  const int* count;
  int* ndense;
};
cudaError_t launch_classify_subproblems(const SubClassArgs& a, cudaStream_t s);
// The driver's cuTensorMapEncodeTiled, looked up once per process (null if
// the driver has none).  makeplan looks it up for type-2 plans, so the first
// lookup does not happen inside a stream capture.
void* tma_encoder();

cudaError_t launch_sub_to_bin(const int* sub_start, int nbins, int nsub, int* sub_to_bin,
                              cudaStream_t s);
// sub_to_bin plus the subproblem headers (hdr[nsub]) of bins bs x nb holding
// count[b] points from start[b] on, at most maxsub per subproblem.
cudaError_t launch_sub_headers(const int* sub_start, const int* start, const int* count, int nbins,
                               int nsub, int maxsub, const int bs[3], const int nb[3], int* sub_to_bin,
                               SubHdr* hdr, cudaStream_t s);

// deconv.cu
struct FseriesNodes {
  double z[kMaxNQuad / 2];   // quadrature nodes on (0, ns/2)
  double f[kMaxNQuad / 2];   // (ns/2) w_n phi(z_n)
  int q;
};

// type3.cu -- elementwise steps of the type-3 transform.  x: the points the
// step reads (sources for the prephase, target frequencies for the post
// factor); C, D: centres of the sources and targets; hg = h gam, the scale
// from target frequency to the inner type-2 frequency; sgn = +-1.
template <typename T>
struct Type3Phase {
  const T* x[3];
  double C[3], D[3], hg[3];
  double sgn;
  int dim;
};
int minmax_partials();
template <typename T>
cudaError_t launch_minmax(const T* a, long long n, double* partial, int* nblocks, cudaStream_t s);
template <typename T>
cudaError_t launch_affine(const T* a, long long n, double centre, double scale, T* out, cudaStream_t s);
template <typename T>
cudaError_t launch_prephase(const Type3Phase<T>& a, long long n, cplx_t<T>* pre, cudaStream_t s);
template <typename T>
cudaError_t launch_postfactor(const Type3Phase<T>& a, const FseriesNodes& nodes, long long n, cplx_t<T>* post,
                              cudaStream_t s);
template <typename T>
cudaError_t launch_cmul_rows(const cplx_t<T>* u, const cplx_t<T>* w, long long n, int ntr, cplx_t<T>* v,
                             cudaStream_t s);
// fac[d][i] = 1 / fhat_d(|i - N_d/2|), i = 0..N_d-1, FP64 evaluation.
template <typename T>
cudaError_t launch_fseries(const FseriesNodes& nodes, int dim, const int nf[3], const int N[3],
                           T* fac0, T* fac1, T* fac2, cudaStream_t s);
// Type 1: fk[t][m] = fw[t][mode m on the grid] * prod_d fac_d.
template <typename T>
cudaError_t launch_deconvolve(int dim, const int nf[3], const int N[3], const cplx_t<T>* fw,
                              cplx_t<T>* fk, const T* fac0, const T* fac1, const T* fac2,
                              int ntr, cudaStream_t s);
// Type 2: fw[t] = 0 except the mode cells, fw[t][mode m] = fk[t][m] * prod fac.
template <typename T>
cudaError_t launch_amplify_modes(int dim, const int nf[3], const int N[3], cplx_t<T>* fw,
                                 const cplx_t<T>* fk, const T* fac0, const T* fac1, const T* fac2,
                                 int ntr, cudaStream_t s);
// Pruned line FFTs (fftpass.cu).  A pass transforms nlines lines of length
// L; line l has indices la = l % A and lb = l / A.  Each side (input, output)
// maps a line and a position to memory:
//   line offset = ma * sa + mb * sb, ma = la, or the grid position of mode
//   index la when acorner is set (mode la - Na/2 at (la - Na/2) mod nfa),
//   and likewise for b;
//   pmode 0: all L positions w at w * sp;
//   pmode 1: the Np modes only, compact: mode index i at i * sp;
//   pmode 2: the Np modes only, in place in the grid: at w(i) * sp,
// where mode index i in [0, Np) is FFT index (i - Np/2) mod L.  Positions
// outside the modes read as zero (input) or are not written (output).
// Factors fa[la] * fb[lb] * fp[i] multiply on load (fac_on_out = 0) or on
// store (1); null factors are 1.
struct LineSide {
  long long st, sa, sb, sp;
  int acorner, Na, nfa;
  int bcorner, Nb, nfb;
  int pmode, Np;
};

template <typename T>
struct LineArgs {
  int L, dir, G, log2G, A, nlines, ntr, nrad;
  int p2;               // power-of-two kernel (block = G * L / 16 threads)
  int rad[24];
  const cplx_t<T>* tw;  // exp(dir 2 pi i m / L), m = 0..L-1
  const cplx_t<T>* in;
  cplx_t<T>* out;
  LineSide si, so;
  const T* fa;
  const T* fb;
  const T* fp;
  int fac_on_out;
};

// Pruned power-of-two passes (halffft.cu) for grids nf in {256, ..., 2048}
// with at most nf/2 modes per axis: per axis F = nf / Mp warp FFTs of Mp
// points (one per output or input class q, grid position F r + q) over the
// lines that hold modes.
enum HalfKind { kHalfT2Rows = 0, kHalfT2Cols = 1, kHalfT1Cols = 2, kHalfT1Rows = 3 };
template <typename T>
struct HalfPass {
  int kind;
  int Mp, F, Fb;              // per-warp FFT size, classes (the axis has F Mp grid points),
                              // classes per block of the strided type-2 pass
  int N;                      // modes on this axis
  const cplx_t<T>* in;
  cplx_t<T>* out;
  const cplx_t<T>* tw;        // W^t = exp(dir 2 pi i t / nf), t < nf
  int ntr;                    // transforms; transform t at in + t in_tr, out + t out_tr
  long long in_tr, out_tr;
  // rows passes: nlines contiguous lines, line g at in + g in_row / out + g out_row;
  // cols passes: in_row / out_row are the strides along the axis
  int nlines;
  long long in_row, out_row;
  const T* fac;               // rows passes: factor of mode i along this axis (or null)
  const T* fac_a;             // line factor fac_a[g % Na] * fac_b[g / Na] (or null)
  const T* fac_b;
  int Na;
  // cols passes: ncols adjacent columns (a multiple of 4) x nouter lines,
  // outer index o at in + o in_plane / out + o out_plane
  int ncols, nouter;
  long long in_plane, out_plane;
  int pitch;                  // shared-memory pitch of a column (elements), half_col_pitch
  int dir;                    // sign of the exponent (+1 or -1)
};
template <typename T> cudaError_t launch_half_pass(const HalfPass<T>& a, cudaStream_t s);
bool half_fft_size_ok(int nf);

// Double-float FFT of FP64 grids (fft_df.cu): 1D transforms of length n (a
// power of two <= 4096) over `rows` consecutive rows, twiddles tw[k] =
// exp(sign 2 pi i k / n), k < n/2, as float pairs (re hi, re lo, im hi,
// im lo); and the batched transpose of R x C planes of double2.
bool fft_df_size_ok(int n);
size_t fft_df_smem(int n);
cudaError_t launch_fft_df_rows(const double2* in, double2* out, int n, long long rows, const float4* tw,
                               cudaStream_t s);
cudaError_t launch_transpose_d2(const double2* in, double2* out, int R, int C, int batch, cudaStream_t s);
int half_fft_mp(int nf);
// Pitch of the column buffers of the strided passes for n values per column
// and Mp-point transforms (at least both, bank-conflict offset added).
template <typename T> int half_col_pitch(int n, int Mp);

template <typename T> int line_fft_cap();
template <typename T> int line_fft_p2_elems();
template <typename T> cudaError_t line_fft_prepare();
template <typename T> cudaError_t launch_line_fft(const LineArgs<T>& a, cudaStream_t s);

}  // namespace cfg
