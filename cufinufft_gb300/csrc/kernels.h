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
  int* rank;               // [M] rank of the point inside its bin
  const int* start;        // [nbins+1] exclusive scan of count
};
template <typename T> cudaError_t launch_bin_count(const PlaceArgs<T>& a, cudaStream_t s);
template <typename T> cudaError_t launch_permute(const PlaceArgs<T>& a, cudaStream_t s);
template <typename T> cudaError_t launch_place_unsorted(const PlaceArgs<T>& a, cudaStream_t s);

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
};
template <typename T> cudaError_t launch_rebin_count(const RebinArgs<T>& a, cudaStream_t s);
template <typename T> cudaError_t launch_rebin_permute(const RebinArgs<T>& a, cudaStream_t s);

// Point counts over fixed feature bins (fb cells per axis) from the stored
// first taps; counts must be zeroed.
cudaError_t launch_feature_count(int dim, int M, const int* const i0[3], const int fb[3],
                                 const int nb[3], int* counts, cudaStream_t s);

// Exclusive scan of n ints: out[0..n] (out[n] = total).  mode 0 scans the
// values, mode 1 scans ceil(v / div).  tmp needs scan_tmp_ints(n) ints.
int scan_tmp_ints(int n);
cudaError_t launch_scan(const int* in, int* out, int n, int mode, int div, int* tmp,
                        cudaStream_t s);
// sub_to_bin[s] = the bin b with sub_start[b] <= s < sub_start[b+1].
cudaError_t launch_sub_to_bin(const int* sub_start, int nbins, int nsub, int* sub_to_bin,
                              cudaStream_t s);

// deconv.cu
struct FseriesNodes {
  double z[kMaxNQuad / 2];   // quadrature nodes on (0, ns/2)
  double f[kMaxNQuad / 2];   // (ns/2) w_n phi(z_n)
  int q;
};
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
cudaError_t launch_amplify(int dim, const int nf[3], const int N[3], cplx_t<T>* fw,
                           const cplx_t<T>* fk, const T* fac0, const T* fac1, const T* fac2,
                           int ntr, cudaStream_t s);

}  // namespace cfg
