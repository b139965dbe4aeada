// interp kernels for double plans in 3D (all kernel widths 2..16).
#include "spreadinterp.cuh"

namespace cfg {
template cudaError_t interp_dim<double, 3>(int, int, const SpreadArgs<double>&, cudaStream_t);
}  // namespace cfg
