// interp kernels for float plans in 1D (all kernel widths 2..16).
#include "spreadinterp.cuh"

namespace cfg {
template cudaError_t interp_dim<float, 1>(int, int, const SpreadArgs<float>&, cudaStream_t);
}  // namespace cfg
