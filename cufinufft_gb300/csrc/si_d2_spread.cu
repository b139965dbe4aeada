// spread kernels for double plans in 2D (all kernel widths 2..16).
#include "spreadinterp.cuh"

namespace cfg {
template cudaError_t spread_dim<double, 2>(int, int, const SpreadArgs<double>&, cudaStream_t);
}  // namespace cfg
