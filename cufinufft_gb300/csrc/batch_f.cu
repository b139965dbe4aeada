// Multi-plan spread/interp kernels of float batches.
#include "batch.cuh"

namespace cfg {

template <typename T>
cudaError_t batch_spreadinterp(Batch<T>* b, const BatchGroup& g) {
  const int n = (int)b->plans.size();
  switch (b->dim) {
    case 1: return batch_spreadinterp_dim<T, 1>(b, n, g);
    case 2: return batch_spreadinterp_dim<T, 2>(b, n, g);
    default: return batch_spreadinterp_dim<T, 3>(b, n, g);
  }
}

template cudaError_t batch_spreadinterp<float>(Batch<float>*, const BatchGroup&);

}  // namespace cfg
