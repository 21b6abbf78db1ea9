// Row-pass kernels, complex64, separable operators: explicit instantiation.
#define SGPE_INSTANTIATE
#include "sgpe_launch.cuh"

namespace sgpe {
template cudaError_t launch_row_ops_s<float, true, 0>(const RowArgs<float>&, int, int, cudaStream_t);
}  // namespace sgpe
