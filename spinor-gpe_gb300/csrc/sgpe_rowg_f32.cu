// Row-pass kernels, complex64, generic operator fields: explicit instantiation.
#define SGPE_INSTANTIATE
#include "sgpe_launch.cuh"

namespace sgpe {
template cudaError_t launch_row_ops_s<float, false, 0>(const RowArgs<float>&, int, int, cudaStream_t);
}  // namespace sgpe
