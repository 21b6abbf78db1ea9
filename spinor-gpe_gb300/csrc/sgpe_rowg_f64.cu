// Row-pass kernels, complex128, generic operator fields: explicit instantiation.
#define SGPE_INSTANTIATE
#include "sgpe_launch.cuh"

namespace sgpe {
template cudaError_t launch_row_ops_s<double, false, 0>(const RowArgs<double>&, int, int, cudaStream_t);
}  // namespace sgpe
