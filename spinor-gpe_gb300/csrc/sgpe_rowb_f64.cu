// Grouped (batched) row-pass kernels, complex128: explicit instantiation.
#define SGPE_INSTANTIATE
#include "sgpe_launch.cuh"

namespace sgpe {
template cudaError_t launch_row_grouped_s<double, 0>(const RowArgs<double>*, int, int, int, cudaStream_t);
}  // namespace sgpe
