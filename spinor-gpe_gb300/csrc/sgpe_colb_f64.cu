// Grouped (batched) column-pass kernels, complex128: explicit instantiation.
#define SGPE_INSTANTIATE
#include "sgpe_launch.cuh"

namespace sgpe {
template cudaError_t launch_col_grouped_s<double, 0>(const ColArgs<double>*, int, int, int, cudaStream_t);
}  // namespace sgpe
