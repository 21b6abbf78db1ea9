// Grouped (batched) row-pass kernels, complex64: explicit instantiation.
#define SGPE_INSTANTIATE
#include "sgpe_launch.cuh"

namespace sgpe {
template cudaError_t launch_row_grouped_s<float, 0>(const RowArgs<float>*, int, int, int, cudaStream_t);
}  // namespace sgpe
