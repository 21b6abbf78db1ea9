// Grouped (batched) row-pass kernels, complex64: explicit instantiation.
#define SGPE_INSTANTIATE
#include "sgpe_launch.cuh"

namespace sgpe {
template cudaError_t launch_row_grouped<float>(const RowArgs<float>*, int, int, int, cudaStream_t);
}  // namespace sgpe
