// Grouped (batched) column-pass kernels, complex64: explicit instantiation.
#define SGPE_INSTANTIATE
#include "sgpe_launch.cuh"

namespace sgpe {
template cudaError_t launch_col_grouped_s<float, 0>(const ColArgs<float>*, int, int, int, cudaStream_t);
}  // namespace sgpe
