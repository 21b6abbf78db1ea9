// Row-pass kernels, complex64: explicit instantiation.
#define SGPE_INSTANTIATE
#include "sgpe_launch.cuh"

namespace sgpe {
template cudaError_t launch_row<float>(const RowArgs<float>&, int, int, cudaStream_t);
}  // namespace sgpe
