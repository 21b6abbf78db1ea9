// Row-pass kernels, complex64, generic operator fields: explicit instantiation.
#define SGPE_INSTANTIATE
#include "sgpe_launch.cuh"

namespace sgpe {
template cudaError_t launch_row_ops<float, false>(const RowArgs<float>&, int, int, cudaStream_t);
}  // namespace sgpe
