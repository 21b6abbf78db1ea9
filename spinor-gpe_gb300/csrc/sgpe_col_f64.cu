// Column-pass kernels, complex128: explicit instantiation.
#define SGPE_INSTANTIATE
#include "sgpe_launch.cuh"

namespace sgpe {
template cudaError_t launch_col_s<double, 0>(const ColArgs<double>&, int, cudaStream_t);
}  // namespace sgpe
