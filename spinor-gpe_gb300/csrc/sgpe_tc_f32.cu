// Tensor-core DFT16 variant of the pass kernels (complex64): instantiation.
#define SGPE_INSTANTIATE
#include "sgpe_launch.cuh"

namespace sgpe {
cudaError_t launch_row_tc(const RowArgs<float>& a, int nx, int ny, cudaStream_t s) {
  return dispatch_tc(nx, RowTcLauncher{&a, ny, s});
}
cudaError_t launch_col_tc(const ColArgs<float>& a, int ny, cudaStream_t s) {
  return dispatch_tc(ny, ColTcLauncher{&a, ny, s});
}
}  // namespace sgpe
