// Kernel shapes 1 and 2 of every pass, complex64: explicit instantiation
// (shape 0 is instantiated with the default kernels).
#define SGPE_INSTANTIATE
#include "sgpe_launch.cuh"

namespace sgpe {
#define SGPE_SHAPE_INSTANCES(S)                                                                          \
  template cudaError_t launch_row_ops_s<float, true, S>(const RowArgs<float>&, int, int, cudaStream_t);     \
  template cudaError_t launch_row_ops_s<float, false, S>(const RowArgs<float>&, int, int, cudaStream_t);    \
  template cudaError_t launch_col_s<float, S>(const ColArgs<float>&, int, cudaStream_t);                    \
  template cudaError_t launch_row_grouped_s<float, S>(const RowArgs<float>*, int, int, int, cudaStream_t);  \
  template cudaError_t launch_col_grouped_s<float, S>(const ColArgs<float>*, int, int, int, cudaStream_t);
SGPE_SHAPE_INSTANCES(1)
SGPE_SHAPE_INSTANCES(2)
#undef SGPE_SHAPE_INSTANCES
}  // namespace sgpe
