// Kernel shapes 1 and 2 of every pass, complex128: explicit instantiation
// (shape 0 is instantiated with the default kernels).
#define SGPE_INSTANTIATE
#include "sgpe_launch.cuh"

namespace sgpe {
#define SGPE_SHAPE_INSTANCES(S)                                                                          \
  template cudaError_t launch_row_ops_s<double, true, S>(const RowArgs<double>&, int, int, cudaStream_t);     \
  template cudaError_t launch_row_ops_s<double, false, S>(const RowArgs<double>&, int, int, cudaStream_t);    \
  template cudaError_t launch_col_s<double, S>(const ColArgs<double>&, int, cudaStream_t);                    \
  template cudaError_t launch_row_grouped_s<double, S>(const RowArgs<double>*, int, int, int, cudaStream_t);  \
  template cudaError_t launch_col_grouped_s<double, S>(const ColArgs<double>*, int, int, int, cudaStream_t);
SGPE_SHAPE_INSTANCES(1)
SGPE_SHAPE_INSTANCES(2)
#undef SGPE_SHAPE_INSTANCES
}  // namespace sgpe
