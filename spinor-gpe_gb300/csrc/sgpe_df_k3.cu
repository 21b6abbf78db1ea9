// Double-float row-pass kernels, separable operators, sides 3 * 2^k: explicit instantiation.
#define SGPE_DF_KERNELS
#define SGPE_INSTANTIATE
#include "sgpe_launch.cuh"

namespace sgpe {
template cudaError_t launch_df_row_n<true, 192>(const RowArgs<DF>&, int, cudaStream_t);
template cudaError_t launch_df_row_n<true, 384>(const RowArgs<DF>&, int, cudaStream_t);
template cudaError_t launch_df_row_n<true, 768>(const RowArgs<DF>&, int, cudaStream_t);
}  // namespace sgpe
