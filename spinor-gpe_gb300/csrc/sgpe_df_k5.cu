// Double-float row-pass kernels, generic operator fields, sides 1024-4096: explicit instantiation.
#define SGPE_DF_KERNELS
#define SGPE_INSTANTIATE
#include "sgpe_launch.cuh"

namespace sgpe {
template cudaError_t launch_df_row_n<false, 1024>(const RowArgs<DF>&, int, cudaStream_t);
template cudaError_t launch_df_row_n<false, 2048>(const RowArgs<DF>&, int, cudaStream_t);
template cudaError_t launch_df_row_n<false, 4096>(const RowArgs<DF>&, int, cudaStream_t);
}  // namespace sgpe
