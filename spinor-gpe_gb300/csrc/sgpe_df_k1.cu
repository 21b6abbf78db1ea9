// Double-float row-pass kernels, separable operators, sides 32-512: explicit instantiation.
#define SGPE_DF_KERNELS
#define SGPE_INSTANTIATE
#include "sgpe_launch.cuh"

namespace sgpe {
template cudaError_t launch_df_row_n<true, 32>(const RowArgs<DF>&, int, cudaStream_t);
template cudaError_t launch_df_row_n<true, 64>(const RowArgs<DF>&, int, cudaStream_t);
template cudaError_t launch_df_row_n<true, 128>(const RowArgs<DF>&, int, cudaStream_t);
template cudaError_t launch_df_row_n<true, 256>(const RowArgs<DF>&, int, cudaStream_t);
template cudaError_t launch_df_row_n<true, 512>(const RowArgs<DF>&, int, cudaStream_t);
}  // namespace sgpe
