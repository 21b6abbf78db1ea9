// Double-float row-pass kernels, generic operator fields, sides 32-512: explicit instantiation.
#define SGPE_DF_KERNELS
#define SGPE_INSTANTIATE
#include "sgpe_launch.cuh"

namespace sgpe {
template cudaError_t launch_df_row_n<false, 32>(const RowArgs<DF>&, int, cudaStream_t);
template cudaError_t launch_df_row_n<false, 64>(const RowArgs<DF>&, int, cudaStream_t);
template cudaError_t launch_df_row_n<false, 128>(const RowArgs<DF>&, int, cudaStream_t);
template cudaError_t launch_df_row_n<false, 256>(const RowArgs<DF>&, int, cudaStream_t);
template cudaError_t launch_df_row_n<false, 512>(const RowArgs<DF>&, int, cudaStream_t);
}  // namespace sgpe
