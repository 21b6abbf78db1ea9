// Double-float column-pass kernels, sides 1024-4096 and 3 * 2^k: explicit instantiation.
#define SGPE_DF_KERNELS
#define SGPE_INSTANTIATE
#include "sgpe_launch.cuh"

namespace sgpe {
template cudaError_t launch_df_col_n<1024>(const ColArgs<DF>&, int, cudaStream_t);
template cudaError_t launch_df_col_n<2048>(const ColArgs<DF>&, int, cudaStream_t);
template cudaError_t launch_df_col_n<4096>(const ColArgs<DF>&, int, cudaStream_t);
template cudaError_t launch_df_col_n<192>(const ColArgs<DF>&, int, cudaStream_t);
template cudaError_t launch_df_col_n<384>(const ColArgs<DF>&, int, cudaStream_t);
template cudaError_t launch_df_col_n<768>(const ColArgs<DF>&, int, cudaStream_t);
}  // namespace sgpe
