// Double-float column-pass kernels, sides 32-512: explicit instantiation.
#define SGPE_DF_KERNELS
#define SGPE_INSTANTIATE
#include "sgpe_launch.cuh"

namespace sgpe {
template cudaError_t launch_df_col_n<32>(const ColArgs<DF>&, int, cudaStream_t);
template cudaError_t launch_df_col_n<64>(const ColArgs<DF>&, int, cudaStream_t);
template cudaError_t launch_df_col_n<128>(const ColArgs<DF>&, int, cudaStream_t);
template cudaError_t launch_df_col_n<256>(const ColArgs<DF>&, int, cudaStream_t);
template cudaError_t launch_df_col_n<512>(const ColArgs<DF>&, int, cudaStream_t);
}  // namespace sgpe
