// Double-float pass launchers (size dispatch): explicit instantiation.  The
// kernels of each size are instantiated in sgpe_df_k*.cu.
#define SGPE_INSTANTIATE
#include "sgpe_launch.cuh"

namespace sgpe {
template cudaError_t launch_row_ops_s<DF, true, 0>(const RowArgs<DF>&, int, int, cudaStream_t);
template cudaError_t launch_row_ops_s<DF, false, 0>(const RowArgs<DF>&, int, int, cudaStream_t);
template cudaError_t launch_col_s<DF, 0>(const ColArgs<DF>&, int, cudaStream_t);
}  // namespace sgpe
