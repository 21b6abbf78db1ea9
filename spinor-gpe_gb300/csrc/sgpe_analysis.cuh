// Post-analysis of a final spinor on the device: the derived fields of the
// original's PropResult (spinor_gpe/pspinor/prop_result.py:76-78) and its
// phase-separation measure (prop_result.py:84-88).
//
//   dens_c  = |psi_c|^2,  densk_c = |psik_c|^2                 (working precision)
//   phase_c = angle(psi_c), set to 0 where dens_c < 1e-6 max(dens_c)
//             (tensor_tools.py:514-539, without unwrapping)
//   sums    = [sum n0 n1, sum n0^2, sum n1^2, max n0, max n1]   (FP64)
//   separation = 1 - sum n0 n1 / sqrt(sum n0^2 sum n1^2)
//
// Densities are formed as re^2 + im^2 (the original takes |z| first and then
// squares it, which can differ in the last bit); sums are FP64 over
// FP64-widened densities, block partials reduced in a fixed order.
#pragma once
#include "sgpe_energy.cuh"

namespace sgpe {

constexpr int kAnalysisBlocks = 304;
constexpr int kAnalysisSums = 5;

template <typename R> struct AnalysisArgs {
  const Cx<R>* psi[2];
  const Cx<R>* psik[2];
  R* dens[2];
  R* densk[2];
  R* phase[2];
  long long n;
  double* part;   // [kAnalysisBlocks][kAnalysisSums]
  double* sums;   // [kAnalysisSums]
};

__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// densities and per-block sums / maxima
template <typename R>
__global__ void __launch_bounds__(256) analysis_dens_kernel(const AnalysisArgs<R> a) {
  double s01 = 0.0, s00 = 0.0, s11 = 0.0, m0 = 0.0, m1 = 0.0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += stride) {
    const R n0 = cabs2(a.psi[0][i]), n1 = cabs2(a.psi[1][i]);
    a.dens[0][i] = n0;
    a.dens[1][i] = n1;
    a.densk[0][i] = cabs2(a.psik[0][i]);
    a.densk[1][i] = cabs2(a.psik[1][i]);
    const double d0 = double(n0), d1 = double(n1);
    s01 += d0 * d1;
    s00 += d0 * d0;
    s11 += d1 * d1;
    m0 = fmax(m0, d0);
    m1 = fmax(m1, d1);
  }
  __shared__ double sh[kAnalysisSums][8];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  s01 = warp_sum(s01);
  s00 = warp_sum(s00);
  s11 = warp_sum(s11);
  m0 = warp_max(m0);
  m1 = warp_max(m1);
  if (lane == 0) {
    sh[0][warp] = s01;
    sh[1][warp] = s00;
    sh[2][warp] = s11;
    sh[3][warp] = m0;
    sh[4][warp] = m1;
  }
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    double v[kAnalysisSums];
#pragma unroll
    for (int k = 0; k < kAnalysisSums; ++k) v[k] = lane < nw ? sh[k][lane] : 0.0;
#pragma unroll
    for (int k = 0; k < 3; ++k) v[k] = warp_sum(v[k]);
    v[3] = warp_max(v[3]);
    v[4] = warp_max(v[4]);
    if (lane == 0)
#pragma unroll
      for (int k = 0; k < kAnalysisSums; ++k) a.part[blockIdx.x * kAnalysisSums + k] = v[k];
  }
}

// fixed-order reduction of the block partials (one warp)
__global__ void __launch_bounds__(32) analysis_finalize_kernel(const double* part, int nblk, double* sums) {
  const int lane = threadIdx.x;
  double v[kAnalysisSums] = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (int b = lane; b < nblk; b += 32) {
#pragma unroll
    for (int k = 0; k < 3; ++k) v[k] += part[b * kAnalysisSums + k];
    v[3] = fmax(v[3], part[b * kAnalysisSums + 3]);
    v[4] = fmax(v[4], part[b * kAnalysisSums + 4]);
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) v[k] = warp_sum(v[k]);
  v[3] = warp_max(v[3]);
  v[4] = warp_max(v[4]);
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < kAnalysisSums; ++k) sums[k] = v[k];
}

__device__ __forceinline__ float angle_of(float2 z) { return atan2f(z.y, z.x); }
__device__ __forceinline__ double angle_of(double2 z) { return atan2(z.y, z.x); }

// phases with the low-density mask (needs the maxima of the first kernel)
template <typename R>
__global__ void __launch_bounds__(256) analysis_phase_kernel(const AnalysisArgs<R> a) {
  const R thr0 = R(a.sums[3]) * R(1e-6), thr1 = R(a.sums[4]) * R(1e-6);
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += stride) {
    a.phase[0][i] = a.dens[0][i] < thr0 ? R(0) : angle_of(a.psi[0][i]);
    a.phase[1][i] = a.dens[1][i] < thr1 ? R(0) : angle_of(a.psi[1][i]);
  }
}

}  // namespace sgpe
