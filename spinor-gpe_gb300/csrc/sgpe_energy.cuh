// FP64 energy and chemical-potential reductions of a spinor.
//
// Replaces the energy expectation value of the original propagator
// (spinor_gpe/pspinor/tensor_propagator.py:273-324), which runs on the host
// with finite differences of the unwrapped phase.  Here the kinetic term is
// spectral, sum_k K_c(k) |psik_c(k)|^2 dv_k, and the other terms are grid
// sums of the real-space spinor psi = ifft_2d(psik):
//   E_pot = sum V_c n_c dv_r
//   E_int = sum (g_uu n0^2/2 + g_dd n1^2/2 + g_ud n0 n1) dv_r
//   E_cpl = sum 2 Re(conj(psi_0) h psi_1) dv_r   (h = upper off-diagonal of the
//           coupling Hamiltonian, (Omega/2) exp(-i theta))
//   mu    = (E_kin + E_pot + E_cpl + 2 E_int) / N
// Every element is widened to FP64 before it is multiplied or summed; block
// partials are reduced in a fixed order (deterministic).
#pragma once
#include "sgpe_kernels.cuh"

namespace sgpe {

template <typename R> struct EnergyArgs {
  const Cx<R>* a[2];      // psik (k pass) or psi (r pass)
  long long n;            // points per component
  int nx;
  Field<double> w[2], wb[2];  // k pass: K_c = w + wb; r pass: V_c = w + wb (real parts)
  Field<double> h;        // r pass: coupling field
  double g_uu, g_dd, g_ud;
  double* part;           // [gridDim.x][kEnergySums]
};

constexpr int kEnergySums = 6;   // k pass: [W|a|^2, |a|^2]; r pass: [V n, S1, S2, cpl, n]

__device__ __forceinline__ double fld64re(const Field<double>& f, int x, int y) {
  return __ldg(&f.p[x * f.sx + y * f.sy].x);
}

template <int NV> __device__ __forceinline__ void block_sums(double (&v)[NV], double* out) {
  __shared__ double s[NV][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    v[i] = warp_sum(v[i]);
    if (lane == 0) s[i][warp] = v[i];
  }
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      double t = lane < nw ? s[i][lane] : 0.0;
      t = warp_sum(t);
      if (lane == 0) out[i] = t;
    }
  }
}

// k-space pass: sum_c W_c |a_c|^2 and sum_c |a_c|^2
template <typename R>
__global__ void __launch_bounds__(256) energy_k_kernel(const EnergyArgs<R> e) {
  double acc[2] = {0.0, 0.0};
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < e.n; i += stride) {
    const int y = int(i / e.nx), x = int(i - (long long)y * e.nx);
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      const Cx<R> v = e.a[c][i];
      const double m = double(v.x) * double(v.x) + double(v.y) * double(v.y);
      acc[0] += (fld64re(e.w[c], x, y) + fld64re(e.wb[c], x, y)) * m;
      acc[1] += m;
    }
  }
  block_sums<2>(acc, e.part + (long long)blockIdx.x * kEnergySums);
}

// real-space pass: potential, interaction (S1 = g_uu n0^2 + g_dd n1^2,
// S2 = g_ud n0 n1), coupling and atom-number sums
template <typename R>
__global__ void __launch_bounds__(256) energy_r_kernel(const EnergyArgs<R> e) {
  double acc[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < e.n; i += stride) {
    const int y = int(i / e.nx), x = int(i - (long long)y * e.nx);
    const Cx<R> p0 = e.a[0][i], p1 = e.a[1][i];
    const double r0 = p0.x, i0 = p0.y, r1 = p1.x, i1 = p1.y;
    const double n0 = r0 * r0 + i0 * i0, n1 = r1 * r1 + i1 * i1;
    acc[0] += (fld64re(e.w[0], x, y) + fld64re(e.wb[0], x, y)) * n0 +
              (fld64re(e.w[1], x, y) + fld64re(e.wb[1], x, y)) * n1;
    acc[1] += e.g_uu * n0 * n0 + e.g_dd * n1 * n1;
    acc[2] += e.g_ud * n0 * n1;
    const double2 h = __ldg(&e.h.p[x * e.h.sx + y * e.h.sy]);
    // conj(p0) * p1 = (r0 r1 + i0 i1) + i (r0 i1 - i0 r1); Re(h * that)
    const double cr = r0 * r1 + i0 * i1, ci = r0 * i1 - i0 * r1;
    acc[3] += 2.0 * (h.x * cr - h.y * ci);
    acc[4] += n0 + n1;
  }
  block_sums<5>(acc, e.part + (long long)blockIdx.x * kEnergySums);
}

// One block: fixed-order sums of the partials of both passes, then
//   out = [E_kin, E_pot, E_int, E_cpl, E_total, mu, N_k, N_r, S1 dv_r, S2 dv_r]
__global__ void __launch_bounds__(32) energy_finalize_kernel(const double* kpart, const double* rpart, int nblk,
                                                             double dv_k, double dv_r, double* out) {
  const int lane = threadIdx.x;
  double k[2] = {0.0, 0.0}, r[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (int b = lane; b < nblk; b += 32) {
#pragma unroll
    for (int i = 0; i < 2; ++i) k[i] += kpart[b * kEnergySums + i];
#pragma unroll
    for (int i = 0; i < 5; ++i) r[i] += rpart[b * kEnergySums + i];
  }
#pragma unroll
  for (int i = 0; i < 2; ++i) k[i] = warp_sum(k[i]);
#pragma unroll
  for (int i = 0; i < 5; ++i) r[i] = warp_sum(r[i]);
  if (lane == 0) {
    const double e_kin = k[0] * dv_k, n_k = k[1] * dv_k;
    const double e_pot = r[0] * dv_r, s1 = r[1] * dv_r, s2 = r[2] * dv_r;
    const double e_int = 0.5 * s1 + s2, e_cpl = r[3] * dv_r, n_r = r[4] * dv_r;
    out[0] = e_kin;
    out[1] = e_pot;
    out[2] = e_int;
    out[3] = e_cpl;
    out[4] = e_kin + e_pot + e_int + e_cpl;
    out[5] = (e_kin + e_pot + e_cpl + 2.0 * e_int) / n_r;
    out[6] = n_k;
    out[7] = n_r;
    out[8] = s1;
    out[9] = s2;
  }
}

}  // namespace sgpe
