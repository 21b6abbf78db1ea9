// Initial-state set-up on the device: the O(Nx Ny) parts of the original's
// PSpinor set-up (spinor_gpe/pspinor/pspinor.py:248-281, 503-545, 680-745)
// for a separable trap V(x, y) = vx(x) + vy(y).
//
// sgpe_setup_spinor: Thomas-Fermi spinor with optional phase noise and
// renormalisation (ttools.norm),
//   psi_c = sqrt(max(mu - V, 0)) * amp_c * exp(i phi_c),
//   phi_c ~ U(-noise, noise) per point (a counter-based hash of (seed,
//   component, point), independent of the launch shape),
//   then, if atom_num > 0, psi <- psi * sqrt(atom_num / (dv_r sum |psi|^2)).
// sgpe_imprint_vortices: psi_c *= prod_j f(r_j / heal_c) exp(i w_j atan2(dy, dx)),
//   f(g) = g / sqrt(g^2 + 1) (seed_vortices, pspinor.py:680-745).
// sgpe_fourier_split_x: out = f_plus S(+s) in + f_minus S(-s) in, with
//   S(s) the multiplication by exp(-2 pi i s fftfreq(nx)[ix]) along x (the
//   scipy.ndimage.fourier_shift of shift_momentum, pspinor.py:503-545).
// Everything is evaluated in FP64 and rounded once to the working precision;
// sums are FP64 in a fixed order.
#include <cmath>
#include <string>

#include "sgpe_kernels.cuh"
#include "spinor_gb300.h"

namespace sgpe_detail {
int set_error(int code, const std::string& msg);  // sgpe_api.cu
}

namespace {

using namespace sgpe;

constexpr int kSetupBlocks = 304;

struct SetupArgs {
  int nx, ny;
  const double* vx;
  const double* vy;
  double mu;
  double amp[2][2];     // [comp][re, im]
  double noise;
  unsigned long long seed;
  double* part;         // [kSetupBlocks]
};

// splitmix64 finaliser: a well-mixed 64-bit hash of a counter
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__device__ __forceinline__ double uniform_pm1(unsigned long long seed, int comp, long long i) {
  const unsigned long long h = mix64(seed ^ mix64(((unsigned long long)comp << 62) ^ (unsigned long long)i));
  return double(h >> 11) * (2.0 / 9007199254740992.0) - 1.0;  // [-1, 1)
}

template <typename R>
__global__ void __launch_bounds__(256) tf_kernel(const SetupArgs a, Cx<R>* psi0, Cx<R>* psi1) {
  const long long n = (long long)a.nx * a.ny;
  double acc = 0.0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int ix = int(i % a.nx), iy = int(i / a.nx);
    const double prof = sqrt(fmax(a.mu - (a.vx[ix] + a.vy[iy]), 0.0));
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      double re = prof * a.amp[c][0], im = prof * a.amp[c][1];
      if (a.noise != 0.0) {
        double s, co;
        sincos(a.noise * uniform_pm1(a.seed, c, i), &s, &co);
        const double r2 = re * co - im * s, i2 = re * s + im * co;
        re = r2;
        im = i2;
      }
      const Cx<R> v = cmake<Cx<R>>(R(re), R(im));
      (c ? psi1 : psi0)[i] = v;
      acc += double(v.x) * double(v.x) + double(v.y) * double(v.y);
    }
  }
  acc = warp_sum(acc);
  __shared__ double sh[8];
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    double t = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
    t = warp_sum(t);
    if (threadIdx.x == 0) a.part[blockIdx.x] = t;
  }
}

struct VortexArgs {
  int nx, ny;
  const double* x;
  const double* y;
  const double* vort;   // [nv][4]: component (0 or 1), x, y, winding
  int nv;
  double heal[2];
};

template <typename R>
__global__ void __launch_bounds__(256) vortex_kernel(const VortexArgs a, Cx<R>* psi0, Cx<R>* psi1) {
  const long long n = (long long)a.nx * a.ny;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int ix = int(i % a.nx), iy = int(i / a.nx);
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      Cx<R>* p = c ? psi1 : psi0;
      double re = double(p[i].x), im = double(p[i].y);
      for (int j = 0; j < a.nv; ++j) {
        const double* v = a.vort + 4 * j;
        if (int(v[0]) != c) continue;
        const double dx = a.x[ix] - v[1], dy = a.y[iy] - v[2];
        const double g = sqrt(dx * dx + dy * dy) / a.heal[c];
        const double f = g / sqrt(g * g + 1.0);
        double s, co;
        sincos(v[3] * atan2(dy, dx), &s, &co);
        const double r2 = f * (re * co - im * s), i2 = f * (re * s + im * co);
        re = r2;
        im = i2;
      }
      p[i] = cmake<Cx<R>>(R(re), R(im));
    }
  }
}

// psi *= sqrt(atom_num / (dv * sum)), the sum of the partials in a fixed order
template <typename R>
__global__ void __launch_bounds__(256) renorm_kernel(const double* part, int nblk, double atom_num, double dv,
                                                     long long n, Cx<R>* psi0, Cx<R>* psi1) {
  __shared__ double s_scale;
  if (threadIdx.x < 32) {
    double t = 0.0;
    for (int b = threadIdx.x; b < nblk; b += 32) t += part[b];
    t = warp_sum(t);
    if (threadIdx.x == 0) s_scale = sqrt(atom_num / (dv * t));
  }
  __syncthreads();
  const R k = R(s_scale);
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    psi0[i] = cscale(psi0[i], k);
    psi1[i] = cscale(psi1[i], k);
  }
}

template <typename R>
__global__ void __launch_bounds__(256) fourier_split_kernel(int nx, long long n, double shift, double fp, double fm,
                                                            const Cx<R>* in, Cx<R>* out) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int ix = int(i % nx);
    const double f = (ix < (nx + 1) / 2 ? double(ix) : double(ix - nx)) / double(nx);  // fftfreq
    double s, co;
    sincospi(-2.0 * shift * f, &s, &co);  // S(+s) = co + i s, S(-s) = co - i s
    const double vr = double(in[i].x), vi = double(in[i].y);
    const double pr = vr * co - vi * s, pi = vr * s + vi * co;
    const double mr = vr * co + vi * s, mi = vi * co - vr * s;
    out[i] = cmake<Cx<R>>(R(fp * pr + fm * mr), R(fp * pi + fm * mi));
  }
}

}  // namespace

extern "C" int sgpe_setup_spinor(int dtype_bits, int ny, int nx, const double* vx, const double* vy, double mu,
                                 const double* amp, double noise, unsigned long long seed, double atom_num,
                                 double dv_r, double* scratch, void* psi0, void* psi1, void* stream) {
  if (!vx || !vy || !amp || !scratch || !psi0 || !psi1)
    return sgpe_detail::set_error(SGPE_ERR_ARG, "setup_spinor: null pointer");
  if (nx < 1 || ny < 1 || !(dv_r > 0))
    return sgpe_detail::set_error(SGPE_ERR_ARG, "setup_spinor: bad sizes or volume element");
  if (dtype_bits != 64 && dtype_bits != 128)
    return sgpe_detail::set_error(SGPE_ERR_ARG, "setup_spinor: dtype_bits must be 64 or 128");
  SetupArgs a{};
  a.nx = nx;
  a.ny = ny;
  a.vx = vx;
  a.vy = vy;
  a.mu = mu;
  for (int c = 0; c < 2; ++c) {
    a.amp[c][0] = amp[2 * c];
    a.amp[c][1] = amp[2 * c + 1];
  }
  a.noise = noise;
  a.seed = seed;
  a.part = scratch;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const long long n = (long long)nx * ny;
  if (dtype_bits == 64) {
    tf_kernel<float><<<kSetupBlocks, 256, 0, s>>>(a, static_cast<float2*>(psi0), static_cast<float2*>(psi1));
    if (atom_num > 0)
      renorm_kernel<float><<<kSetupBlocks, 256, 0, s>>>(scratch, kSetupBlocks, atom_num, dv_r, n,
                                                        static_cast<float2*>(psi0), static_cast<float2*>(psi1));
  } else {
    tf_kernel<double><<<kSetupBlocks, 256, 0, s>>>(a, static_cast<double2*>(psi0), static_cast<double2*>(psi1));
    if (atom_num > 0)
      renorm_kernel<double><<<kSetupBlocks, 256, 0, s>>>(scratch, kSetupBlocks, atom_num, dv_r, n,
                                                         static_cast<double2*>(psi0), static_cast<double2*>(psi1));
  }
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return sgpe_detail::set_error(SGPE_ERR_CUDA, std::string("setup_spinor: ") + cudaGetErrorString(e));
  return SGPE_OK;
}

extern "C" int sgpe_imprint_vortices(int dtype_bits, int ny, int nx, const double* x, const double* y,
                                     const double* vort, int n_vort, const double* heal, void* psi0, void* psi1,
                                     void* stream) {
  if (!x || !y || !heal || !psi0 || !psi1 || (n_vort > 0 && !vort) || n_vort < 0 || nx < 1 || ny < 1)
    return sgpe_detail::set_error(SGPE_ERR_ARG, "imprint_vortices: bad arguments");
  if (dtype_bits != 64 && dtype_bits != 128)
    return sgpe_detail::set_error(SGPE_ERR_ARG, "imprint_vortices: dtype_bits must be 64 or 128");
  VortexArgs a{};
  a.nx = nx;
  a.ny = ny;
  a.x = x;
  a.y = y;
  a.vort = vort;
  a.nv = n_vort;
  a.heal[0] = heal[0];
  a.heal[1] = heal[1];
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (dtype_bits == 64)
    vortex_kernel<float><<<kSetupBlocks, 256, 0, s>>>(a, static_cast<float2*>(psi0), static_cast<float2*>(psi1));
  else
    vortex_kernel<double><<<kSetupBlocks, 256, 0, s>>>(a, static_cast<double2*>(psi0), static_cast<double2*>(psi1));
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return sgpe_detail::set_error(SGPE_ERR_CUDA, std::string("imprint_vortices: ") + cudaGetErrorString(e));
  return SGPE_OK;
}

extern "C" int sgpe_fourier_split_x(int dtype_bits, int ny, int nx, double shift, double f_plus, double f_minus,
                                    const void* in, void* out, void* stream) {
  if (!in || !out || nx < 1 || ny < 1) return sgpe_detail::set_error(SGPE_ERR_ARG, "fourier_split_x: bad arguments");
  if (dtype_bits != 64 && dtype_bits != 128)
    return sgpe_detail::set_error(SGPE_ERR_ARG, "fourier_split_x: dtype_bits must be 64 or 128");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const long long n = (long long)nx * ny;
  if (dtype_bits == 64)
    fourier_split_kernel<float><<<kSetupBlocks, 256, 0, s>>>(nx, n, shift, f_plus, f_minus,
                                                             static_cast<const float2*>(in), static_cast<float2*>(out));
  else
    fourier_split_kernel<double><<<kSetupBlocks, 256, 0, s>>>(nx, n, shift, f_plus, f_minus,
                                                              static_cast<const double2*>(in), static_cast<double2*>(out));
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return sgpe_detail::set_error(SGPE_ERR_CUDA, std::string("fourier_split_x: ") + cudaGetErrorString(e));
  return SGPE_OK;
}
