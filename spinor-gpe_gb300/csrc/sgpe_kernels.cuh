// Split-step kernels for the pseudospin-1/2 GPE on sm_103a.
//
// Storage: each spinor component is an (Ny, Nx) row-major complex array (x
// contiguous).  Between kernels the state is kept in "mixed" form: natural
// (unshifted) kx along rows and real-space y along columns.  One Strang
// sub-step of the original propagator (spinor_gpe/pspinor/tensor_propagator.py:224-271)
// is two sweeps over the state:
//
//   column pass:  F_y -> psik *= K_prev -> sum|psik_c|^2 (populations)
//                 -> psik *= K_next -> sum|psik|^2 (norm) -> F_y^-1
//   row pass:     F_x^-1 -> psi *= lambda (renormalised real-space psi)
//                 -> interaction, coupling, potential, coupling, interaction
//                 -> F_x
//
// The k-space renormalisation of the original (``norm(psik, dv_k)``,
// tensor_propagator.py:271) is a uniform scale, so it is folded into the next
// real-space renormalisation: lambda is computed from the k-space sum of the
// column pass by Parseval, which is exactly the real-space atom number of the
// original's step 3 (tensor_propagator.py:244).  A column pass therefore
// joins the end of one sub-step (kinetic half step) and the start of the next.
//
// F denotes the unnormalised DFT; constant factors are absorbed by the
// renormalisation (see RowArgs::norm_num).
#pragma once
#include "sgpe_fft.cuh"

namespace sgpe {

// A complex operator field with broadcast strides: value(x, y) = p[x*sx + y*sy].
// sx = sy = 0 is a uniform value, (1, 0) an x-table, (0, 1) a y-table and
// (1, Nx) a full field.
template <typename R> struct Field {
  const Cx<R>* p;
  int sx, sy;
};
template <typename R> __device__ __forceinline__ Cx<R> fld(const Field<R>& f, int x, int y) {
  return __ldg(f.p + (x * f.sx + y * f.sy));
}

// Kinetic propagator exp(-i K_c t/2) = a_c(x, y) * b_c(x, y) in natural k order.
template <typename R> struct KinOp {
  Field<R> a[2], b[2];
};

// Real-space operators of one sub-step:
//  potential exp(-i V_c t) = pa_c * pb_c,
//  coupling  [[c, s conj(e)], [s e, c]] with c = cos(Omega t/4),
//            s = -i sin(Omega t/4), e = exp(i theta),
//  interaction exp(z E_c) with z = -i t/2.
template <typename R> struct RealOp {
  Field<R> pa[2], pb[2];
  Field<R> cc, cs, ce;
  R zr, zi;
};

enum RowMode { kRowStep = 0, kRowForward = 1, kRowInverse = 2 };

template <typename R> struct RowArgs {
  const Cx<R>* in[2];
  Cx<R>* out[2];
  const Cx<R>* tw;        // W_Nx table
  int mode;               // RowMode
  R scale;                // forward/inverse modes: constant output scale
  // step mode: renormalisation from the preceding column pass
  const double* part;     // [2 comps][ntile][u, w]
  int ntile;
  double norm_num;        // lambda^2 * sum|w|^2 = atom_num / (Nx Ny dv_r)
  R g_uu, g_dd, g_ud;
  int coupling;
  RealOp<R> op;
  double* pops;           // non-null: block 0 writes the populations of the state
                          // the preceding column pass started from
  double atom_num;
};

template <typename R> struct ColArgs {
  const Cx<R>* in[2];
  Cx<R>* out[2];
  const Cx<R>* tw;        // W_Ny table
  int nx;
  int fwd, inv;           // forward F_y first / inverse F_y^-1 last
  int in_shift, out_shift;  // centred (fftshift) order on input / output
  int has_kprev, has_knext;
  KinOp<R> kprev, knext;
  R scale;
  double* part;           // non-null: per block [u, w] sums
};

template <typename R> struct ScaleArgs {
  Cx<R>* d[2];
  long long n;            // elements per component
  const double* part;
  int ntile;
  double atom_num, dv;
  double* pops;
};

template <typename R> struct CopyArgs {
  const Cx<R>* in[2];
  Cx<R>* out[2];
  int nx, ny;
  int shift;              // 1: out = fftshift(in) in both axes (even sizes)
  R scale;
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sum of |v[m]|^2 over the E points of a thread: pairwise in the working
// precision, so the per-thread error stays at log2(E) roundings.
template <int E, class C> __device__ __forceinline__ double thread_norm2(const C (&v)[E]) {
  using R = decltype(C::x);
  R s[E];
#pragma unroll
  for (int m = 0; m < E; ++m) s[m] = cabs2(v[m]);
#pragma unroll
  for (int w = 1; w < E; w <<= 1)
#pragma unroll
    for (int m = 0; m + w < E; m += 2 * w) s[m] += s[m + w];
  return double(s[0]);
}

__device__ __forceinline__ void sin_cos(float x, float* s, float* c) { sincosf(x, s, c); }
__device__ __forceinline__ void sin_cos(double x, double* s, double* c) { sincos(x, s, c); }
__device__ __forceinline__ float exp_r(float x) { return expf(x); }
__device__ __forceinline__ double exp_r(double x) { return exp(x); }

// exp(z * e) for the interaction operator (library expf/sincosf, not the
// reduced-accuracy intrinsics).
template <typename R> __device__ __forceinline__ Cx<R> cexp_z(R zr, R zi, R e) {
  using C = Cx<R>;
  if (zi == R(0)) return cmake<C>(exp_r(zr * e), R(0));
  R sn, cs;
  sin_cos(zi * e, &sn, &cs);
  if (zr == R(0)) return cmake<C>(cs, sn);
  const R g = exp_r(zr * e);
  return cmake<C>(g * cs, g * sn);
}

// ----------------------------------------------------------------- row pass
template <typename R, int N, int E, int ROWS>
__global__ void __launch_bounds__((N / E) * ROWS)
row_kernel(const RowArgs<R> a) {
  using C = Cx<R>;
  constexpr int T = N / E;
  constexpr int LS = N + N / E;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* sm = reinterpret_cast<C*>(smem_raw);
  __shared__ double s_lambda;

  const int tid = threadIdx.x;
  const int rho = tid / T;
  const int j = tid - rho * T;
  const int y = blockIdx.x * ROWS + rho;
  const long long row_off = (long long)y * N;

  C v[2][E];
#pragma unroll
  for (int m = 0; m < E; ++m) {
    v[0][m] = a.in[0][row_off + j + m * T];
    v[1][m] = a.in[1][row_off + j + m * T];
  }
  const LineSmem<C, E> smv{sm + rho * LS, ROWS * LS};

  if (a.mode == kRowStep) {
    if (tid < 32) {
      double su0 = 0.0, su1 = 0.0, sw = 0.0;
      for (int i = tid; i < 2 * a.ntile; i += 32) {
        const double u = a.part[2 * i], w = a.part[2 * i + 1];
        sw += w;
        if (i < a.ntile) su0 += u; else su1 += u;
      }
      sw = warp_sum(sw);
      if (tid == 0) s_lambda = sqrt(a.norm_num / sw);
      if (a.pops != nullptr && blockIdx.x == 0) {
        su0 = warp_sum(su0);
        su1 = warp_sum(su1);
        if (tid == 0) {
          a.pops[0] = a.atom_num * su0 / (su0 + su1);
          a.pops[1] = a.atom_num * su1 / (su0 + su1);
        }
      }
    }
    __syncthreads();
    const R lam = R(s_lambda);
#pragma unroll
    for (int m = 0; m < E; ++m) {
      v[0][m] = cscale(v[0][m], lam);
      v[1][m] = cscale(v[1][m], lam);
    }
    fft_lines<N, E, +1, 2>(v, j, smv, a.tw);

    const RealOp<R>& op = a.op;
#pragma unroll
    for (int m = 0; m < E; ++m) {
      const int x = j + m * T;
      C p0 = v[0][m], p1 = v[1][m];
      const R n0 = cabs2(p0), n1 = cabs2(p1);
      // interaction half step (tensor_propagator.py:247-250)
      const R e0 = fmadd(a.g_uu, n0, a.g_ud * n1);
      const R e1 = fmadd(a.g_dd, n1, a.g_ud * n0);
      const C i0 = cexp_z(op.zr, op.zi, e0);
      const C i1 = cexp_z(op.zr, op.zi, e1);
      p0 = cmul(p0, i0);
      p1 = cmul(p1, i1);
      C cc, s01, s10;
      if (a.coupling) {  // first coupling half step (:252-254)
        cc = fld(op.cc, x, y);
        const C s = fld(op.cs, x, y), e = fld(op.ce, x, y);
        s01 = cmulc(s, e);
        s10 = cmul(s, e);
        const C q0 = cadd(cmul(cc, p0), cmul(s01, p1));
        const C q1 = cadd(cmul(s10, p0), cmul(cc, p1));
        p0 = q0;
        p1 = q1;
      }
      // potential full step (:256)
      p0 = cmul(p0, cmul(fld(op.pa[0], x, y), fld(op.pb[0], x, y)));
      p1 = cmul(p1, cmul(fld(op.pa[1], x, y), fld(op.pb[1], x, y)));
      if (a.coupling) {  // second coupling half step (:258-260)
        const C q0 = cadd(cmul(cc, p0), cmul(s01, p1));
        const C q1 = cadd(cmul(s10, p0), cmul(cc, p1));
        p0 = q0;
        p1 = q1;
      }
      // second interaction half step with the same operator (:262-267)
      v[0][m] = cmul(p0, i0);
      v[1][m] = cmul(p1, i1);
    }
    fft_lines<N, E, -1, 2>(v, j, smv, a.tw);
  } else {
    if (a.mode == kRowForward) fft_lines<N, E, -1, 2>(v, j, smv, a.tw);
    else fft_lines<N, E, +1, 2>(v, j, smv, a.tw);
#pragma unroll
    for (int m = 0; m < E; ++m) {
      v[0][m] = cscale(v[0][m], a.scale);
      v[1][m] = cscale(v[1][m], a.scale);
    }
  }
#pragma unroll
  for (int m = 0; m < E; ++m) {
    a.out[0][row_off + j + m * T] = v[0][m];
    a.out[1][row_off + j + m * T] = v[1][m];
  }
}

// -------------------------------------------------------------- column pass
template <typename R, int N, int E, int COLS>
__global__ void __launch_bounds__((N / E) * COLS)
col_kernel(const ColArgs<R> a) {
  using C = Cx<R>;
  constexpr int T = N / E;
  constexpr int LS = N + N / E + 2;
  constexpr int NT = T * COLS;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* sm = reinterpret_cast<C*>(smem_raw);
  __shared__ double s_red[2][NT / 32 > 0 ? NT / 32 : 1];

  const int tid = threadIdx.x;
  const int c = tid % COLS;
  const int j = tid / COLS;
  const int comp = blockIdx.y;
  const int nx = a.nx;
  const int x = blockIdx.x * COLS + c;
  const int half = nx / 2;
  const int xin = a.in_shift ? (x + half) % nx : x;
  const int xout = a.out_shift ? (x + half) % nx : x;
  const C* __restrict__ in = a.in[comp];
  C* out = a.out[comp];

  C v[1][E];
#pragma unroll
  for (int m = 0; m < E; ++m) {
    const int row = j + (a.in_shift ? (m + E / 2) % E : m) * T;
    v[0][m] = in[(long long)row * nx + xin];
  }
  const LineSmem<C, E> smv{sm + c * LS, 0};
  if (a.fwd) fft_lines<N, E, -1, 1>(v, j, smv, a.tw);

  double su = 0.0, sw = 0.0;
  if (a.has_kprev) {
    const Field<R>& ka = a.kprev.a[comp];
    const Field<R>& kb = a.kprev.b[comp];
#pragma unroll
    for (int m = 0; m < E; ++m) {
      const int ky = j + m * T;
      v[0][m] = cmul(v[0][m], cmul(fld(ka, x, ky), fld(kb, x, ky)));
    }
  }
  if (a.part != nullptr) su = thread_norm2(v[0]);
  if (a.has_knext) {
    const Field<R>& ka = a.knext.a[comp];
    const Field<R>& kb = a.knext.b[comp];
#pragma unroll
    for (int m = 0; m < E; ++m) {
      const int ky = j + m * T;
      v[0][m] = cmul(v[0][m], cmul(fld(ka, x, ky), fld(kb, x, ky)));
    }
  }
  if (a.part != nullptr) sw = thread_norm2(v[0]);
  if (a.inv) fft_lines<N, E, +1, 1>(v, j, smv, a.tw);
  if (a.scale != R(1)) {
#pragma unroll
    for (int m = 0; m < E; ++m) v[0][m] = cscale(v[0][m], a.scale);
  }
#pragma unroll
  for (int m = 0; m < E; ++m) {
    const int row = j + (a.out_shift ? (m + E / 2) % E : m) * T;
    out[(long long)row * nx + xout] = v[0][m];
  }
  if (a.part != nullptr) {
    su = warp_sum(su);
    sw = warp_sum(sw);
    const int warp = tid >> 5, lane = tid & 31;
    if (lane == 0) {
      s_red[0][warp] = su;
      s_red[1][warp] = sw;
    }
    __syncthreads();
    if (tid == 0) {
      double tu = 0.0, tw = 0.0;
      for (int w = 0; w < NT / 32; ++w) {
        tu += s_red[0][w];
        tw += s_red[1][w];
      }
      double* dst = a.part + 2 * ((long long)comp * gridDim.x + blockIdx.x);
      dst[0] = tu;
      dst[1] = tw;
    }
  }
}

// Final k-space renormalisation of a materialised psik
// (tensor_propagator.py:271) and, optionally, its populations
// (tensor_tools.py:466-484).
template <typename R>
__global__ void __launch_bounds__(256) scale_kernel(const ScaleArgs<R> a) {
  using C = Cx<R>;
  __shared__ double s_alpha;
  if (threadIdx.x < 32) {
    double s0 = 0.0, s1 = 0.0;
    for (int i = threadIdx.x; i < 2 * a.ntile; i += 32) {
      if (i < a.ntile) s0 += a.part[2 * i]; else s1 += a.part[2 * i];
    }
    s0 = warp_sum(s0);
    s1 = warp_sum(s1);
    if (threadIdx.x == 0) {
      s_alpha = sqrt(a.atom_num / (a.dv * (s0 + s1)));
      if (a.pops != nullptr && blockIdx.x == 0) {
        a.pops[0] = a.atom_num * s0 / (s0 + s1);
        a.pops[1] = a.atom_num * s1 / (s0 + s1);
      }
    }
  }
  __syncthreads();
  const R alpha = R(s_alpha);
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += stride) {
    a.d[0][i] = cscale(a.d[0][i], alpha);
    a.d[1][i] = cscale(a.d[1][i], alpha);
  }
}

// out = scale * (shift ? fftshift(in) : in), both components.
template <typename R>
__global__ void __launch_bounds__(256) copy_kernel(const CopyArgs<R> a) {
  const long long n = (long long)a.nx * a.ny;
  const long long stride = (long long)gridDim.x * blockDim.x;
  const int sx = a.shift ? a.nx / 2 : 0, sy = a.shift ? a.ny / 2 : 0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int y = int(i / a.nx), x = int(i - (long long)y * a.nx);
    const long long src = (long long)((y + sy) % a.ny) * a.nx + (x + sx) % a.nx;
    a.out[0][i] = cscale(a.in[0][src], a.scale);
    a.out[1][i] = cscale(a.in[1][src], a.scale);
  }
}

}  // namespace sgpe
