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
// renormalisation (see ColArgs::norm_num).
#pragma once
#include "sgpe_fft.cuh"
#include "sgpe_tma.cuh"

// Row-pass lines through bulk asynchronous copies (TMA) for sides of at
// least SGPE_ROW_TMA_MIN_N: 1 stages the input lines in shared memory,
// 2 also writes the output lines from shared memory with bulk stores.
// Measured on GB300 (1024^2 complex64 row pass): loads alone no change,
// loads and stores 22.9 -> 21.8 us before the exchange addressing was
// folded, a tie (21.3 us) after; at 256^2-512^2 both were slower.
#ifndef SGPE_ROW_TMA
#define SGPE_ROW_TMA 2
#endif
// Row-pass exchanges synchronise each line's own warps (named barriers)
// instead of the whole block.  Off: measured on GB300 the 1024^2 row pass
// took 21.4 -> 25.5 us with it (the two component lines drift apart and the
// block-wide barrier of the point-wise step waits for the later one),
// 2048^2 63.8 -> 62.7 us.
#ifndef SGPE_ROW_LINE_BARRIERS
#define SGPE_ROW_LINE_BARRIERS 0
#endif
#ifndef SGPE_ROW_TMA_MIN_N
#define SGPE_ROW_TMA_MIN_N 1024
#endif
// Column-pass tiles (COLS columns x N rows) through 2-D tensor copies (TMA
// loads into shared memory on an mbarrier, TMA stores back) for column
// lengths of at least SGPE_COL_TMA_MIN_N, when the host passes tensor maps
// (in-place steady-state passes).  Off by default: measured on GB300 the
// column pass took 19.4 -> 20.3 us at 1024^2 and 62.6 -> 69.0 us at 2048^2
// with it (the block waits for its whole tile either way; one thread's
// copies replace the 16 strided loads per thread but not the wait).
#ifndef SGPE_COL_TMA
#define SGPE_COL_TMA 0
#endif
#ifndef SGPE_COL_TMA_MIN_N
#define SGPE_COL_TMA_MIN_N 512
#endif

// Unroll factor of the row kernel's point-wise loop (small: keeps the code
// within the instruction cache).
#ifndef SGPE_OPS_UNROLL
#define SGPE_OPS_UNROLL 4
#endif

namespace sgpe {

constexpr int kOpsUnroll = SGPE_OPS_UNROLL;
// the double-float point-wise loop is long enough without unrolling
template <typename R> __host__ __device__ constexpr int ops_unroll() { return is_df<R>::value ? 1 : kOpsUnroll; }

// Device error word codes (a kernel that gives up a bounded wait records one
// and carries on with plain loads).
enum { kErrNone = 0, kErrCopyTimeout = 1 };

// Programmatic dependent launch: the pass kernels are launched so that they
// may start while the previous kernel in the stream is finishing.  Before
// reading anything the previous kernel wrote, a kernel waits for that grid to
// complete (griddepcontrol.wait); once it has loaded its own inputs it lets
// the next kernel be scheduled (griddepcontrol.launch_dependents), which only
// moves that kernel's launch earlier -- its own wait still orders the data.
#ifndef SGPE_PDL
#define SGPE_PDL 1
#endif
__device__ __forceinline__ void wait_for_previous_grid() {
#if SGPE_PDL
  asm volatile("griddepcontrol.wait;" ::: "memory");
#endif
}
__device__ __forceinline__ void allow_next_grid() {
#if SGPE_PDL
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
#endif
}

// State loads and stores of the pass kernels.  With SGPE_STATE_CG the state
// bypasses L1 (cached in L2 only), leaving L1 to the operator and twiddle
// tables that every block re-reads.
#ifndef SGPE_STATE_CG
#define SGPE_STATE_CG 0
#endif
template <class C> __device__ __forceinline__ C ld_state(const C* p) {
#if SGPE_STATE_CG
  return __ldcg(p);
#else
  return *p;
#endif
}
template <class C> __device__ __forceinline__ void st_state(C* p, C v) {
#if SGPE_STATE_CG
  __stcg(p, v);
#else
  *p = v;
#endif
}

// A complex operator field with broadcast strides: value(x, y) = p[x*sx + y*sy].
// sx = sy = 0 is a uniform value, (1, 0) an x-table, (0, 1) a y-table and
// (1, Nx) a full field.
template <typename R> struct Field {
  const Cx<R>* p;
  int sx, sy;
};
template <typename R> __device__ __forceinline__ Cx<R> fld(const Field<R>& f, int x, int y) {
  return ldg(f.p + (x * f.sx + y * f.sy));
}

// Kinetic propagator exp(-i K_c t/2) = a_c(x, y) * b_c(x, y) in natural k order.
// sep: a_c is an x-table of Nx values and b_c a y-table of Ny values (unit
// strides), read with compile-time offsets.
template <typename R> struct KinOp {
  Field<R> a[2], b[2];
  int sep;
  int real;   // every factor has a zero imaginary part (imaginary time)
};

// Real-space operators of one sub-step:
//  potential exp(-i V_c t) = pa_c * pb_c,
//  coupling  [[c, s conj(e)], [s e, c]] with c = cos(Omega t/4),
//            s = -i sin(Omega t/4), e = exp(i theta),
//  interaction exp(z E_c) with z = -i t/2.
template <typename R> struct RealOp {
  Field<R> pa[2], pb[2];
  Field<R> cc, cs, ce;
  // off-diagonal coupling elements s conj(e) and s e, pre-multiplied in FP64
  // on the host when that keeps them 1-D tables (has_s01), else computed here
  Field<R> s01, s10;
  int has_s01;
  // sep: pa_c, s01, s10 are x-tables of Nx values, pb_c y-tables of Ny
  // values (unit strides), cc is uniform
  int sep;
  // zero imaginary parts (imaginary time): real multiplies give the same bits
  int real_pot, real_cc;
  R zr, zi;
  // sep: the separable row kernels apply coupling, potential and coupling
  // as one matrix per point, pb(y) A(x) with m[0..3] = A00, A01, A10, A11
  // x-tables of Nx values and mb the y-table of Ny values; diag: no
  // coupling, A = diag(m[0], m[3]) (m[1], m[2] unread); real_mb: mb has zero
  // imaginary parts
  int diag, real_mb;
  Field<R> m[4], mb;
};

// Field slots of RealOp in a fixed order (for the per-row hoisting below).
enum { kPa0 = 0, kPb0, kPa1, kPb1, kCc, kCs, kCe, kS01, kS10, kNumRealFields };

template <typename R> __device__ __forceinline__ const Field<R>& real_field(const RealOp<R>& op, int k) {
  switch (k) {
    case kPa0: return op.pa[0];
    case kPb0: return op.pb[0];
    case kPa1: return op.pa[1];
    case kPb1: return op.pb[1];
    case kCc: return op.cc;
    case kCs: return op.cs;
    case kCe: return op.ce;
    case kS01: return op.s01;
    default: return op.s10;
  }
}

// The real-space operator values along one row y.  Fields that do not vary
// along x (uniform values, y-tables) are loaded once per row into registers
// (the row pass runs its point-wise loop while the transform data sits in
// shared memory, so registers are free then); the others are read per point.
template <typename R> struct RowFields {
  const RealOp<R>* op;
  int y;
  unsigned row_const;
  Cx<R> h[kNumRealFields];
  __device__ __forceinline__ void init(const RealOp<R>& o, int yy) {
    op = &o;
    y = yy;
    row_const = 0;
#pragma unroll
    for (int k = 0; k < kNumRealFields; ++k) {
      const Field<R>& f = real_field(o, k);
      if (f.sx == 0) {
        row_const |= 1u << k;
        h[k] = fld(f, 0, y);
      } else {
        h[k] = Cx<R>{};
      }
    }
  }
  __device__ __forceinline__ Cx<R> at(int k, int x) const {
    return ((row_const >> k) & 1u) ? h[k] : fld(real_field(*op, k), x, y);
  }
};

enum RowMode { kRowStep = 0, kRowForward = 1, kRowInverse = 2 };

template <typename R> struct RowArgs {
  const Cx<R>* in[2];
  Cx<R>* out[2];
  const Cx<R>* tw;        // per-stage twiddle table of the x transform
  int mode;               // RowMode
  R scale;                // forward/inverse modes: constant output scale
  // step mode: renormalisation from the partial sums of the preceding
  // column pass, lambda = sqrt(norm_num / sum w)
  const R* part;          // [2 comps][ntile][u, w]
  int ntile;
  // non-null: the sums of those partials (sum u_0, sum u_1, sum w), formed
  // once by the last block of the column pass (ColArgs::fin); read instead
  // of summing the partials in every block
  const double* fin;
  double norm_num;        // atom_num / (Nx Ny dv_r)
  R g_uu, g_dd, g_ud;
  int coupling;
  RealOp<R> op;
  double* pops;           // non-null: block 0 writes the populations of the
                          // state the preceding column pass started from
  double atom_num;
  int tc;                 // launch the tensor-core DFT16 kernels (host side)
  const uint32_t* tcb;    // their B fragments (kTcBfragWords, device)
  int shape;              // kernel shape of the launch (host side)
  int* err;               // non-null: device error word (kErr* codes)
};

template <typename R> struct ColArgs {
  const Cx<R>* in[2];
  Cx<R>* out[2];
  const Cx<R>* tw;        // per-stage twiddle table of the y transform
  int nx;
  int fwd, inv;           // forward F_y first / inverse F_y^-1 last
  int in_shift, out_shift;  // centred (fftshift) order on input / output
  int nk;                 // kinetic tables applied after F_y: 0, 1 or 2
  KinOp<R> k1, k2;        // k1 first; u = sum|psik|^2 after k1, w after k2
                          // (w = u when nk < 2)
  R scale;
  R* part;                // non-null: per-block partial sums [comp][tile][u, w]
                          // in the working precision; the consumer of the
                          // pass sums them with (at least) FP64 accuracy
  // non-null (with part): the block that finishes last sums the partials
  // (sum_partials, the order every consumer uses) into fin[0..2] and resets
  // the arrival counter *count to zero for the next pass
  double* fin;
  unsigned* count;
  int tc;                 // launch the tensor-core DFT16 kernels (host side)
  const uint32_t* tcb;    // their B fragments (kTcBfragWords, device)
  int shape;              // kernel shape of the launch (host side)
  // non-null: two 2-D tensor maps (128 bytes each, device memory) of the
  // components, in == out, no shifts; box {2 COLS scalars, min(N, 256) rows}
  const void* tmap;
  int* err;               // non-null: device error word (kErr* codes)
};

template <typename R> struct ScaleArgs {
  Cx<R>* d[2];
  long long n;            // elements per component
  const R* part;          // partials of the column pass that wrote d
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

// Butterfly (pairwise) sum over a warp.
template <typename T> __device__ __forceinline__ T shfl_xor(T v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
template <typename T> __device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = v + shfl_xor(v, o);
  return v;
}

// Sums of the column-pass partials [2][ntile][u, w] by one warp, in a fixed
// order: (sum u_0, sum u_1, sum w) returned on every lane.
// FP64 partials are summed in FP64.
// The partials are read kPartialBatch at a time per lane (independent loads
// in flight together, one memory latency per batch instead of one per
// entry) and added in the same order as one at a time.
constexpr int kPartialBatch = 8;

__device__ __forceinline__ void sum_partials(const double* part, int ntile, int lane, double* u0, double* u1,
                                             double* w) {
  double su0 = 0.0, su1 = 0.0, sw = 0.0;
  const double2* p2 = reinterpret_cast<const double2*>(part);
  for (int i0 = lane; i0 < 2 * ntile; i0 += 32 * kPartialBatch) {
    double2 v[kPartialBatch];
#pragma unroll
    for (int k = 0; k < kPartialBatch; ++k) {
      const int i = i0 + 32 * k;
      v[k] = i < 2 * ntile ? p2[i] : make_double2(0.0, 0.0);
    }
#pragma unroll
    for (int k = 0; k < kPartialBatch; ++k) {
      const int i = i0 + 32 * k;
      if (i >= 2 * ntile) break;
      sw += v[k].y;
      if (i < ntile) su0 += v[k].x; else su1 += v[k].x;
    }
  }
  *u0 = warp_sum(su0);
  *u1 = warp_sum(su1);
  *w = warp_sum(sw);
}

// Double-float accumulator: the value is hi + lo with |lo| <= ulp(hi)/2, so
// sums of FP32 terms keep about 48 significant bits using FP32 arithmetic
// only (Knuth's TwoSum for each addition; Dekker's FastTwoSum to
// renormalise).  FP64 arithmetic runs at a small fraction of the FP32 rate on
// this GPU, which made the FP64 sum of the partials a serial bottleneck at
// the start of every row-pass block.
struct FloatFloat {
  float hi = 0.0f, lo = 0.0f;
  __device__ __forceinline__ void add(float x) {
    const float s = hi + x;
    const float bp = s - hi;
    const float err = (hi - (s - bp)) + (x - bp);
    hi = s;
    lo += err;
  }
  __device__ __forceinline__ void add(const FloatFloat& o) {
    const float s = hi + o.hi;
    const float bp = s - hi;
    float err = (hi - (s - bp)) + (o.hi - bp);
    err += lo + o.lo;
    hi = s + err;                 // FastTwoSum(s, err), |s| >= |err|
    lo = err - (hi - s);
  }
  __device__ __forceinline__ void warp_reduce() {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      FloatFloat t;
      t.hi = __shfl_xor_sync(0xffffffffu, hi, o);
      t.lo = __shfl_xor_sync(0xffffffffu, lo, o);
      add(t);
    }
  }
  __device__ __forceinline__ double value() const { return double(hi) + double(lo); }
};

// FP32 partials: double-float sums in FP32 arithmetic.  Every lane of the
// warp ends with the same bits (the butterfly adds the same pairs in the same
// order on all lanes up to commutation, and each step is commutative).
__device__ __forceinline__ void sum_partials(const float* part, int ntile, int lane, FloatFloat* u0,
                                             FloatFloat* u1, FloatFloat* w) {
  FloatFloat su0, su1, sw;
  const float2* p2 = reinterpret_cast<const float2*>(part);
  for (int i0 = lane; i0 < 2 * ntile; i0 += 32 * kPartialBatch) {
    float2 v[kPartialBatch];
#pragma unroll
    for (int k = 0; k < kPartialBatch; ++k) {
      const int i = i0 + 32 * k;
      v[k] = i < 2 * ntile ? p2[i] : make_float2(0.0f, 0.0f);
    }
#pragma unroll
    for (int k = 0; k < kPartialBatch; ++k) {
      const int i = i0 + 32 * k;
      if (i >= 2 * ntile) break;
      sw.add(v[k].y);
      if (i < ntile) su0.add(v[k].x); else su1.add(v[k].x);
    }
  }
  su0.warp_reduce();
  su1.warp_reduce();
  sw.warp_reduce();
  *u0 = su0;
  *u1 = su1;
  *w = sw;
}
__device__ __forceinline__ void sum_partials(const float* part, int ntile, int lane, double* u0, double* u1,
                                             double* w) {
  FloatFloat a, b, c;
  sum_partials(part, ntile, lane, &a, &b, &c);
  *u0 = a.value();
  *u1 = b.value();
  *w = c.value();
}

// Double-float partials [comp][tile][u, w]: double-float sums in a fixed
// order (every lane ends with the same bits, as above).
__device__ __forceinline__ void sum_partials(const DF* part, int ntile, int lane, DF* u0, DF* u1, DF* w) {
  DF su0(0), su1(0), sw(0);
  const float4* p4 = reinterpret_cast<const float4*>(part);
  for (int i0 = lane; i0 < 2 * ntile; i0 += 32 * kPartialBatch) {
    float4 v[kPartialBatch];
#pragma unroll
    for (int k = 0; k < kPartialBatch; ++k) {
      const int i = i0 + 32 * k;
      v[k] = i < 2 * ntile ? p4[i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
#pragma unroll
    for (int k = 0; k < kPartialBatch; ++k) {
      const int i = i0 + 32 * k;
      if (i >= 2 * ntile) break;
      sw += DF(v[k].z, v[k].w);
      if (i < ntile) su0 += DF(v[k].x, v[k].y); else su1 += DF(v[k].x, v[k].y);
    }
  }
  *u0 = warp_sum(su0);
  *u1 = warp_sum(su1);
  *w = warp_sum(sw);
}
__device__ __forceinline__ void sum_partials(const DF* part, int ntile, int lane, double* u0, double* u1,
                                             double* w) {
  DF a, b, c;
  sum_partials(part, ntile, lane, &a, &b, &c);
  *u0 = from_df(a);
  *u1 = from_df(b);
  *w = from_df(c);
}

// lambda = sqrt(num / w) of the row pass, in the working precision.
__device__ __forceinline__ float row_lambda(const float* part, int ntile, int lane, float norm_num, double* u0,
                                            double* u1, bool want_u) {
  FloatFloat a, b, c;
  sum_partials(part, ntile, lane, &a, &b, &c);
  if (want_u) {
    *u0 = a.value();
    *u1 = b.value();
  }
  return sqrtf(norm_num / (c.hi + c.lo));
}
__device__ __forceinline__ double row_lambda(const double* part, int ntile, int lane, double norm_num, double* u0,
                                             double* u1, bool) {
  double sw;
  sum_partials(part, ntile, lane, u0, u1, &sw);
  return sqrt(norm_num / sw);
}
// double-float: the sums in double-float, the square root of the quotient in
// FP64 (a few FP64 operations per block) rounded to a double-float value
__device__ __forceinline__ DF row_lambda(const DF* part, int ntile, int lane, DF norm_num, double* u0, double* u1,
                                         bool want_u) {
  DF a, b, c;
  sum_partials(part, ntile, lane, &a, &b, &c);
  if (want_u) {
    *u0 = from_df(a);
    *u1 = from_df(b);
  }
  return to_df(sqrt(from_df(norm_num) / from_df(c)));
}

// lambda (and the population sums) from the column pass's final sums
// (u0, u1, w) as exact FP64 values of the sums above: the same bits as
// row_lambda computes from the partials.
__device__ __forceinline__ float row_lambda_final(const double* f, float norm_num, double* u0, double* u1) {
  *u0 = f[0];
  *u1 = f[1];
  return sqrtf(norm_num / float(f[2]));
}
__device__ __forceinline__ double row_lambda_final(const double* f, double norm_num, double* u0, double* u1) {
  *u0 = f[0];
  *u1 = f[1];
  return sqrt(norm_num / f[2]);
}
__device__ __forceinline__ DF row_lambda_final(const double* f, DF norm_num, double* u0, double* u1) {
  *u0 = f[0];
  *u1 = f[1];
  return to_df(sqrt(from_df(norm_num) / f[2]));
}

// Sums (u_0, u_1, w) of the column-pass partials [2][ntile][u, w] by every
// thread of one block, in FP64 (the partials' values are exact in FP64):
// each thread adds a strided share (all loads in flight at once), then warp
// butterflies and warp 0 combine the warps in a fixed order.  Called by the
// block that finishes a column pass last; out[0..2] receive the sums.
template <typename R> __device__ __forceinline__ double partial_value(const R* p) { return double(*p); }
template <> __device__ __forceinline__ double partial_value<DF>(const DF* p) { return from_df(*p); }
template <typename R>
__device__ __forceinline__ void final_sums(const R* part, int ntile, int tid, int nthreads, double* out) {
  __shared__ double s_sum[3][32];
  double u0 = 0.0, u1 = 0.0, w = 0.0;
  for (int i = tid; i < 2 * ntile; i += nthreads) {
    const double u = partial_value(part + 2 * i), ww = partial_value(part + 2 * i + 1);
    w += ww;
    if (i < ntile) u0 += u; else u1 += u;
  }
  u0 = warp_sum(u0);
  u1 = warp_sum(u1);
  w = warp_sum(w);
  const int warp = tid >> 5, lane = tid & 31, nw = (nthreads + 31) >> 5;
  if (lane == 0) {
    s_sum[0][warp] = u0;
    s_sum[1][warp] = u1;
    s_sum[2][warp] = w;
  }
  __syncthreads();
  if (warp == 0) {
    u0 = lane < nw ? s_sum[0][lane] : 0.0;
    u1 = lane < nw ? s_sum[1][lane] : 0.0;
    w = lane < nw ? s_sum[2][lane] : 0.0;
    u0 = warp_sum(u0);
    u1 = warp_sum(u1);
    w = warp_sum(w);
    if (lane == 0) {
      out[0] = u0;
      out[1] = u1;
      out[2] = w;
    }
  }
}

// Sum of |v[m]|^2 over the E points of a thread, pairwise in the working
// precision.  Block sums continue pairwise (warp butterfly, then across
// warps), so a block partial carries about log2(block points) roundings; only
// the cross-block sum is FP64.  (FP64 arithmetic runs at a small fraction of
// the FP32 rate on this GPU, so it is kept out of the per-thread work.)
template <int E, class C> __device__ __forceinline__ decltype(C::x) thread_norm2(const C (&v)[E]) {
  using R = decltype(C::x);
  R s[E];
#pragma unroll
  for (int m = 0; m < E; ++m) s[m] = cabs2(v[m]);
#pragma unroll
  for (int w = 1; w < E; w <<= 1)
#pragma unroll
    for (int m = 0; m + w < E; m += 2 * w) s[m] += s[m + w];
  return s[0];
}

__device__ __forceinline__ void sin_cos(float x, float* s, float* c) { sincosf(x, s, c); }
__device__ __forceinline__ void sin_cos(double x, double* s, double* c) { sincos(x, s, c); }
__device__ __forceinline__ float exp_r(float x) { return expf(x); }
__device__ __forceinline__ double exp_r(double x) { return exp(x); }

// sin and cos of an FP32 argument.  For |x| <= pi/4 (always the case for the
// interaction phases of a stable time step) the Taylor series of sin to x^9
// and of cos to x^10 in Horner form; the first omitted terms are below
// 2e-9 (sin, relative) and 1.2e-10 (cos) there, under half an FP32 ulp.
// Larger arguments use the library sincosf.
__device__ __forceinline__ void sin_cos_phase(float x, float* s, float* c) {
  if (fabsf(x) <= 0.125f) {
    // real-time phases of a stable step are this small: sin to x^5 and cos
    // to x^6 (omitted terms below 1e-9 relative / 2e-12 absolute there)
    const float x2 = x * x;
    float ps = fmadd(x2, 1.0f / 120.0f, -1.0f / 6.0f);
    *s = fmadd(ps * x2, x, x);
    float pc = fmadd(x2, -1.0f / 720.0f, 1.0f / 24.0f);
    pc = fmadd(pc, x2, -0.5f);
    *c = fmadd(pc, x2, 1.0f);
  } else if (fabsf(x) <= 0.78539816f) {
    const float x2 = x * x;
    float ps = fmadd(x2, 1.0f / 362880.0f, -1.0f / 5040.0f);
    ps = fmadd(ps, x2, 1.0f / 120.0f);
    ps = fmadd(ps, x2, -1.0f / 6.0f);
    *s = fmadd(ps * x2, x, x);
    float pc = fmadd(x2, -1.0f / 3628800.0f, 1.0f / 40320.0f);
    pc = fmadd(pc, x2, -1.0f / 720.0f);
    pc = fmadd(pc, x2, 1.0f / 24.0f);
    pc = fmadd(pc, x2, -0.5f);
    *c = fmadd(pc, x2, 1.0f);
  } else {
    sincosf(x, s, c);
  }
}
__device__ __forceinline__ void sin_cos_phase(double x, double* s, double* c) { sincos(x, s, c); }
__device__ __forceinline__ void sin_cos_phase(DF x, DF* s, DF* c) { df_sincos(x, s, c); }
__device__ __forceinline__ DF exp_r(DF x) { return df_exp(x); }

// exp(z * e) for the interaction operator.
template <typename R> __device__ __forceinline__ Cx<R> cexp_z(R zr, R zi, R e) {
  using C = Cx<R>;
  if (zi == R(0)) return cmake<C>(exp_r(zr * e), R(0));
  R sn, cs;
  sin_cos_phase(zi * e, &sn, &cs);
  if (zr == R(0)) return cmake<C>(cs, sn);
  const R g = exp_r(zr * e);
  return cmake<C>(g * cs, g * sn);
}

// Operator values at one point: coupling c, s conj(e), s e; potential
// factors (x part, y part) of each component.
template <typename R> struct PointOps {
  Cx<R> cc, s01, s10, pa0, pb0, pa1, pb1;
};

// Real-space operators of one sub-step at one point x of a row, both
// components (tensor_propagator.py:247-267): interaction, coupling,
// potential, coupling, and the interaction again with the same operator.
template <typename R>
__device__ __forceinline__ void apply_real_ops(Cx<R>& p0, Cx<R>& p1, const PointOps<R>& v, const RowArgs<R>& a) {
  using C = Cx<R>;
  const RealOp<R>& op = a.op;
  const R n0 = cabs2(p0), n1 = cabs2(p1);
  const R e0 = fmadd(a.g_uu, n0, a.g_ud * n1);
  const R e1 = fmadd(a.g_dd, n1, a.g_ud * n0);
  const C i0 = cexp_z(op.zr, op.zi, e0);
  const C i1 = cexp_z(op.zr, op.zi, e1);
  // Factors with zero imaginary parts are applied as real scalings: for
  // b = (x, 0), cmul(a, b) = (fma(a.x, x, -0), fma(a.x, 0, a.y x)) is
  // bit-identical to (a.x x, a.y x).
  const bool ireal = (op.zi == R(0));
  if (ireal) {
    p0 = cscale(p0, i0.x);
    p1 = cscale(p1, i1.x);
  } else {
    p0 = cmul(p0, i0);
    p1 = cmul(p1, i1);
  }
  const C cc = v.cc, s01 = v.s01, s10 = v.s10;
  if (a.coupling) {
    const C c0 = op.real_cc ? cscale(p0, cc.x) : cmul(cc, p0);
    const C c1 = op.real_cc ? cscale(p1, cc.x) : cmul(cc, p1);
    const C q0 = cadd(c0, cmul(s01, p1));
    const C q1 = cadd(cmul(s10, p0), c1);
    p0 = q0;
    p1 = q1;
  }
  if (op.real_pot) {
    p0 = cscale(p0, v.pa0.x * v.pb0.x);
    p1 = cscale(p1, v.pa1.x * v.pb1.x);
  } else {
    p0 = cmul(p0, cmul(v.pa0, v.pb0));
    p1 = cmul(p1, cmul(v.pa1, v.pb1));
  }
  if (a.coupling) {
    const C c0 = op.real_cc ? cscale(p0, cc.x) : cmul(cc, p0);
    const C c1 = op.real_cc ? cscale(p1, cc.x) : cmul(cc, p1);
    const C q0 = cadd(c0, cmul(s01, p1));
    const C q1 = cadd(cmul(s10, p0), c1);
    p0 = q0;
    p1 = q1;
  }
  if (ireal) {
    p0 = cscale(p0, i0.x);
    p1 = cscale(p1, i1.x);
  } else {
    p0 = cmul(p0, i0);
    p1 = cmul(p1, i1);
  }
}

// The same with coupling, potential and coupling applied as one 2x2 matrix
// per point, pb(y) A(x) (the separable kernels, RealOp::sep): interaction,
// A, then pb times the interaction again (pb is a scalar for both
// components, so it commutes).
template <typename R>
__device__ __forceinline__ void apply_fused_ops(Cx<R>& p0, Cx<R>& p1, const Cx<R> (&m)[4], Cx<R> pb,
                                                const RowArgs<R>& a) {
  using C = Cx<R>;
  const RealOp<R>& op = a.op;
  const R n0 = cabs2(p0), n1 = cabs2(p1);
  const R e0 = fmadd(a.g_uu, n0, a.g_ud * n1);
  const R e1 = fmadd(a.g_dd, n1, a.g_ud * n0);
  const C i0 = cexp_z(op.zr, op.zi, e0);
  const C i1 = cexp_z(op.zr, op.zi, e1);
  const bool ireal = (op.zi == R(0));
  if (ireal) {
    p0 = cscale(p0, i0.x);
    p1 = cscale(p1, i1.x);
  } else {
    p0 = cmul(p0, i0);
    p1 = cmul(p1, i1);
  }
  C q0, q1;
  if (op.diag) {
    q0 = cmul(m[0], p0);
    q1 = cmul(m[3], p1);
  } else {
    q0 = cadd(cmul(m[0], p0), cmul(m[1], p1));
    q1 = cadd(cmul(m[2], p0), cmul(m[3], p1));
  }
  if (ireal && op.real_mb) {
    p0 = cscale(q0, i0.x * pb.x);
    p1 = cscale(q1, i1.x * pb.x);
  } else if (ireal) {
    p0 = cmul(q0, cscale(pb, i0.x));
    p1 = cmul(q1, cscale(pb, i1.x));
  } else {
    p0 = cmul(q0, cmul(i0, pb));
    p1 = cmul(q1, cmul(i1, pb));
  }
}

// The same with the operator values read through the generic broadcast
// fields (any stride pattern, row-constant values hoisted by RowFields).
template <typename R>
__device__ __forceinline__ void real_space_ops(Cx<R>& p0, Cx<R>& p1, int x, const RowFields<R>& rf,
                                               const RowArgs<R>& a) {
  using C = Cx<R>;
  PointOps<R> v;
  if (a.coupling) {
    v.cc = rf.at(kCc, x);
    if (a.op.has_s01) {
      v.s01 = rf.at(kS01, x);
      v.s10 = rf.at(kS10, x);
    } else {
      const C sv = rf.at(kCs, x), e = rf.at(kCe, x);
      v.s01 = cmulc(sv, e);
      v.s10 = cmul(sv, e);
    }
  } else {
    v.cc = v.s01 = v.s10 = C{};
  }
  v.pa0 = rf.at(kPa0, x);
  v.pb0 = rf.at(kPb0, x);
  v.pa1 = rf.at(kPa1, x);
  v.pb1 = rf.at(kPb1, x);
  apply_real_ops(p0, p1, v, a);
}

// v[m] *= ka(x, ky) * kb(x, ky) for ky = j + m*T along one column x; a
// factor that does not vary along the column (sy == 0) is loaded once.
template <typename R, int E, int T>
__device__ __forceinline__ void apply_kinetic(Cx<R> (&v)[E], const KinOp<R>& k, int comp, int x, int j) {
  using C = Cx<R>;
  if (k.sep) {  // x-table times y-table, unit strides
    const C ka = ldg(k.a[comp].p + x);
    const C* kb = k.b[comp].p + j;
    if (k.real) {  // same bits as the complex products (see apply_real_ops)
#pragma unroll
      for (int m = 0; m < E; ++m) v[m] = cscale(v[m], ka.x * ldg(&kb[m * T].x));
    } else {
#pragma unroll
      for (int m = 0; m < E; ++m) v[m] = cmul(v[m], cmul(ka, ldg(kb + m * T)));
    }
    return;
  }
  const Field<R>& fa = k.a[comp];
  const Field<R>& fb = k.b[comp];
  const bool a_const = (fa.sy == 0), b_const = (fb.sy == 0);
  const C a0 = fld(fa, x, j), b0 = fld(fb, x, j);
#pragma unroll
  for (int m = 0; m < E; ++m) {
    const int ky = j + m * T;
    const C ka = (a_const || m == 0) ? a0 : fld(fa, x, ky);
    const C kb = (b_const || m == 0) ? b0 : fld(fb, x, ky);
    v[m] = cmul(v[m], cmul(ka, kb));
  }
}

// ----------------------------------------------------------------- row pass
// Block: ROWS rows, both components; T = N/E threads per (row, component)
// line, so 2*T*ROWS threads.  Thread (rho, comp, j) transforms one line; the
// point-wise operators, which couple the components, run between the
// transforms on the natural-order rows left in shared memory.
// Tensor-core DFT16 staging for a block whose exchange area takes
// `exchange_bytes`: B fragments after it (16-byte aligned), copied from the
// plan's table `tcb`, then one tile per warp.  Every thread copies its share
// of the fragments; the caller synchronises the block before the first
// transform.
template <bool TC>
__device__ __forceinline__ TcScratch tc_setup(unsigned char* smem_raw, size_t exchange_bytes, const uint32_t* tcb,
                                              int tid, int nthreads) {
  TcScratch t{};
  if constexpr (TC) {
    const size_t off = (exchange_bytes + 15) & ~size_t(15);
    uint32_t* bfrag = reinterpret_cast<uint32_t*>(smem_raw + off);
    // copy of the plan's B fragments (tc_fill_bfrag, computed once)
    for (int i = tid; i < kTcBfragWords / 4; i += nthreads)
      reinterpret_cast<uint4*>(bfrag)[i] = __ldg(reinterpret_cast<const uint4*>(tcb) + i);
    t.bfrag = bfrag;
    t.tile = reinterpret_cast<float*>(smem_raw + off + sizeof(uint32_t) * kTcBfragWords) + (tid >> 5) * kTcScratchFloats;
  }
  return t;
}

// Position of a pass block among the blocks of its pass: block indices x
// (lines or tiles) and y (the column pass's component), and the number of
// x positions.  The pass kernels take it from the grid; the batch queue
// kernel gives each work item its own.
struct BlockPos {
  int x, y, nx;
};
__device__ __forceinline__ BlockPos grid_pos() { return BlockPos{int(blockIdx.x), int(blockIdx.y), int(gridDim.x)}; }

// SEP selects the point-wise code at compile time (separable operator
// tables, RealOp::sep, or the generic broadcast fields), so each kernel
// carries one of the two loops and stays small in the instruction cache.
// TC: radix-16 stages on the tensor cores (complex64 only).
// QUEUE: called by the batch queue kernel (plain loads and stores instead of
// bulk copies: the state is written by other blocks of the same launch).
template <typename R, int N, int E, int ROWS, bool SEP, bool TC = false, bool QUEUE = false>
__device__ __forceinline__ void row_body(const RowArgs<R>& a, const BlockPos pos) {
  using C = Cx<R>;
  static_assert(!TC || sizeof(R) == 4, "tensor-core DFT16 is complex64 only");
  constexpr int T = N / E;
  constexpr int LS = N + N / E;
  constexpr int NT = 2 * T * ROWS;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* sm = reinterpret_cast<C*>(smem_raw);
  __shared__ R s_lambda;

  const int tid = threadIdx.x;
  const TcScratch tcs = tc_setup<TC>(smem_raw, sizeof(C) * 2 * ROWS * LS, a.tcb, tid, NT);
  if constexpr (TC) __syncthreads();
  const int rho = tid / (2 * T);
  const int comp = (tid / T) & 1;
  const int j = tid % T;
  const int y = pos.x * ROWS + rho;
  const long long row_off = (long long)y * N;

  C v[1][E];
  const C* __restrict__ in = a.in[comp];
  constexpr int kTma = (N >= SGPE_ROW_TMA_MIN_N && !QUEUE) ? SGPE_ROW_TMA : 0;
  bool staged = false;
  if constexpr (kTma >= 1) {
    // The block's 2*ROWS input lines are staged by bulk copies into the
    // start of the exchange area (unpadded, line after line) when both
    // components are 16-byte aligned (a line of N*sizeof(C) bytes always is
    // a multiple of 16).
    __shared__ __align__(8) uint64_t s_bar;
    const bool tma = aligned16(a.in[0]) && aligned16(a.in[1]);
    if (tma) {
      if (tid == 0) mbar_init(&s_bar, 1);
      __syncthreads();
    }
    wait_for_previous_grid();
    if (tma) {
      constexpr uint32_t kLine = N * sizeof(C);
      if (tid == 0) {
        mbar_arrive_expect_tx(&s_bar, 2 * ROWS * kLine);
#pragma unroll
        for (int c = 0; c < 2; ++c)
#pragma unroll
          for (int r = 0; r < ROWS; ++r)
            bulk_load(sm + (c * ROWS + r) * N, a.in[c] + (long long)(pos.x * ROWS + r) * N, kLine, &s_bar);
      }
      staged = mbar_wait_bounded(&s_bar, 0);
      if (staged) {
        const C* line = sm + (comp * ROWS + rho) * N;
#pragma unroll
        for (int m = 0; m < E; ++m) v[0][m] = line[j + m * T];
      } else if (a.err != nullptr) {
        atomicExch(a.err, kErrCopyTimeout);
      }
      __syncthreads();  // the staged lines overlap the exchange lines
    }
  } else {
    wait_for_previous_grid();
  }
  if (!staged) {
#pragma unroll
    for (int m = 0; m < E; ++m) v[0][m] = ld_state(in + row_off + j + m * T);
  }
  allow_next_grid();
  // line (comp, rho) at sm + (comp*ROWS + rho)*LS; a line's T threads lie in
  // one warp when T divides 32 (the transforms then synchronise per warp)
  // lines of T >= 32 threads are whole warps: each synchronises its own
  // exchanges on named barrier 1 + line (SGPE_ROW_LINE_BARRIERS)
  constexpr bool kLineBar = SGPE_ROW_LINE_BARRIERS && (T % 32 == 0) && (2 * ROWS <= 15);
  const LineSmem<C, E, (32 % T == 0), TC> smv{sm + (comp * ROWS + rho) * LS, 0, tcs,
                                              kLineBar ? 1 + comp * ROWS + rho : 0, kLineBar ? T : 0};

  if (a.mode == kRowStep) {
    // inverse x transform, result left in shared memory (natural order)
    fft_lines<N, E, +1, 1, false, true>(v, j, smv, a.tw);
    // lambda (and the populations) from the partials of the column pass;
    // warp 0 does this after its own part of the transform, so the other
    // warps are not held up
    if (tid < 32) {
      double su0 = 0.0, su1 = 0.0;
      const bool want_u = (a.pops != nullptr && pos.x == 0);
      const R l = a.fin != nullptr ? row_lambda_final(a.fin, R(a.norm_num), &su0, &su1)
                                   : row_lambda(a.part, a.ntile, tid, R(a.norm_num), &su0, &su1, want_u);
      if (tid == 0) {
        s_lambda = l;
        if (want_u) {
          a.pops[0] = a.atom_num * su0 / (su0 + su1);
          a.pops[1] = a.atom_num * su1 / (su0 + su1);
        }
      }
    }
    __syncthreads();
    const R lam = s_lambda;
    // point-wise operators: the 2T threads of a row share its N points
    {
      const LineSmem<C, E> r0{sm + rho * LS, 0};
      const LineSmem<C, E> r1{sm + (ROWS + rho) * LS, 0};
      const int jj = tid % (2 * T);
      // element x = jj + m*2T of each row: padded position pad(jj) + m*kStep
      // when 2T is a multiple of E (every power-of-two plan)
      using LS0 = LineSmem<C, E>;
      constexpr bool kOpsFold = (2 * T) % E == 0;
      constexpr int kStep = 2 * T + (2 * T) / E;
      C* const q0 = r0.line(0) + LS0::pad(unsigned(jj));
      C* const q1 = r1.line(0) + LS0::pad(unsigned(jj));
      auto at0 = [&](int m, int x) -> C& { return kOpsFold ? q0[m * kStep] : r0.line(0)[LS0::pad(unsigned(x))]; };
      auto at1 = [&](int m, int x) -> C& { return kOpsFold ? q1[m * kStep] : r1.line(0)[LS0::pad(unsigned(x))]; };
      if constexpr (SEP) {
        // separable operators as pb(y) A(x): the x-tables read at jj + m*2T
        // (compile-time offsets from one base), the row's pb hoisted
        const C pb = ldg(a.op.mb.p + y);
        const C* m0 = a.op.m[0].p + jj;
        const C* m1 = a.op.m[1].p + jj;
        const C* m2 = a.op.m[2].p + jj;
        const C* m3 = a.op.m[3].p + jj;
        const bool diag = a.op.diag != 0;
#pragma unroll ops_unroll<R>()
        for (int m = 0; m < E / 2; ++m) {
          const int x = jj + m * 2 * T;
          C p0 = cscale(at0(m, x), lam), p1 = cscale(at1(m, x), lam);
          C mm[4];
          mm[0] = ldg(m0 + m * 2 * T);
          mm[3] = ldg(m3 + m * 2 * T);
          if (!diag) {
            mm[1] = ldg(m1 + m * 2 * T);
            mm[2] = ldg(m2 + m * 2 * T);
          }
          apply_fused_ops<R>(p0, p1, mm, pb, a);
          at0(m, x) = p0;
          at1(m, x) = p1;
        }
      } else {
        RowFields<R> rf;
        rf.init(a.op, y);
#pragma unroll ops_unroll<R>()
        for (int m = 0; m < E / 2; ++m) {
          const int x = jj + m * 2 * T;
          C p0 = cscale(at0(m, x), lam), p1 = cscale(at1(m, x), lam);
          real_space_ops<R>(p0, p1, x, rf, a);
          at0(m, x) = p0;
          at1(m, x) = p1;
        }
      }
    }
    __syncthreads();
    // forward x transform straight from shared memory
    fft_lines<N, E, -1, 1, true, false>(v, j, smv, a.tw);
  } else {
    if (a.mode == kRowForward) fft_lines<N, E, -1, 1>(v, j, smv, a.tw);
    else fft_lines<N, E, +1, 1>(v, j, smv, a.tw);
#pragma unroll
    for (int m = 0; m < E; ++m) v[0][m] = cscale(v[0][m], a.scale);
  }
  C* out = a.out[comp];
  if (kTma >= 2 && aligned16(a.out[0]) && aligned16(a.out[1])) {
    // output lines through shared memory and bulk stores
    constexpr uint32_t kLine = N * sizeof(C);
    __syncthreads();  // the transform's last exchange has been read
    C* line = sm + (comp * ROWS + rho) * N;
#pragma unroll
    for (int m = 0; m < E; ++m) line[j + m * T] = v[0][m];
    fence_proxy_async_smem();
    __syncthreads();
    if (tid == 0) {
#pragma unroll
      for (int c = 0; c < 2; ++c)
#pragma unroll
        for (int r = 0; r < ROWS; ++r)
          bulk_store(a.out[c] + (long long)(pos.x * ROWS + r) * N, sm + (c * ROWS + r) * N, kLine);
      bulk_commit();
      bulk_wait_read();
    }
    return;
  }
#pragma unroll
  for (int m = 0; m < E; ++m) st_state(out + row_off + j + m * T, v[0][m]);
  (void)NT;
}

template <typename R, int N, int E, int ROWS, int MINB, bool SEP, bool TC = false>
__global__ void __launch_bounds__(2 * (N / E) * ROWS, MINB)
row_kernel(const RowArgs<R> a) {
  row_body<R, N, E, ROWS, SEP, TC>(a, grid_pos());
}

// Several solves of one size in one launch (a batch): blockIdx.y selects the
// solve's arguments.
template <typename R, int N, int E, int ROWS, int MINB, bool SEP>
__global__ void __launch_bounds__(2 * (N / E) * ROWS, MINB)
row_kernel_grouped(const RowArgs<R>* __restrict__ args) {
  row_body<R, N, E, ROWS, SEP>(args[blockIdx.y], grid_pos());
}

// -------------------------------------------------------------- column pass
template <typename R, int N, int E, int COLS, bool TC = false, bool QUEUE = false>
__device__ __forceinline__ void col_body(const ColArgs<R>& a, const BlockPos pos) {
  using C = Cx<R>;
  static_assert(!TC || sizeof(R) == 4, "tensor-core DFT16 is complex64 only");
  constexpr int T = N / E;
  constexpr int LS = N + N / E + 2;
  constexpr int NT = T * COLS;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* sm = reinterpret_cast<C*>(smem_raw);
  constexpr int NW = NT / 32;
  __shared__ R s_red[2][NW];

  const int tid = threadIdx.x;
  const TcScratch tcs = tc_setup<TC>(smem_raw, sizeof(C) * COLS * LS, a.tcb, tid, NT);
  if constexpr (TC) __syncthreads();
  const int c = tid % COLS;
  const int j = tid / COLS;
  const int comp = pos.y;
  const int nx = a.nx;
  const int x = pos.x * COLS + c;
  const int half = nx / 2;
  const int xin = a.in_shift ? (x + half) % nx : x;
  const int xout = a.out_shift ? (x + half) % nx : x;
  const C* __restrict__ in = a.in[comp];
  C* out = a.out[comp];

  C v[1][E];
  // TMA staging of the block's tile: rows of COLS complex values, row-major,
  // at a 128-byte aligned start of the exchange area
  constexpr bool kTma = SGPE_COL_TMA && N >= SGPE_COL_TMA_MIN_N && !QUEUE;
  constexpr int kBoxY = N < 256 ? N : 256;
  constexpr uint32_t kTileBytes = uint32_t(COLS) * N * sizeof(C);
  static_assert(!kTma || sizeof(C) * COLS * (N / E + 2) >= 128, "the aligned tile must fit the exchange area");
  static_assert(!kTma || (COLS * sizeof(C)) % 16 == 0, "tile rows must be whole 16-byte units");
  C* const stage = reinterpret_cast<C*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
  const char* const tmap = static_cast<const char*>(a.tmap) + comp * 128;
  bool staged = false;
  if constexpr (kTma) {
    __shared__ __align__(8) uint64_t s_bar;
    const bool tma = a.tmap != nullptr;
    if (tma) {
      if (tid == 0) {
        mbar_init(&s_bar, 1);
        prefetch_tensormap(tmap);
      }
      __syncthreads();
    }
    wait_for_previous_grid();
    if (tma) {
      if (tid == 0) {
        mbar_arrive_expect_tx(&s_bar, kTileBytes);
#pragma unroll
        for (int b = 0; b < N / kBoxY; ++b)
          tensor_load_2d(stage + b * kBoxY * COLS, tmap, pos.x * COLS * 2, b * kBoxY, &s_bar);
      }
      staged = mbar_wait_bounded(&s_bar, 0);
      if (staged) {
#pragma unroll
        for (int m = 0; m < E; ++m) v[0][m] = stage[(j + m * T) * COLS + c];
      } else if (a.err != nullptr) {
        atomicExch(a.err, kErrCopyTimeout);
      }
      __syncthreads();  // the tile overlaps the exchange lines
    }
  } else {
    wait_for_previous_grid();
  }
  if (!staged) {
#pragma unroll
    for (int m = 0; m < E; ++m) {
      const int row = j + (a.in_shift ? (m + E / 2) % E : m) * T;
      v[0][m] = ld_state(in + (long long)row * nx + xin);
    }
  }
  allow_next_grid();
  const LineSmem<C, E, false, TC> smv{sm + c * LS, 0, tcs};
  if (a.fwd) fft_lines<N, E, -1, 1>(v, j, smv, a.tw);

  R su = R(0), sw = R(0);
  if (a.nk >= 1) apply_kinetic<R, E, T>(v[0], a.k1, comp, x, j);
  if (a.part != nullptr) su = thread_norm2(v[0]);
  sw = su;
  if (a.nk >= 2) {
    apply_kinetic<R, E, T>(v[0], a.k2, comp, x, j);
    if (a.part != nullptr) sw = thread_norm2(v[0]);
  }
  if (a.inv) fft_lines<N, E, +1, 1>(v, j, smv, a.tw);
  if (a.scale != R(1)) {
#pragma unroll
    for (int m = 0; m < E; ++m) v[0][m] = cscale(v[0][m], a.scale);
  }
  if (kTma && a.tmap != nullptr) {
    // the tile back through shared memory and tensor stores (in place)
    __syncthreads();  // the transform's last exchange has been read
#pragma unroll
    for (int m = 0; m < E; ++m) stage[(j + m * T) * COLS + c] = v[0][m];
    fence_proxy_async_smem();
    __syncthreads();
    if (tid == 0) {
#pragma unroll
      for (int b = 0; b < N / kBoxY; ++b)
        tensor_store_2d(tmap, pos.x * COLS * 2, b * kBoxY, stage + b * kBoxY * COLS);
      bulk_commit();
      bulk_wait_read();
    }
  } else {
#pragma unroll
    for (int m = 0; m < E; ++m) {
      const int row = j + (a.out_shift ? (m + E / 2) % E : m) * T;
      st_state(out + (long long)row * nx + xout, v[0][m]);
    }
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
    if (warp == 0) {
      R bu = lane < NW ? s_red[0][lane] : R(0);
      R bw = lane < NW ? s_red[1][lane] : R(0);
      bu = warp_sum(bu);
      bw = warp_sum(bw);
      if (lane == 0) {
        R* dst = a.part + 2 * ((long long)comp * pos.nx + pos.x);
        dst[0] = bu;
        dst[1] = bw;
      }
    }
    if (a.fin != nullptr) {
      // the last block to finish sums every block's partials (no block waits)
      __shared__ bool s_last;
      if (tid == 0) {
        __threadfence();  // this block's partial is visible before its arrival
        const unsigned ticket = atomicAdd(a.count, 1u);
        s_last = (ticket == 2u * unsigned(pos.nx) - 1u);
      }
      __syncthreads();
      if (s_last) {
        __threadfence();
        final_sums(static_cast<const R*>(a.part), pos.nx, tid, NT, a.fin);
        if (tid == 0) *a.count = 0u;
      }
    }
  }
}

template <typename R, int N, int E, int COLS, int MINB, bool TC = false>
__global__ void __launch_bounds__((N / E) * COLS, MINB)
col_kernel(const ColArgs<R> a) {
  col_body<R, N, E, COLS, TC>(a, grid_pos());
}

// Several solves of one size in one launch: blockIdx.z selects the solve.
template <typename R, int N, int E, int COLS, int MINB>
__global__ void __launch_bounds__((N / E) * COLS, MINB)
col_kernel_grouped(const ColArgs<R>* __restrict__ args) {
  col_body<R, N, E, COLS>(args[blockIdx.z], grid_pos());
}

// Final k-space renormalisation of a materialised psik
// (tensor_propagator.py:271) and, optionally, its populations
// (tensor_tools.py:466-484).
template <typename R>
__global__ void __launch_bounds__(256) scale_kernel(const ScaleArgs<R> a) {
  __shared__ double s_alpha;
  if (threadIdx.x < 32) {
    double s0, s1, sw;
    sum_partials(a.part, a.ntile, threadIdx.x, &s0, &s1, &sw);
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

// Conversion copies of a double-float plan's state: complex128 psik into
// the double-float state (load), and the double-float state out to complex128
// (store), with the fftshift of psik's centred order and, on store, the final
// k-space renormalisation from the column pass's partials.
struct DfCopyArgs {
  const void* in[2];
  void* out[2];
  int nx, ny;
  int shift;            // out = fftshift(in) in both axes (even sizes)
  int to_df;            // 1: double2 -> DFC, 0: DFC -> double2
  const DF* part;       // non-null (store): renormalise with these partials
  int ntile;
  double atom_num, dv;
  double* pops;         // non-null (store): populations
};

}  // namespace sgpe
