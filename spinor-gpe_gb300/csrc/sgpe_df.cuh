// Double-float arithmetic (FP32 pairs) for the double-float precision of the
// split-step solver.
//
// A double-float value is hi + lo with |lo| <= ulp(hi)/2: about 48
// significant bits carried by FP32 numbers, so that every operation runs on
// the FP32 pipes (GB300 executes FP64 at a small fraction of its FP32 rate).
// The building blocks are the error-free transformations of Knuth (TwoSum:
// the exact rounding error of a sum), Dekker (FastTwoSum, for |a| >= |b|) and
// the FMA form of the exact product (the rounding error of a*b is
// fma(a, b, -a*b)); see T. J. Dekker, "A floating-point technique for
// extending the available precision", Numer. Math. 18 (1971), and
// Y. Hida, X. S. Li, D. H. Bailey, "Algorithms for quad-double precision
// floating point arithmetic", ARITH-15 (2001), whose "sloppy" double-double
// addition is used here: the tails are added without a second TwoSum, an
// error of order 2^-47 of the operands' magnitude.
//
// Elementary functions (exp, sin, cos) are Taylor series in double-float
// arithmetic with 1/n! coefficients, after exact scaling of the argument by a
// power of two and the matching number of squarings / double-angle steps.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <type_traits>

namespace sgpe {

// (the _rn intrinsics keep the compiler from contracting these sequences
// into FMAs, which would break the error-free transformations)
struct DF {
  float hi, lo;
  DF() = default;
  __host__ __device__ constexpr DF(float h, float l) : hi(h), lo(l) {}
  __host__ __device__ constexpr explicit DF(double d) : hi(float(d)), lo(float(d - double(float(d)))) {}
  __host__ __device__ constexpr explicit DF(int i) : hi(float(i)), lo(0.0f) {}
};

template <class T> struct is_df : std::false_type {};
template <> struct is_df<DF> : std::true_type {};

__device__ __forceinline__ DF df_fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return DF(s, __fsub_rn(b, __fsub_rn(s, a)));
}
__device__ __forceinline__ DF operator+(DF a, DF b) {
  const float s = __fadd_rn(a.hi, b.hi);
  const float bb = __fsub_rn(s, a.hi);
  const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
  return df_fast_two_sum(s, __fadd_rn(e, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ DF operator-(DF a) { return DF(-a.hi, -a.lo); }
__device__ __forceinline__ DF operator-(DF a, DF b) { return a + (-b); }
__device__ __forceinline__ DF operator*(DF a, DF b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return df_fast_two_sum(p, e);
}
__device__ __forceinline__ DF& operator+=(DF& a, DF b) {
  a = a + b;
  return a;
}
__host__ __device__ __forceinline__ bool operator==(DF a, DF b) { return a.hi == b.hi && a.lo == b.lo; }
__host__ __device__ __forceinline__ bool operator!=(DF a, DF b) { return !(a == b); }

// a + b without the final renormalisation: the heads' TwoSum is exact and
// every lower-order term goes into the tail, but the tail may exceed half an
// ulp of the head by a few ulps.  The butterflies of a transform stage add
// with this and renormalise each value once at the end of the stage
// (df_renorm), which keeps ~47 bits at three fewer operations per sum.
__device__ __forceinline__ DF df_add_lazy(DF a, DF b) {
  const float s = __fadd_rn(a.hi, b.hi);
  const float bb = __fsub_rn(s, a.hi);
  const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
  return DF(s, __fadd_rn(e, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ DF df_renorm(DF a) { return df_fast_two_sum(a.hi, a.lo); }

// a * b + c with one renormalisation: the exact product's head and c's head
// through TwoSum, every lower-order term into the tail.
__device__ __forceinline__ DF df_fma(DF a, DF b, DF c) {
  const float p = __fmul_rn(a.hi, b.hi);
  const float pe = __fmaf_rn(a.hi, b.hi, -p);
  const float s = __fadd_rn(p, c.hi);
  const float bb = __fsub_rn(s, p);
  float e = __fadd_rn(__fsub_rn(p, __fsub_rn(s, bb)), __fsub_rn(c.hi, bb));
  e = __fadd_rn(e, __fadd_rn(pe, c.lo));
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return df_fast_two_sum(s, e);
}

// a * 2^k (exact)
__device__ __forceinline__ DF df_ldexp(DF a, int k) { return DF(ldexpf(a.hi, k), ldexpf(a.lo, k)); }

// Double-float complex value, 16 bytes: (re.hi, re.lo, im.hi, im.lo).
struct __align__(16) DFC {
  DF x, y;
};

// a.x * b.x - a.y * b.y (S = -1) or a.x * b.x + a.y * b.y (S = +1) with one
// TwoSum of the two product heads and one renormalisation.
template <int S> __device__ __forceinline__ DF df_dot2(DF ax, DF bx, DF ay, DF by) {
  const float p1 = __fmul_rn(ax.hi, bx.hi);
  const float e1 = __fmaf_rn(ax.hi, bx.hi, -p1);
  const float q = __fmul_rn(ay.hi, by.hi);
  const float e2 = __fmaf_rn(ay.hi, by.hi, -q);
  const float p2 = S > 0 ? q : -q;
  const float s = __fadd_rn(p1, p2);
  const float bb = __fsub_rn(s, p1);
  float t = __fadd_rn(__fsub_rn(p1, __fsub_rn(s, bb)), __fsub_rn(p2, bb));
  t = __fadd_rn(t, S > 0 ? __fadd_rn(e1, e2) : __fsub_rn(e1, e2));
  t = __fmaf_rn(ax.hi, bx.lo, t);
  t = __fmaf_rn(ax.lo, bx.hi, t);
  t = __fmaf_rn(S > 0 ? ay.hi : -ay.hi, by.lo, t);
  t = __fmaf_rn(S > 0 ? ay.lo : -ay.lo, by.hi, t);
  return df_fast_two_sum(s, t);
}

__device__ __forceinline__ DF to_df(double d) {
  const float h = __double2float_rn(d);
  return DF(h, __double2float_rn(d - double(h)));
}
__device__ __forceinline__ double from_df(DF a) { return double(a.hi) + double(a.lo); }
__device__ __forceinline__ DFC to_dfc(double2 z) { return DFC{to_df(z.x), to_df(z.y)}; }
__device__ __forceinline__ double2 from_dfc(DFC z) { return make_double2(from_df(z.x), from_df(z.y)); }

// Read-only loads through the non-coherent path, for the scalar and complex
// element types of every precision.
template <class T> __device__ __forceinline__ T ldg(const T* p) { return __ldg(p); }
template <> __device__ __forceinline__ DF ldg<DF>(const DF* p) {
  const float2 v = __ldg(reinterpret_cast<const float2*>(p));
  return DF(v.x, v.y);
}
template <> __device__ __forceinline__ DFC ldg<DFC>(const DFC* p) {
  const float4 v = __ldg(reinterpret_cast<const float4*>(p));
  return DFC{DF(v.x, v.y), DF(v.z, v.w)};
}

// Warp shuffle of a double-float value.
__device__ __forceinline__ DF shfl_xor(DF v, int o) {
  return DF(__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o));
}

// exp(x) for |x| <= 1/8: Taylor series to x^11 (the omitted terms are below
// 2^-50 of the result there).
__device__ __forceinline__ DF df_exp_small(DF x) {
  constexpr double kInvFact[12] = {1.0, 1.0, 1.0 / 2, 1.0 / 6, 1.0 / 24, 1.0 / 120, 1.0 / 720, 1.0 / 5040,
                                   1.0 / 40320, 1.0 / 362880, 1.0 / 3628800, 1.0 / 39916800};
  DF p = DF(kInvFact[11]);
#pragma unroll
  for (int n = 10; n >= 0; --n) p = df_fma(p, x, DF(kInvFact[n]));
  return p;
}

// Number of halvings that bring |x| (FP32 head) to at most 1/8.
__device__ __forceinline__ int df_reduction_steps(float ax) {
  if (!(ax > 0.125f)) return 0;
  int e = 0;
  frexpf(ax * 8.0f, &e);  // ax * 8 = m 2^e, m in [0.5, 1)
  return e;
}

// exp(x) for real x with |x| up to a few hundred: exp(x 2^-k)^(2^k).
// (Not inlined: one copy per kernel keeps the point-wise loops, and their
// compile time, small.)
static __device__ __noinline__ DF df_exp(DF x) {
  const int k = df_reduction_steps(fabsf(x.hi));
  DF r = df_exp_small(df_ldexp(x, -k));
  for (int i = 0; i < k; ++i) r = r * r;
  return r;
}

// sin and cos of x for |x| <= 1/8: Taylor series of sin to x^11 and of cos
// to x^12, Horner form in x^2.
__device__ __forceinline__ void df_sincos_small(DF x, DF* s, DF* c) {
  const DF x2 = x * x;
  // sin x = x (1 - x^2/3! + x^4/5! - x^6/7! + x^8/9! - x^10/11!)
  DF ps = DF(-1.0 / 39916800);
  ps = df_fma(ps, x2, DF(1.0 / 362880));
  ps = df_fma(ps, x2, DF(-1.0 / 5040));
  ps = df_fma(ps, x2, DF(1.0 / 120));
  ps = df_fma(ps, x2, DF(-1.0 / 6));
  ps = df_fma(ps, x2, DF(1.0f, 0.0f));
  *s = ps * x;
  // cos x = 1 - x^2/2! + x^4/4! - ... + x^12/12!
  DF pc = DF(1.0 / 479001600);
  pc = df_fma(pc, x2, DF(-1.0 / 3628800));
  pc = df_fma(pc, x2, DF(1.0 / 40320));
  pc = df_fma(pc, x2, DF(-1.0 / 720));
  pc = df_fma(pc, x2, DF(1.0 / 24));
  pc = df_fma(pc, x2, DF(-0.5f, 0.0f));
  *c = df_fma(pc, x2, DF(1.0f, 0.0f));
}

// sin and cos of x for |x| <= 1/32: Taylor series of sin to x^9 and of cos
// to x^10 (the omitted terms are below 2^-56 there); the interaction phases
// of real-time steps are this small.
__device__ __forceinline__ void df_sincos_tiny(DF x, DF* s, DF* c) {
  const DF x2 = x * x;
  DF ps = DF(1.0 / 362880);
  ps = df_fma(ps, x2, DF(-1.0 / 5040));
  ps = df_fma(ps, x2, DF(1.0 / 120));
  ps = df_fma(ps, x2, DF(-1.0 / 6));
  ps = df_fma(ps, x2, DF(1.0f, 0.0f));
  *s = ps * x;
  DF pc = DF(-1.0 / 3628800);
  pc = df_fma(pc, x2, DF(1.0 / 40320));
  pc = df_fma(pc, x2, DF(-1.0 / 720));
  pc = df_fma(pc, x2, DF(1.0 / 24));
  pc = df_fma(pc, x2, DF(-0.5f, 0.0f));
  *c = df_fma(pc, x2, DF(1.0f, 0.0f));
}

// sin and cos of x: halve the argument until |x| <= 1/8, then double the
// angle back (sin 2a = 2 sin a cos a, cos 2a = 1 - 2 sin^2 a).  Each doubling
// at most doubles the absolute error, so arguments of the interaction
// phases of a stable time step (|x| below a few radians) keep ~45 bits.
// (Not inlined, as df_exp.)
static __device__ __noinline__ void df_sincos(DF x, DF* s, DF* c) {
  if (fabsf(x.hi) <= 0.03125f) {
    df_sincos_tiny(x, s, c);
    return;
  }
  const int k = df_reduction_steps(fabsf(x.hi));
  DF sn, cs;
  df_sincos_small(df_ldexp(x, -k), &sn, &cs);
  for (int i = 0; i < k; ++i) {
    const DF s2 = df_ldexp(sn * cs, 1);
    cs = DF(1.0f, 0.0f) - df_ldexp(sn * sn, 1);
    sn = s2;
  }
  *s = sn;
  *c = cs;
}

}  // namespace sgpe
