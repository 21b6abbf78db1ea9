// Register/shared-memory FFT engine for the split-step solver (sm_103a).
//
// A line of N complex points is held by T = N/E threads, E points each.
// Thread j holds the points at positions j + m*T (m = 0..E-1) both before
// and after a transform: the Stockham autosort stages below are arranged so
// that the first stage reads straight from registers and the last stage
// writes straight back to registers, with (stages - 1) exchanges through
// shared memory in between.  Loads and stores of a line are therefore
// coalesced (consecutive threads hold consecutive points for each m) and the
// output is in natural order, which lets a kernel apply point-wise operators
// between an inverse and a forward transform without any reordering.
//
// Stage s has radix R_s (E, E, ..., remainder; for N = 3 * 2^k power-of-two
// radices then 3, see stage_radix) and sub-length Ns = prod of the earlier
// radices.  A thread runs Q = E/R_s butterflies per stage on the
// "virtual threads" vt = j + q*T; inputs are at vt + r*N/R, twiddle
// W_N^{(vt mod Ns) * r * N/(Ns*R)}, outputs at (vt/Ns)*Ns*R + vt mod Ns + r*Ns.
//
// Twiddles come from per-stage tables computed in FP64 on the host and rounded
// once to the working precision: stage (NS, R) uses
//   T[(r - 1) * NS + k] = exp(-2 pi i k r / (NS R)),  r = 1..R-1, k = 0..NS-1,
// after the blocks of the earlier stages (tw_offset).  For a fixed r,
// threads with consecutive k read consecutive entries, so a warp's twiddle
// loads are coalesced.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

// Complex64 twiddles stored as head + tail (float4: hi.x, hi.y, lo.x, lo.y,
// lo = the FP32 rounding of the FP64 remainder), applied as a*hi + a*lo: the
// table values then carry ~48 bits instead of 24, which removes the
// systematic (same every step) error of rounded twiddles.  (1) on, (0) off.
#ifndef SGPE_TW_COMP
#define SGPE_TW_COMP 0
#endif

// Twiddles of a stage whose butterflies sit at j + qT with NS = TQ: one row
// of table loads and constant roots (1), or a table load per twiddle (0).
// Off: the product of two rounded factors made the complex64 error after
// 10^4 steps 35-55% larger for a 1-3% shorter step.
#ifndef SGPE_TW_FACTOR
#define SGPE_TW_FACTOR 0
#endif

#include <type_traits>

#include "sgpe_df.cuh"
#include "sgpe_tc.cuh"

namespace sgpe {

// Complex element type of each precision: complex64 (float2), complex128
// (double2) and double-float (DFC, FP32 head + tail pairs).
template <typename R> struct CxT;
template <> struct CxT<float> { using type = float2; };
template <> struct CxT<double> { using type = double2; };
template <> struct CxT<DF> { using type = DFC; };
template <typename R> using Cx = typename CxT<R>::type;

// conversion between a storage complex type CS and a compute type C
template <class C, class CS> __device__ __forceinline__ C to_compute(CS z) {
  if constexpr (std::is_same<C, CS>::value) return z;
  else return to_dfc(z);
}
template <class CS, class C> __device__ __forceinline__ CS to_storage(C z) {
  if constexpr (std::is_same<C, CS>::value) return z;
  else return from_dfc(z);
}

// Element type of the twiddle tables (see SGPE_TW_COMP): double-float
// transforms read FP32 head + tail entries (hi.x, hi.y, lo.x, lo.y).
template <typename R> struct TwT { using type = Cx<R>; };
#if SGPE_TW_COMP
template <> struct TwT<float> { using type = float4; };
#endif
template <> struct TwT<DF> { using type = float4; };
template <typename R> using TwE = typename TwT<R>::type;

__device__ __forceinline__ float fmadd(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fmadd(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ DF fmadd(DF a, DF b, DF c) { return df_fma(a, b, c); }

// v or -v for DIR > 0 or DIR < 0 (exact; the same bits as (+-1) * v)
template <int DIR, class T> __device__ __forceinline__ T sgn(T v) { return DIR < 0 ? -v : v; }

template <class C> __device__ __forceinline__ C cmake(decltype(C::x) a, decltype(C::x) b) {
  C r; r.x = a; r.y = b; return r;
}
template <class C> __device__ __forceinline__ C cadd(C a, C b) { return cmake<C>(a.x + b.x, a.y + b.y); }
template <class C> __device__ __forceinline__ C csub(C a, C b) { return cmake<C>(a.x - b.x, a.y - b.y); }
template <class C> __device__ __forceinline__ C cmul(C a, C b) {
  return cmake<C>(fmadd(a.x, b.x, -a.y * b.y), fmadd(a.x, b.y, a.y * b.x));
}
// a * conj(b)
template <class C> __device__ __forceinline__ C cmulc(C a, C b) {
  return cmake<C>(fmadd(a.x, b.x, a.y * b.y), fmadd(a.y, b.x, -a.x * b.y));
}
// Double-float butterflies: sums without renormalisation (df_add_lazy),
// each value renormalised once at the end of its transform stage
// (fft_stage).  (1) on, (0) renormalise every sum.
#ifndef SGPE_DF_LAZY
#define SGPE_DF_LAZY 1
#endif
#if SGPE_DF_LAZY
template <> __device__ __forceinline__ DFC cadd<DFC>(DFC a, DFC b) {
  return DFC{df_add_lazy(a.x, b.x), df_add_lazy(a.y, b.y)};
}
template <> __device__ __forceinline__ DFC csub<DFC>(DFC a, DFC b) {
  return DFC{df_add_lazy(a.x, -b.x), df_add_lazy(a.y, -b.y)};
}
#endif
template <class C> __device__ __forceinline__ void renorm(C&) {}
template <> __device__ __forceinline__ void renorm<DFC>(DFC& a) {
  if (SGPE_DF_LAZY) {
    a.x = df_renorm(a.x);
    a.y = df_renorm(a.y);
  }
}

// double-float complex products: each part one two-product dot (df_dot2)
template <> __device__ __forceinline__ DFC cmul<DFC>(DFC a, DFC b) {
  return DFC{df_dot2<-1>(a.x, b.x, a.y, b.y), df_dot2<1>(a.x, b.y, a.y, b.x)};
}
template <> __device__ __forceinline__ DFC cmulc<DFC>(DFC a, DFC b) {
  return DFC{df_dot2<1>(a.x, b.x, a.y, b.y), df_dot2<-1>(a.y, b.x, a.x, b.y)};
}
template <class C> __device__ __forceinline__ C cscale(C a, decltype(C::x) s) { return cmake<C>(a.x * s, a.y * s); }

// a * w (DIR < 0) or a * conj(w) (DIR > 0) for a twiddle-table entry: a
// complex value, or a head + tail pair (float4) multiplied as a*hi + a*lo.
template <int DIR, class C> __device__ __forceinline__ C tw_mul(C a, C w) {
  return DIR < 0 ? cmul(a, w) : cmulc(a, w);
}
template <int DIR> __device__ __forceinline__ float2 tw_mul(float2 a, float4 w) {
  if (DIR < 0) {
    const float tr = fmadd(a.x, w.z, -a.y * w.w), ti = fmadd(a.x, w.w, a.y * w.z);
    return make_float2(fmadd(a.x, w.x, fmadd(-a.y, w.y, tr)), fmadd(a.x, w.y, fmadd(a.y, w.x, ti)));
  }
  const float tr = fmadd(a.x, w.z, a.y * w.w), ti = fmadd(a.y, w.z, -a.x * w.w);
  return make_float2(fmadd(a.x, w.x, fmadd(a.y, w.y, tr)), fmadd(a.y, w.x, fmadd(-a.x, w.y, ti)));
}
// double-float values times a head + tail table entry (hi.x, hi.y, lo.x, lo.y)
template <int DIR> __device__ __forceinline__ DFC tw_mul(DFC a, float4 w) {
  const DFC wc{DF(w.x, w.z), DF(w.y, w.w)};
  return DIR < 0 ? cmul(a, wc) : cmulc(a, wc);
}
template <class C> __device__ __forceinline__ decltype(C::x) cabs2(C a) { return fmadd(a.x, a.x, a.y * a.y); }
// a * (DIR * i): DIR = -1 gives a * (-i), DIR = +1 gives a * i
template <int DIR, class C> __device__ __forceinline__ C crot(C a) {
  return DIR < 0 ? cmake<C>(a.y, -a.x) : cmake<C>(-a.y, a.x);
}
// multiply by the twiddle factor exp(DIR * 2 pi i m / 16), m a compile-time constant
template <int DIR, int M, class C> __device__ __forceinline__ C tw16(C a) {
  using R = decltype(C::x);
  constexpr int m = M & 15;
  const R c1 = R(0.92387953251128675613);  // cos(pi/8)
  const R s1 = R(0.38268343236508977173);  // sin(pi/8)
  const R h = R(0.70710678118654752440);   // sqrt(1/2)
  // products with DIR = +-1 are written as sign changes (same bits)
  if constexpr (m == 0) return a;
  else if constexpr (m == 4) return crot<DIR>(a);
  else if constexpr (m == 8) return cmake<C>(-a.x, -a.y);
  else if constexpr (m == 12) return crot<-DIR>(a);
  else if constexpr (m == 2) return cscale(cmake<C>(a.x - sgn<DIR>(a.y), a.y + sgn<DIR>(a.x)), h);
  else if constexpr (m == 6) return cscale(cmake<C>(-a.x - sgn<DIR>(a.y), sgn<DIR>(a.x) - a.y), h);
  else if constexpr (m == 1) return cmul(a, cmake<C>(c1, sgn<DIR>(s1)));
  else if constexpr (m == 3) return cmul(a, cmake<C>(s1, sgn<DIR>(c1)));
  else if constexpr (m == 9) return cmul(a, cmake<C>(-c1, sgn<-DIR>(s1)));
  else if constexpr (m == 5) return crot<DIR>(cmul(a, cmake<C>(c1, sgn<DIR>(s1))));  // W^4 W^1
  else if constexpr (m == 7) return crot<DIR>(cmul(a, cmake<C>(s1, sgn<DIR>(c1))));  // W^4 W^3
  else return crot<DIR>(tw16<DIR, m - 4>(a));                                   // 10, 11, 13, 14, 15
}

// The same with the exponent known only after unrolling (the switch folds).
template <int DIR, class C> __device__ __forceinline__ C tw16r(C a, int m) {
  switch (m & 15) {
    case 0: return a;
    case 1: return tw16<DIR, 1>(a);
    case 2: return tw16<DIR, 2>(a);
    case 3: return tw16<DIR, 3>(a);
    case 4: return tw16<DIR, 4>(a);
    case 5: return tw16<DIR, 5>(a);
    case 6: return tw16<DIR, 6>(a);
    case 7: return tw16<DIR, 7>(a);
    case 8: return tw16<DIR, 8>(a);
    case 9: return tw16<DIR, 9>(a);
    case 10: return tw16<DIR, 10>(a);
    case 11: return tw16<DIR, 11>(a);
    case 12: return tw16<DIR, 12>(a);
    case 13: return tw16<DIR, 13>(a);
    case 14: return tw16<DIR, 14>(a);
    default: return tw16<DIR, 15>(a);
  }
}

// multiply by exp(DIR * 2 pi i m / 32), m a compile-time constant
template <int DIR, int M, class C> __device__ __forceinline__ C tw32(C a) {
  using R = decltype(C::x);
  constexpr int m = M & 31;
  if constexpr (m % 2 == 0) {
    return tw16<DIR, m / 2>(a);
  } else if constexpr (m > 8) {
    return crot<DIR>(tw32<DIR, m - 8>(a));  // exp(DIR i pi/2) = DIR * i
  } else {
    const R c1 = R(0.98078528040323044913);  // cos(pi/16)
    const R s1 = R(0.19509032201612826785);  // sin(pi/16)
    const R c3 = R(0.83146961230254523708);  // cos(3 pi/16)
    const R s3 = R(0.55557023301960222474);  // sin(3 pi/16)
    if constexpr (m == 1) return cmul(a, cmake<C>(c1, sgn<DIR>(s1)));
    else if constexpr (m == 3) return cmul(a, cmake<C>(c3, sgn<DIR>(s3)));
    else if constexpr (m == 5) return cmul(a, cmake<C>(s3, sgn<DIR>(c3)));  // cos(5pi/16) = sin(3pi/16)
    else return cmul(a, cmake<C>(s1, sgn<DIR>(c1)));                        // m == 7
  }
}

// multiply by exp(DIR * 2 pi i m / 24), m a compile-time constant
template <int DIR, int M, class C> __device__ __forceinline__ C tw24(C a) {
  using R = decltype(C::x);
  constexpr int m = ((M % 24) + 24) % 24;
  if constexpr (m == 0) {
    return a;
  } else if constexpr (m >= 6) {
    return crot<DIR>(tw24<DIR, m - 6>(a));  // exp(DIR i pi/2) = DIR * i
  } else {
    // cos and sin of pi m / 12, m = 1..5
    constexpr double kc[6] = {1.0, 0.96592582628906828675, 0.86602540378443864676, 0.70710678118654752440, 0.5,
                              0.25881904510252076235};
    return cmul(a, cmake<C>(R(kc[m]), sgn<DIR>(R(kc[6 - m]))));  // sin(pi m/12) = cos(pi (6-m)/12)
  }
}
// The same with the exponent known only after unrolling (the switch folds).
template <int DIR, class C> __device__ __forceinline__ C tw24r(C a, int m) {
  switch (((m % 24) + 24) % 24) {
    case 0: return a;
    case 1: return tw24<DIR, 1>(a);
    case 2: return tw24<DIR, 2>(a);
    case 3: return tw24<DIR, 3>(a);
    case 4: return tw24<DIR, 4>(a);
    case 5: return tw24<DIR, 5>(a);
    case 6: return tw24<DIR, 6>(a);
    case 7: return tw24<DIR, 7>(a);
    case 8: return tw24<DIR, 8>(a);
    case 9: return tw24<DIR, 9>(a);
    case 10: return tw24<DIR, 10>(a);
    case 11: return tw24<DIR, 11>(a);
    case 12: return tw24<DIR, 12>(a);
    case 13: return tw24<DIR, 13>(a);
    case 14: return tw24<DIR, 14>(a);
    case 15: return tw24<DIR, 15>(a);
    case 16: return tw24<DIR, 16>(a);
    case 17: return tw24<DIR, 17>(a);
    case 18: return tw24<DIR, 18>(a);
    case 19: return tw24<DIR, 19>(a);
    case 20: return tw24<DIR, 20>(a);
    case 21: return tw24<DIR, 21>(a);
    case 22: return tw24<DIR, 22>(a);
    default: return tw24<DIR, 23>(a);
  }
}

// a * exp(-2 pi i m / E) for the points-per-thread E of the engine, m known
// after unrolling.
template <int E, class C> __device__ __forceinline__ C root_fwd(C a, int m) {
  if constexpr (E == 16) return tw16r<-1>(a, m);
  else if constexpr (E == 8) return tw16r<-1>(a, 2 * m);
  else if constexpr (E == 4) return tw16r<-1>(a, 4 * m);
  else if constexpr (E == 2) return tw16r<-1>(a, 8 * m);
  else if constexpr (E == 24) return tw24r<-1>(a, m);
  else if constexpr (E == 12) return tw24r<-1>(a, 2 * m);
  else {
    static_assert(E == 32, "no constant roots for this E");
    switch (m & 31) {
      case 0: return a;
      case 1: return tw32<-1, 1>(a);
      case 3: return tw32<-1, 3>(a);
      case 5: return tw32<-1, 5>(a);
      case 7: return tw32<-1, 7>(a);
      case 9: return tw32<-1, 9>(a);
      case 11: return tw32<-1, 11>(a);
      case 13: return tw32<-1, 13>(a);
      case 15: return tw32<-1, 15>(a);
      case 17: return tw32<-1, 17>(a);
      case 19: return tw32<-1, 19>(a);
      case 21: return tw32<-1, 21>(a);
      case 23: return tw32<-1, 23>(a);
      case 25: return tw32<-1, 25>(a);
      case 27: return tw32<-1, 27>(a);
      case 29: return tw32<-1, 29>(a);
      case 31: return tw32<-1, 31>(a);
      default: return tw16r<-1>(a, (m & 31) / 2);
    }
  }
}

// In-register DFT of size R in natural order: a[k] <- sum_n a[n] exp(DIR 2 pi i nk/R)
template <int R, int DIR> struct Dft;

template <int DIR> struct Dft<1, DIR> {
  template <class C> __device__ __forceinline__ static void run(C*) {}
};
template <int DIR> struct Dft<2, DIR> {
  template <class C> __device__ __forceinline__ static void run(C* a) {
    C t = a[0];
    a[0] = cadd(t, a[1]);
    a[1] = csub(t, a[1]);
  }
};
template <int DIR> struct Dft<3, DIR> {
  template <class C> __device__ __forceinline__ static void run(C* a) {
    using R = decltype(C::x);
    const R half = R(0.5);
    const R s3 = R(0.86602540378443864676);  // sqrt(3)/2
    const C t1 = cadd(a[1], a[2]);
    const C t2 = csub(a[1], a[2]);
    const C m = cmake<C>(a[0].x - half * t1.x, a[0].y - half * t1.y);
    // +/- i DIR sqrt(3)/2 (a1 - a2)
    const C r = crot<DIR>(cscale(t2, s3));
    a[0] = cadd(a[0], t1);
    a[1] = cadd(m, r);
    a[2] = csub(m, r);
  }
};
template <int DIR> struct Dft<4, DIR> {
  template <class C> __device__ __forceinline__ static void run(C* a) {
    C t0 = cadd(a[0], a[2]), t1 = csub(a[0], a[2]);
    C t2 = cadd(a[1], a[3]), t3 = crot<DIR>(csub(a[1], a[3]));
    a[0] = cadd(t0, t2);
    a[2] = csub(t0, t2);
    a[1] = cadd(t1, t3);
    a[3] = csub(t1, t3);
  }
};
template <int DIR> struct Dft<8, DIR> {
  template <class C> __device__ __forceinline__ static void run(C* a) {
    C e[4] = {a[0], a[2], a[4], a[6]};
    C o[4] = {a[1], a[3], a[5], a[7]};
    Dft<4, DIR>::run(e);
    Dft<4, DIR>::run(o);
    o[1] = tw16<DIR, 2>(o[1]);
    o[2] = tw16<DIR, 4>(o[2]);
    o[3] = tw16<DIR, 6>(o[3]);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      a[k] = cadd(e[k], o[k]);
      a[k + 4] = csub(e[k], o[k]);
    }
  }
};
template <int DIR> struct Dft<16, DIR> {
  template <class C> __device__ __forceinline__ static void run(C* a) {
    // n = n2 + 4 n1, k = k1 + 4 k2: inner DFT4 over n1, twiddle W16^{n2 k1},
    // outer DFT4 over n2.
    C b[16];
#pragma unroll
    for (int n2 = 0; n2 < 4; ++n2) {
      C t[4] = {a[n2], a[n2 + 4], a[n2 + 8], a[n2 + 12]};
      Dft<4, DIR>::run(t);
#pragma unroll
      for (int k1 = 0; k1 < 4; ++k1) b[4 * k1 + n2] = t[k1];
    }
    b[4 * 1 + 1] = tw16<DIR, 1>(b[4 * 1 + 1]);
    b[4 * 1 + 2] = tw16<DIR, 2>(b[4 * 1 + 2]);
    b[4 * 1 + 3] = tw16<DIR, 3>(b[4 * 1 + 3]);
    b[4 * 2 + 1] = tw16<DIR, 2>(b[4 * 2 + 1]);
    b[4 * 2 + 2] = tw16<DIR, 4>(b[4 * 2 + 2]);
    b[4 * 2 + 3] = tw16<DIR, 6>(b[4 * 2 + 3]);
    b[4 * 3 + 1] = tw16<DIR, 3>(b[4 * 3 + 1]);
    b[4 * 3 + 2] = tw16<DIR, 6>(b[4 * 3 + 2]);
    b[4 * 3 + 3] = tw16<DIR, 9>(b[4 * 3 + 3]);
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) {
      C t[4] = {b[4 * k1 + 0], b[4 * k1 + 1], b[4 * k1 + 2], b[4 * k1 + 3]};
      Dft<4, DIR>::run(t);
#pragma unroll
      for (int k2 = 0; k2 < 4; ++k2) a[k1 + 4 * k2] = t[k2];
    }
  }
};

template <int DIR> struct Dft<32, DIR> {
  template <class C> __device__ __forceinline__ static void run(C* a) {
    // decimation in time: DFT16 of the even and of the odd points, then
    // a[k] = e[k] + W32^k o[k], a[k + 16] = e[k] - W32^k o[k]
    C e[16], o[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      e[k] = a[2 * k];
      o[k] = a[2 * k + 1];
    }
    Dft<16, DIR>::run(e);
    Dft<16, DIR>::run(o);
    o[1] = tw32<DIR, 1>(o[1]);
    o[2] = tw32<DIR, 2>(o[2]);
    o[3] = tw32<DIR, 3>(o[3]);
    o[4] = tw32<DIR, 4>(o[4]);
    o[5] = tw32<DIR, 5>(o[5]);
    o[6] = tw32<DIR, 6>(o[6]);
    o[7] = tw32<DIR, 7>(o[7]);
    o[8] = tw32<DIR, 8>(o[8]);
    o[9] = tw32<DIR, 9>(o[9]);
    o[10] = tw32<DIR, 10>(o[10]);
    o[11] = tw32<DIR, 11>(o[11]);
    o[12] = tw32<DIR, 12>(o[12]);
    o[13] = tw32<DIR, 13>(o[13]);
    o[14] = tw32<DIR, 14>(o[14]);
    o[15] = tw32<DIR, 15>(o[15]);
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      a[k] = cadd(e[k], o[k]);
      a[k + 16] = csub(e[k], o[k]);
    }
  }
};

// DFT of size 3P (P = 4, 8): n = P n2 + n1, k = k1 + 3 k2; DFT3 over n2,
// twiddle W_{3P}^{n1 k1}, DFT_P over n1.
template <int P, int DIR> struct Dft3P {
  template <class C> __device__ __forceinline__ static void run(C* a) {
    constexpr int R = 3 * P;
    constexpr int U = 24 / R;  // W_R^m = W_24^{U m}
    C y[P][3];
#pragma unroll
    for (int n1 = 0; n1 < P; ++n1) {
      C t[3] = {a[n1], a[P + n1], a[2 * P + n1]};
      Dft<3, DIR>::run(t);
      y[n1][0] = t[0];
      y[n1][1] = tw24r<DIR>(t[1], U * n1);
      y[n1][2] = tw24r<DIR>(t[2], U * 2 * n1);
    }
#pragma unroll
    for (int k1 = 0; k1 < 3; ++k1) {
      C u[P];
#pragma unroll
      for (int n1 = 0; n1 < P; ++n1) u[n1] = y[n1][k1];
      Dft<P, DIR>::run(u);
#pragma unroll
      for (int k2 = 0; k2 < P; ++k2) a[k1 + 3 * k2] = u[k2];
    }
  }
};
template <int DIR> struct Dft<12, DIR> : Dft3P<4, DIR> {};
template <int DIR> struct Dft<24, DIR> : Dft3P<8, DIR> {};

// Radix of the stage with sub-length NS of an (N, E) transform.  With P the
// largest power of two dividing E: powers of two take stages of P (the
// remainder last).  N = 3 * 2^k with E a multiple of 3 dividing N (E = 24 or
// 12): the first stage has radix E (an in-register DFT 3 x P), the rest are
// powers of two, e.g. 768 = 24 x 8 x 4.  Otherwise N = 3 * 2^k takes
// power-of-two stages of at most P and one radix-3 stage last.
__host__ __device__ constexpr int stage_radix(int N, int E, int NS) {
  const int m = N / NS;
  int p = 1;
  while (E % (2 * p) == 0) p *= 2;
  if (m % 3 == 0) {
    if (E % 3 == 0 && m % E == 0) return E;
    if (m == 3) return 3;
    const int two = m / 3;
    return two < p ? two : p;
  }
  return m < p ? m : p;
}

// Offset of the twiddle block of the stage with sub-length NS in the table
// of an (N, E) transform; tw_offset(N, E, N) is the table length.
__host__ __device__ constexpr int tw_offset(int N, int E, int NS) {
  int off = 0, ns = 1;
  while (ns < NS) {
    const int r = stage_radix(N, E, ns);
    off += (r - 1) * ns;
    ns *= r;
  }
  return off;
}

// Shared-memory view used by the exchange stages: element i of line l of the
// calling thread's group lives at base[l * line_stride + i + i / E] (one pad
// element per E elements keeps the radix-E scatter free of bank conflicts).
// WARP: every line is held by threads of one warp (T divides 32), so the
// exchange between stages needs only a warp barrier.
// TC: radix-16 stages take their DFT16 on the tensor cores (split-BF16,
// sgpe_tc.cuh) with the staging area in `tc`.
// bar > 0 (and !WARP): the line's threads are whole warps, and the
// exchanges synchronise only them, on named barrier `bar` of `bar_threads`
// threads, so lines of one block do not wait for each other.
template <class C, int E, bool WARP = false, bool TC = false> struct LineSmem {
  static constexpr bool kTc = TC;
  C* base;
  int line_stride;
  TcScratch tc;
  int bar = 0;
  int bar_threads = 0;
  // padded position of element i (i >= 0)
  static __device__ __forceinline__ unsigned pad(unsigned i) { return i + i / unsigned(E); }
  __device__ __forceinline__ C* line(int l) const { return base + l * line_stride; }
  __device__ __forceinline__ C ld(int l, int i) const { return line(l)[pad(unsigned(i))]; }
  __device__ __forceinline__ void st(int l, int i, C v) const { line(l)[pad(unsigned(i))] = v; }
  __device__ __forceinline__ void sync() const {
    if constexpr (WARP) {
      __syncwarp();
    } else {
      if (bar > 0) asm volatile("bar.sync %0, %1;" ::"r"(bar), "r"(bar_threads) : "memory");
      else __syncthreads();
    }
  }
  // the same lines viewed as another complex type of the same size
  template <class C2> __device__ __forceinline__ LineSmem<C2, E, WARP, TC> retype() const {
    static_assert(sizeof(C2) == sizeof(C), "retyped lines must keep the element size");
    return LineSmem<C2, E, WARP, TC>{reinterpret_cast<C2*>(base), line_stride, tc, bar, bar_threads};
  }
};

// Compile-time address folding for the exchanges.  A stage reads element
// j + c (c = qT + r N/R) and writes element b(vt) + r NS; when the pad term
// floor(i / E) of every such element differs from that of the base (j, or
// b(vt)) by a constant for all threads, each access is the padded base plus
// a compile-time offset.  These predicates check that exhaustively over the
// threads of a line.
__host__ __device__ constexpr int pad_div(int i, int e) { return i / e; }
template <int N, int E, int R, int Q> __host__ __device__ constexpr bool loads_fold() {
  constexpr int T = N / E;
  for (int q = 0; q < Q; ++q)
    for (int r = 0; r < R; ++r) {
      const int c = q * T + r * (N / R);
      const int d = pad_div(c, E);
      for (int j = 1; j < T; ++j)
        if (pad_div(j + c, E) - pad_div(j, E) != d) return false;
    }
  return true;
}
template <int N, int E, int R, int NS> __host__ __device__ constexpr bool stores_fold() {
  for (int vt = 0; vt < N / R; ++vt) {
    const int b = (vt / NS) * NS * R + (vt % NS);
    for (int r = 1; r < R; ++r)
      if (pad_div(b + r * NS, E) - pad_div(b, E) != pad_div(r * NS, E)) return false;
  }
  return true;
}

// One Stockham stage (and, recursively, the stages after it) on L lines.
// FROM_SMEM: the first stage reads the natural-order line from shared memory
// instead of registers; TO_SMEM: the last stage writes the natural-order
// result to shared memory instead of registers.  In both cases a thread
// touches exactly the positions j + m*T it holds in the register layout, so
// no barrier is needed between a thread's own point-wise pass over those
// positions and the adjacent transform.  Those natural-order lines hold the
// storage type CS (converted from / to the compute type C at that boundary);
// the exchanges between stages hold C.
template <int N, int E, int DIR, int L, int NS, bool FROM_SMEM, bool TO_SMEM, class C, class SM, class CS = C>
__device__ __forceinline__ void fft_stage(C (&v)[L][E], int j, const SM& sm, const C* __restrict__ tw) {
  constexpr int T = N / E;
  constexpr int R = stage_radix(N, E, NS);
  constexpr int Q = E / R;
  constexpr bool kFirst = (NS == 1);
  constexpr bool kLast = (NS * R == N);
  static_assert(E % R == 0, "radix must divide the points per thread");
  C a[L][Q][R];
  constexpr bool kLdFold = loads_fold<N, E, R, Q>();
  const unsigned pj = SM::pad(unsigned(j));
#pragma unroll
  for (int l = 0; l < L; ++l)
#pragma unroll
    for (int q = 0; q < Q; ++q)
#pragma unroll
      for (int r = 0; r < R; ++r) {
        if constexpr (kFirst && !FROM_SMEM) {
          a[l][q][r] = v[l][q + r * Q];
        } else if constexpr (kFirst && !std::is_same<C, CS>::value) {
          const CS* line = reinterpret_cast<const CS*>(sm.line(l));
          a[l][q][r] = to_compute<C>(line[SM::pad(unsigned(j + q * T + r * (N / R)))]);
        } else if constexpr (kLdFold) {
          const int c = q * T + r * (N / R);
          a[l][q][r] = sm.line(l)[pj + unsigned(c + c / E)];
        } else {
          a[l][q][r] = sm.ld(l, j + q * T + r * (N / R));
        }
      }
  if constexpr (!kFirst && SGPE_TW_FACTOR && Q > 1 && T * Q == NS) {
    // The Q butterflies of the thread sit at k = j + qT with NS = TQ, so
    // W_{NS R}^{(j + qT) r} = W_{NS R}^{j r} W_E^{q r}: R - 1 table values
    // times compile-time roots of order E (instead of Q (R - 1) loads).
    constexpr int kOff = tw_offset(N, E, NS);
    static_assert(sizeof(TwE<decltype(C::x)>) == sizeof(C), "factorised twiddles need plain tables");
    C w1[R];
#pragma unroll
    for (int r = 1; r < R; ++r) w1[r] = __ldg(tw + kOff + j + (r - 1) * NS);
#pragma unroll
    for (int q = 0; q < Q; ++q)
#pragma unroll
      for (int r = 1; r < R; ++r) {
        const C w = q == 0 ? w1[r] : root_fwd<E>(w1[r], q * r);
#pragma unroll
        for (int l = 0; l < L; ++l) a[l][q][r] = (DIR < 0) ? cmul(a[l][q][r], w) : cmulc(a[l][q][r], w);
      }
  } else if constexpr (!kFirst) {
    constexpr int kOff = tw_offset(N, E, NS);
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const int vt = j + q * T;
      using W = TwE<decltype(C::x)>;
      const W* twq = reinterpret_cast<const W*>(tw) + kOff + (vt % NS);
#pragma unroll
      for (int r = 1; r < R; ++r) {
        const W w = __ldg(twq + (r - 1) * NS);
#pragma unroll
        for (int l = 0; l < L; ++l) a[l][q][r] = tw_mul<DIR>(a[l][q][r], w);
      }
    }
  }
#pragma unroll
  for (int l = 0; l < L; ++l)
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      if constexpr (SM::kTc && R == 16) tc_dft16<DIR>(a[l][q], sm.tc);
      else Dft<R, DIR>::run(a[l][q]);
#pragma unroll
      for (int r = 0; r < R; ++r) renorm(a[l][q][r]);
    }
  if constexpr (kLast && !TO_SMEM) {
#pragma unroll
    for (int l = 0; l < L; ++l)
#pragma unroll
      for (int q = 0; q < Q; ++q)
#pragma unroll
        for (int r = 0; r < R; ++r) v[l][q + r * Q] = a[l][q][r];
  } else {
    sm.sync();  // earlier readers of the exchange buffer are done
    constexpr bool kStFold = stores_fold<N, E, R, NS>();
#pragma unroll
    for (int l = 0; l < L; ++l)
#pragma unroll
      for (int q = 0; q < Q; ++q) {
        const int vt = j + q * T;
        const int base = (vt / NS) * NS * R + (vt % NS);
        if constexpr (kLast && !std::is_same<C, CS>::value) {
          CS* line = reinterpret_cast<CS*>(sm.line(l));
#pragma unroll
          for (int r = 0; r < R; ++r) line[SM::pad(unsigned(base + r * NS))] = to_storage<CS>(a[l][q][r]);
        } else if constexpr (kStFold) {
          C* sp = sm.line(l) + SM::pad(unsigned(base));
#pragma unroll
          for (int r = 0; r < R; ++r) sp[r * NS + (r * NS) / E] = a[l][q][r];
        } else {
#pragma unroll
          for (int r = 0; r < R; ++r) sm.st(l, base + r * NS, a[l][q][r]);
        }
      }
    if constexpr (!kLast) {
      sm.sync();
      fft_stage<N, E, DIR, L, NS * R, FROM_SMEM, TO_SMEM, C, SM, CS>(v, j, sm, tw);
    }
  }
}

// Transform L lines of length N held as described above.  DIR = -1 is the
// unnormalised forward DFT (exp(-2 pi i kn/N)), DIR = +1 the unnormalised
// inverse.  Every thread of the block must call this the same number of
// times (it synchronises the block between stages).  With FROM_SMEM the
// input is read from the shared-memory view (natural order; the caller must
// have synchronised after other threads wrote it, unless each thread wrote
// only its own positions); with TO_SMEM the output is left there in natural
// order and `v` is not written.
template <int N, int E, int DIR, int L, bool FROM_SMEM = false, bool TO_SMEM = false, class C, class SM>
__device__ __forceinline__ void fft_lines(C (&v)[L][E], int j, const SM& sm, const C* __restrict__ tw) {
  static_assert(N % E == 0, "N must be a multiple of E");
  fft_stage<N, E, DIR, L, 1, FROM_SMEM, TO_SMEM>(v, j, sm, tw);
}

}  // namespace sgpe
