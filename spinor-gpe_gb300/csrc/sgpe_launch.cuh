// Launch configuration and size dispatch for the split-step kernels.
//
// Line lengths are compile-time: every power of two from 32 to 4096, and 192,
// 384 and 768, along either axis, instantiated for complex64 (float),
// complex128 (double) and double-float (DF, kernel shape 0 only).
#pragma once
#include "sgpe_kernels.cuh"

namespace sgpe {

// Points per thread E and the preferred column-tile width per precision.
// complex64: E = 16, 8 columns (64-byte row segments per column tile);
// complex128: E = 8, 4 columns (also 64-byte segments).  The complex64
// values can be overridden at compile time (-DSGPE_F32_...) for tuning sweeps.
template <typename R> struct Tune;
// ROW_MINB / COL_MINB: resident blocks per SM requested from the compiler
// (register cap); 2 makes every block of a 1024^2 pass co-resident.
#ifndef SGPE_F32_ROW_E
#define SGPE_F32_ROW_E 16
#endif
// Points per thread of the row transforms for sides >= 2048 (longer lines
// spill with larger E).
#ifndef SGPE_F32_ROW_E_LARGE
#define SGPE_F32_ROW_E_LARGE 16
#endif
#ifndef SGPE_F32_ROW_MINB_LARGE
#define SGPE_F32_ROW_MINB_LARGE 8
#endif
#ifndef SGPE_F32_ROW_THREADS
#define SGPE_F32_ROW_THREADS 128
#endif
#ifndef SGPE_F32_ROW_MINB
#define SGPE_F32_ROW_MINB 8
#endif
#ifndef SGPE_F32_COL_E
#define SGPE_F32_COL_E 16
#endif
#ifndef SGPE_F32_COLS
#define SGPE_F32_COLS 8
#endif
#ifndef SGPE_F32_COL_MINB
#define SGPE_F32_COL_MINB 2
#endif
// Sides 3 * 2^k: points per thread (a multiple of 3, so that the radix-3
// stage divides it) and the register caps of their passes.
#ifndef SGPE_F32_R3_E
#define SGPE_F32_R3_E 12
#endif
// ... for 768: 24 points per thread (768 = 24 x 8 x 4, three stages)
#ifndef SGPE_F32_R3_E_LARGE
#define SGPE_F32_R3_E_LARGE 24
#endif
#ifndef SGPE_F32_R3_COL_MINB_LARGE
#define SGPE_F32_R3_COL_MINB_LARGE 2
#endif
#ifndef SGPE_F32_R3_ROW_MINB
#define SGPE_F32_R3_ROW_MINB 4
#endif
#ifndef SGPE_F32_R3_COL_MINB
#define SGPE_F32_R3_COL_MINB 4
#endif
template <> struct Tune<float> {
  static constexpr int ROW_E = SGPE_F32_ROW_E, ROW_THREADS = SGPE_F32_ROW_THREADS, ROW_MINB = SGPE_F32_ROW_MINB;
  static constexpr int ROW_E_LARGE = SGPE_F32_ROW_E_LARGE, ROW_MINB_LARGE = SGPE_F32_ROW_MINB_LARGE;
  static constexpr int COL_E = SGPE_F32_COL_E, COLS = SGPE_F32_COLS, COL_MINB = SGPE_F32_COL_MINB;
  static constexpr int R3_E = SGPE_F32_R3_E, R3_ROW_MINB = SGPE_F32_R3_ROW_MINB, R3_COL_MINB = SGPE_F32_R3_COL_MINB;
  static constexpr int R3_E_LARGE = SGPE_F32_R3_E_LARGE, R3_COL_MINB_LARGE = SGPE_F32_R3_COL_MINB_LARGE;
  static constexpr int COL_MAX_THREADS = 1024, COL_MINB_LARGE = SGPE_F32_COL_MINB;
};
// complex128: two 256-thread row blocks (128 registers; at three the
// generic-operator row kernels spill) and two 512-thread column blocks (64
// registers) per SM; measured on GB300 at 1024^2, two column blocks against
// one: column pass 351.7 -> 346.7 us (the passes are bound by the FP64
// pipe; 256^2 unchanged).
#ifndef SGPE_F64_ROW_MINB
#define SGPE_F64_ROW_MINB 2
#endif
#ifndef SGPE_F64_COL_MINB
#define SGPE_F64_COL_MINB 2
#endif
template <> struct Tune<double> {
  static constexpr int ROW_E = 8, ROW_THREADS = 256, ROW_MINB = SGPE_F64_ROW_MINB;
  static constexpr int ROW_E_LARGE = 8, ROW_MINB_LARGE = 2;
  static constexpr int COL_E = 8, COLS = 4, COL_MINB = SGPE_F64_COL_MINB;
  static constexpr int R3_E = 12, R3_ROW_MINB = 2, R3_COL_MINB = 1;
  static constexpr int R3_E_LARGE = 12, R3_COL_MINB_LARGE = 1;
  static constexpr int COL_MAX_THREADS = 1024, COL_MINB_LARGE = 1;
};
// Double-float: a complex value is four FP32 registers, so 8 points per
// thread (12 for sides 3 * 2^k); 256-thread row blocks and 2-column tiles,
// four blocks per SM (64 registers at 1024; no row spills, 16 bytes of
// column spills).  Measured on GB300 at 1024^2: two row blocks and 4-column
// tiles with one block -> three of each: row pass 107 -> 99 us, column pass
// 75 -> 68 us; three -> four of each (later build): column pass 75.7 ->
// 73.0 us, row pass 85.3 -> 85.0 us, 2,183 -> 2,240 steps/s.
#ifndef SGPE_DF_ROW_THREADS
#define SGPE_DF_ROW_THREADS 256
#endif
#ifndef SGPE_DF_ROW_MINB
#define SGPE_DF_ROW_MINB 4
#endif
#ifndef SGPE_DF_COLS
#define SGPE_DF_COLS 2
#endif
#ifndef SGPE_DF_COL_MINB
#define SGPE_DF_COL_MINB 4
#endif
// Sides of 2048 and more: 512-thread row and column blocks, two per SM (64
// registers; no row spills, 16-20 bytes of column spills).  Measured on
// GB300 at 2048^2 against one block per SM (128 registers): row pass 394.5
// -> 328.3 us, column pass 329.1 -> 279.6 us, 440 -> 555 steps/s.
#ifndef SGPE_DF_ROW_MINB_LARGE
#define SGPE_DF_ROW_MINB_LARGE 2
#endif
#ifndef SGPE_DF_COL_MINB_LARGE
#define SGPE_DF_COL_MINB_LARGE 2
#endif
template <> struct Tune<DF> {
  static constexpr int ROW_E = 8, ROW_THREADS = SGPE_DF_ROW_THREADS, ROW_MINB = SGPE_DF_ROW_MINB;
  static constexpr int ROW_E_LARGE = 8, ROW_MINB_LARGE = SGPE_DF_ROW_MINB_LARGE;
  static constexpr int COL_E = 8, COLS = SGPE_DF_COLS, COL_MINB = SGPE_DF_COL_MINB;
  static constexpr int R3_E = 12, R3_ROW_MINB = 2, R3_COL_MINB = SGPE_DF_COL_MINB;
  static constexpr int R3_E_LARGE = 12, R3_COL_MINB_LARGE = SGPE_DF_COL_MINB;
  static constexpr int COL_MAX_THREADS = 512, COL_MINB_LARGE = SGPE_DF_COL_MINB_LARGE;
};

constexpr int cmin(int a, int b) { return a < b ? a : b; }
constexpr int cmax(int a, int b) { return a > b ? a : b; }

// Points per thread: the tuned E for powers of two; Tune::R3_E (R3_E_LARGE
// from 768) for N = 3 * 2^k, multiples of 3 dividing N.
template <typename R> constexpr int pick_e(int n, int e_pow2) {
  return (n % 3 == 0) ? (n >= 768 ? Tune<R>::R3_E_LARGE : Tune<R>::R3_E) : cmin(n, e_pow2);
}

// Kernel shapes.  A pass over lines of one length can run in several
// shapes: launch configurations that differ in points per thread E (and so in
// the radix plan and the twiddle tables) and in lines per block.  Shape 0 is
// the configuration chosen by Tune above; the others (ShapeTune) take fewer
// points per thread or fewer lines per block for power-of-two sides up to
// 512, which gives small grids more warps and blocks per SM for more
// transform stages, 32 points per thread for complex64 rows of 1024, and the
// other multiple of 3 for sides 3 * 2^k.  Every shape computes the same
// transform; the rounding differs with the radix plan.  A plan picks one
// shape per axis (built-in defaults measured on GB300, or its autotuner).
constexpr int kMaxShapes = 3;
constexpr bool is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }
template <typename R> struct ShapeTune;
template <> struct ShapeTune<float> {
  // rows: 8 / 4 points per thread up to 512; at 1024 one alternative with
  // 32 points per thread (two radix-32 stages, warp-synchronous lines,
  // 128 registers); sides 3 * 2^k: the other multiple of 3 (12 <-> 24)
  static constexpr int r3_alt(int n) { return n >= 768 ? 12 : 24; }
  static constexpr int row_shapes(int n) {
    return n % 3 == 0 ? 2 : !is_pow2(n) ? 1 : n <= 512 ? 3 : n == 1024 ? 2 : 1;
  }
  static constexpr int col_shapes(int n) { return n % 3 == 0 ? 2 : (is_pow2(n) && n <= 512) ? 3 : 1; }
  static constexpr int row_e(int n, int s) { return n % 3 == 0 ? r3_alt(n) : n == 1024 ? 32 : s == 1 ? 8 : 4; }
  static constexpr int row_minb(int n, int) { return n == 1024 ? 4 : 0; }  // 0: the shape-0 rule
  static constexpr int row_threads(int, int) { return Tune<float>::ROW_THREADS; }
  static constexpr int col_e(int n, int) { return n % 3 == 0 ? r3_alt(n) : 8; }
  static constexpr int cols(int n, int s) { return (n % 3 != 0 && s == 2) ? 4 : Tune<float>::COLS; }
};
// complex128: 4 points per thread up to 512; shape 2 also halves the lines
// per block (128-thread row blocks, 2-column tiles of 32-byte row segments),
// so that grids of up to 256^2 give every SM a block of FP64 butterflies
template <> struct ShapeTune<double> {
  static constexpr int row_shapes(int n) { return (is_pow2(n) && n <= 512) ? 3 : 1; }
  static constexpr int col_shapes(int n) { return (is_pow2(n) && n <= 512) ? 3 : 1; }
  static constexpr int row_e(int, int) { return 4; }
  static constexpr int row_minb(int, int) { return 0; }
  static constexpr int row_threads(int, int s) { return s == 2 ? 128 : Tune<double>::ROW_THREADS; }
  static constexpr int col_e(int, int) { return 4; }
  static constexpr int cols(int, int s) { return s == 2 ? 2 : Tune<double>::COLS; }
};
// double-float: kernel shape 0 only
template <> struct ShapeTune<DF> {
  static constexpr int row_shapes(int) { return 1; }
  static constexpr int col_shapes(int) { return 1; }
  static constexpr int row_e(int, int) { return 8; }
  static constexpr int row_minb(int, int) { return 0; }
  static constexpr int row_threads(int, int) { return Tune<DF>::ROW_THREADS; }
  static constexpr int col_e(int, int) { return 8; }
  static constexpr int cols(int, int) { return Tune<DF>::COLS; }
};
template <typename R> constexpr int row_shape_count(int n) { return ShapeTune<R>::row_shapes(n); }
template <typename R> constexpr int col_shape_count(int n) { return ShapeTune<R>::col_shapes(n); }

template <typename R, int N, int S = 0> struct RowCfg {
  static constexpr bool VALID = S < row_shape_count<R>(N);
  static constexpr int E = S == 0 ? pick_e<R>(N, N >= 2048 ? Tune<R>::ROW_E_LARGE : Tune<R>::ROW_E)
                                  : cmin(N, ShapeTune<R>::row_e(N, S));
  static constexpr int T = N / E;
  // threads: 2 components x T per row; at least one warp, at most 16 rows
  static constexpr int RT = S == 0 ? Tune<R>::ROW_THREADS : ShapeTune<R>::row_threads(N, S);
  static constexpr int ROWS = cmax(cmax(cmin(RT / (2 * T), 16), 1), 32 / (2 * T));
  static constexpr int THREADS = 2 * T * ROWS;
  static constexpr size_t SMEM = 2ull * ROWS * (N + N / E) * sizeof(Cx<R>);
  static constexpr int MINB_RULE =
      (S > 0 && ShapeTune<R>::row_minb(N, S) > 0)
          ? ShapeTune<R>::row_minb(N, S)
          : (N % 3 == 0 ? Tune<R>::R3_ROW_MINB : N >= 2048 ? Tune<R>::ROW_MINB_LARGE : Tune<R>::ROW_MINB);
  static constexpr int MINB = cmax(1, cmin(MINB_RULE, 1024 / THREADS));
};

template <typename R, int N, int S = 0> struct ColCfg {
  static constexpr bool VALID = S < col_shape_count<R>(N);
  static constexpr int E = S == 0 ? pick_e<R>(N, Tune<R>::COL_E) : cmin(N, ShapeTune<R>::col_e(N, S));
  static constexpr int T = N / E;
  static constexpr int COLS =
      cmax(cmin(S == 0 ? Tune<R>::COLS : ShapeTune<R>::cols(N, S), Tune<R>::COL_MAX_THREADS / T), 32 / T);
  static constexpr int THREADS = T * COLS;
  static constexpr size_t SMEM = size_t(COLS) * (N + N / E + 2) * sizeof(Cx<R>);
  static constexpr int MINB = cmax(
      1, cmin(N % 3 == 0 ? (N >= 768 ? Tune<R>::R3_COL_MINB_LARGE : Tune<R>::R3_COL_MINB)
                         : (N >= 2048 ? Tune<R>::COL_MINB_LARGE : Tune<R>::COL_MINB),
              1024 / THREADS));
};

// Supported line lengths: powers of two 32..4096 and 3 * 2^k for 192, 384, 768.
inline bool size_supported(int n) {
  if (n == 192 || n == 384 || n == 768) return true;
  return n >= 32 && n <= 4096 && (n & (n - 1)) == 0;
}

// Calls F::template run<N>() for the compile-time N equal to n.
template <class F> inline cudaError_t dispatch_n(int n, F&& f) {
  switch (n) {
    case 32: return f.template run<32>();
    case 64: return f.template run<64>();
    case 128: return f.template run<128>();
    case 192: return f.template run<192>();
    case 384: return f.template run<384>();
    case 768: return f.template run<768>();
    case 256: return f.template run<256>();
    case 512: return f.template run<512>();
    case 1024: return f.template run<1024>();
    case 2048: return f.template run<2048>();
    case 4096: return f.template run<4096>();
    default: return cudaErrorInvalidValue;
  }
}

// Raise a kernel's dynamic shared-memory limit once per device (the first
// launch on that device); later launches skip the driver call.
template <class K> inline cudaError_t smem_limit_once(K kernel, size_t bytes, unsigned long long* done_mask) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const unsigned long long bit = 1ull << (dev & 63);
  if (*done_mask & bit) return cudaSuccess;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes));
  if (e == cudaSuccess) *done_mask |= bit;
  return e;
}

// Launch with programmatic stream serialisation (see SGPE_PDL), so the
// kernel may be scheduled while its predecessor drains.
template <class K, class A>
inline cudaError_t launch_pdl(K kernel, dim3 grid, dim3 block, size_t smem, cudaStream_t s, const A& args) {
#if SGPE_PDL
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, args);
#else
  kernel<<<grid, block, smem, s>>>(args);
  return cudaGetLastError();
#endif
}

// Resident row blocks per SM requested for a kernel: the configuration's,
// except for the double-float rows with generic operator fields, whose
// point-wise code needs more registers (at the separable kernels' 64 they
// spill 200+ bytes): three blocks below 2048, one from 2048.
template <typename R, bool SEP, int N> constexpr int row_minb(int cfg_minb) {
  if constexpr (is_df<R>::value && !SEP) return cmin(cfg_minb, N >= 2048 ? 1 : 3);
  return cfg_minb;
}

template <typename R, bool SEP, int S> struct RowLauncher {
  const RowArgs<R>* a;
  int ny;
  cudaStream_t s;
  template <int N> cudaError_t run() const {
    using Cfg = RowCfg<R, N, S>;
    if constexpr (!Cfg::VALID) {
      return cudaErrorInvalidValue;
    } else {
      if (ny % Cfg::ROWS != 0) return cudaErrorInvalidValue;
      auto k = row_kernel<R, N, Cfg::E, Cfg::ROWS, row_minb<R, SEP, N>(Cfg::MINB), SEP>;
      static unsigned long long done = 0;
      cudaError_t e = smem_limit_once(k, Cfg::SMEM, &done);
      if (e != cudaSuccess) return e;
      return launch_pdl(k, dim3(ny / Cfg::ROWS), dim3(Cfg::THREADS), Cfg::SMEM, s, *a);
    }
  }
};

template <typename R, int S> struct ColLauncher {
  const ColArgs<R>* a;
  int ny;
  cudaStream_t s;
  template <int N> cudaError_t run() const {
    using Cfg = ColCfg<R, N, S>;
    if constexpr (!Cfg::VALID) {
      return cudaErrorInvalidValue;
    } else {
      const int nx = a->nx;
      if (nx % Cfg::COLS != 0 || (nx / 2) % Cfg::COLS != 0) return cudaErrorInvalidValue;
      auto k = col_kernel<R, N, Cfg::E, Cfg::COLS, Cfg::MINB>;
      static unsigned long long done = 0;
      cudaError_t e = smem_limit_once(k, Cfg::SMEM, &done);
      if (e != cudaSuccess) return e;
      return launch_pdl(k, dim3(nx / Cfg::COLS, 2), dim3(Cfg::THREADS), Cfg::SMEM, s, *a);
    }
  }
};

// Double-float kernels are heavy to compile: the kernels of each size are
// launched through the function templates below, which are defined only in
// the sgpe_df_k*.cu translation units (SGPE_DF_KERNELS) and explicitly
// instantiated there, a few sizes per unit, so the build compiles them in
// parallel; every other unit sees only their declarations.
template <bool SEP, int N> cudaError_t launch_df_row_n(const RowArgs<DF>& a, int ny, cudaStream_t s);
template <int N> cudaError_t launch_df_col_n(const ColArgs<DF>& a, int ny, cudaStream_t s);
#ifdef SGPE_DF_KERNELS
template <bool SEP, int N> cudaError_t launch_df_row_n(const RowArgs<DF>& a, int ny, cudaStream_t s) {
  return RowLauncher<DF, SEP, 0>{&a, ny, s}.template run<N>();
}
template <int N> cudaError_t launch_df_col_n(const ColArgs<DF>& a, int ny, cudaStream_t s) {
  return ColLauncher<DF, 0>{&a, ny, s}.template run<N>();
}
#endif
template <bool SEP> struct DfRowDispatch {
  const RowArgs<DF>* a;
  int ny;
  cudaStream_t s;
  template <int N> cudaError_t run() const { return launch_df_row_n<SEP, N>(*a, ny, s); }
};
struct DfColDispatch {
  const ColArgs<DF>* a;
  int ny;
  cudaStream_t s;
  template <int N> cudaError_t run() const { return launch_df_col_n<N>(*a, ny, s); }
};

// Tensor-core DFT16 variant (complex64; sides with radix-16 stages:
// 64, 256, 1024, 2048).  Rows: the row configuration with a 128-register
// cap; columns: 4 columns per block (at least one warp), so the staging
// tiles of every warp fit in shared memory at 2048.
#ifndef SGPE_TC_ROW_MINB
#define SGPE_TC_ROW_MINB 3
#endif
#ifndef SGPE_TC_COL_MINB
#define SGPE_TC_COL_MINB 2
#endif
inline bool tc_size_supported(int n) { return n == 64 || n == 256 || n == 1024 || n == 2048; }

template <int N> struct RowTcCfg {
  using B = RowCfg<float, N>;
  static constexpr int E = B::E, ROWS = B::ROWS, THREADS = B::THREADS;
  static constexpr int MINB = cmax(1, cmin(SGPE_TC_ROW_MINB, 1024 / THREADS));
  static constexpr size_t SMEM = ((B::SMEM + 15) & ~size_t(15)) + sizeof(uint32_t) * kTcBfragWords +
                                 size_t(THREADS / 32) * kTcScratchFloats * sizeof(float);
};

template <int N> struct ColTcCfg {
  static constexpr int E = pick_e<float>(N, Tune<float>::COL_E);
  static constexpr int T = N / E;
  static constexpr int COLS = cmax(4, 32 / T);
  static constexpr int THREADS = T * COLS;
  static constexpr int MINB = cmax(1, cmin(SGPE_TC_COL_MINB, 1024 / THREADS));
  static constexpr size_t XBYTES = size_t(COLS) * (N + N / E + 2) * sizeof(float2);
  static constexpr size_t SMEM = ((XBYTES + 15) & ~size_t(15)) + sizeof(uint32_t) * kTcBfragWords +
                                 size_t(THREADS / 32) * kTcScratchFloats * sizeof(float);
};

template <class F> inline cudaError_t dispatch_tc(int n, F&& f) {
  switch (n) {
    case 64: return f.template run<64>();
    case 256: return f.template run<256>();
    case 1024: return f.template run<1024>();
    case 2048: return f.template run<2048>();
    default: return cudaErrorInvalidValue;
  }
}

struct RowTcLauncher {
  const RowArgs<float>* a;
  int ny;
  cudaStream_t s;
  template <int N> cudaError_t run() const {
    using Cfg = RowTcCfg<N>;
    if (ny % Cfg::ROWS != 0) return cudaErrorInvalidValue;
    auto k = row_kernel<float, N, Cfg::E, Cfg::ROWS, Cfg::MINB, true, true>;
    static unsigned long long done = 0;
    cudaError_t e = smem_limit_once(k, Cfg::SMEM, &done);
    if (e != cudaSuccess) return e;
    return launch_pdl(k, dim3(ny / Cfg::ROWS), dim3(Cfg::THREADS), Cfg::SMEM, s, *a);
  }
};

struct ColTcLauncher {
  const ColArgs<float>* a;
  int ny;
  cudaStream_t s;
  template <int N> cudaError_t run() const {
    using Cfg = ColTcCfg<N>;
    const int nx = a->nx;
    if (nx % Cfg::COLS != 0 || (nx / 2) % Cfg::COLS != 0) return cudaErrorInvalidValue;
    auto k = col_kernel<float, N, Cfg::E, Cfg::COLS, Cfg::MINB, true>;
    static unsigned long long done = 0;
    cudaError_t e = smem_limit_once(k, Cfg::SMEM, &done);
    if (e != cudaSuccess) return e;
    return launch_pdl(k, dim3(nx / Cfg::COLS, 2), dim3(Cfg::THREADS), Cfg::SMEM, s, *a);
  }
};

cudaError_t launch_row_tc(const RowArgs<float>& a, int nx, int ny, cudaStream_t s);  // sgpe_tc_f32.cu
cudaError_t launch_col_tc(const ColArgs<float>& a, int ny, cudaStream_t s);
inline cudaError_t launch_row_tc(const RowArgs<double>&, int, int, cudaStream_t) { return cudaErrorInvalidValue; }
inline cudaError_t launch_col_tc(const ColArgs<double>&, int, cudaStream_t) { return cudaErrorInvalidValue; }
inline cudaError_t launch_row_tc(const RowArgs<DF>&, int, int, cudaStream_t) { return cudaErrorInvalidValue; }
inline cudaError_t launch_col_tc(const ColArgs<DF>&, int, cudaStream_t) { return cudaErrorInvalidValue; }

struct ColTcColsQuery {
  int* out;
  template <int N> cudaError_t run() const {
    *out = ColTcCfg<N>::COLS;
    return cudaSuccess;
  }
};
// Column-tile width of the tensor-core column kernels (0 if unsupported).
inline int tc_col_tile_width(int ny) {
  int c = 0;
  if (dispatch_tc(ny, ColTcColsQuery{&c}) != cudaSuccess) return 0;
  return c;
}

// Grouped launches: G solves of the same size in one launch, per-solve
// arguments in device memory (blockIdx.y / blockIdx.z selects the solve).
template <typename R, bool SEP, int S> struct RowGroupedLauncher {
  const RowArgs<R>* args;
  int groups, ny;
  cudaStream_t s;
  template <int N> cudaError_t run() const {
    using Cfg = RowCfg<R, N, S>;
    if constexpr (!Cfg::VALID) {
      return cudaErrorInvalidValue;
    } else {
      if (ny % Cfg::ROWS != 0) return cudaErrorInvalidValue;
      auto k = row_kernel_grouped<R, N, Cfg::E, Cfg::ROWS, Cfg::MINB, SEP>;
      static unsigned long long done = 0;
      cudaError_t e = smem_limit_once(k, Cfg::SMEM, &done);
      if (e != cudaSuccess) return e;
      return launch_pdl(k, dim3(ny / Cfg::ROWS, groups), dim3(Cfg::THREADS), Cfg::SMEM, s, args);
    }
  }
};

template <typename R, int S> struct ColGroupedLauncher {
  const ColArgs<R>* args;
  int groups, nx;
  cudaStream_t s;
  template <int N> cudaError_t run() const {
    using Cfg = ColCfg<R, N, S>;
    if constexpr (!Cfg::VALID) {
      return cudaErrorInvalidValue;
    } else {
      if (nx % Cfg::COLS != 0 || (nx / 2) % Cfg::COLS != 0) return cudaErrorInvalidValue;
      auto k = col_kernel_grouped<R, N, Cfg::E, Cfg::COLS, Cfg::MINB>;
      static unsigned long long done = 0;
      cudaError_t e = smem_limit_once(k, Cfg::SMEM, &done);
      if (e != cudaSuccess) return e;
      return launch_pdl(k, dim3(nx / Cfg::COLS, 2, groups), dim3(Cfg::THREADS), Cfg::SMEM, s, args);
    }
  }
};

// Per-shape launch functions, explicitly instantiated in their own
// translation units (shape 0 with the default kernels, shapes 1-2 together).
template <typename R, bool SEP, int S> cudaError_t launch_row_ops_s(const RowArgs<R>& a, int nx, int ny, cudaStream_t s) {
  if constexpr (is_df<R>::value) return dispatch_n(nx, DfRowDispatch<SEP>{&a, ny, s});
  else return dispatch_n(nx, RowLauncher<R, SEP, S>{&a, ny, s});
}
template <typename R, int S> cudaError_t launch_col_s(const ColArgs<R>& a, int ny, cudaStream_t s) {
  if constexpr (is_df<R>::value) return dispatch_n(ny, DfColDispatch{&a, ny, s});
  else return dispatch_n(ny, ColLauncher<R, S>{&a, ny, s});
}
template <typename R, int S>
cudaError_t launch_row_grouped_s(const RowArgs<R>* args, int groups, int nx, int ny, cudaStream_t s) {
  return dispatch_n(nx, RowGroupedLauncher<R, true, S>{args, groups, ny, s});
}
template <typename R, int S>
cudaError_t launch_col_grouped_s(const ColArgs<R>* args, int groups, int nx, int ny, cudaStream_t s) {
  return dispatch_n(ny, ColGroupedLauncher<R, S>{args, groups, nx, s});
}

#define SGPE_SHAPE_SWITCH(shape, CALL0, CALL1, CALL2) \
  switch (shape) {                                   \
    case 0: return CALL0;                            \
    case 1: return CALL1;                            \
    case 2: return CALL2;                            \
    default: return cudaErrorInvalidValue;           \
  }

// Row kernels with the separable (SEP) or the generic point-wise code, in
// the shape a.shape.
template <typename R, bool SEP> cudaError_t launch_row_ops(const RowArgs<R>& a, int nx, int ny, cudaStream_t s) {
  if constexpr (is_df<R>::value) {
    return a.shape == 0 ? launch_row_ops_s<R, SEP, 0>(a, nx, ny, s) : cudaErrorInvalidValue;
  } else {
    SGPE_SHAPE_SWITCH(a.shape, (launch_row_ops_s<R, SEP, 0>(a, nx, ny, s)), (launch_row_ops_s<R, SEP, 1>(a, nx, ny, s)),
                      (launch_row_ops_s<R, SEP, 2>(a, nx, ny, s)))
  }
}

template <typename R> cudaError_t launch_col(const ColArgs<R>& a, int ny, cudaStream_t s) {
  if (a.tc) return launch_col_tc(a, ny, s);
  if constexpr (is_df<R>::value) {
    return a.shape == 0 ? launch_col_s<R, 0>(a, ny, s) : cudaErrorInvalidValue;
  } else {
    SGPE_SHAPE_SWITCH(a.shape, (launch_col_s<R, 0>(a, ny, s)), (launch_col_s<R, 1>(a, ny, s)),
                      (launch_col_s<R, 2>(a, ny, s)))
  }
}

// `args` in device memory, `groups` solves of an (ny, nx) grid, all in the
// kernel shape `shape`.
template <typename R>
cudaError_t launch_row_grouped(const RowArgs<R>* args, int shape, int groups, int nx, int ny, cudaStream_t s) {
  SGPE_SHAPE_SWITCH(shape, (launch_row_grouped_s<R, 0>(args, groups, nx, ny, s)),
                    (launch_row_grouped_s<R, 1>(args, groups, nx, ny, s)),
                    (launch_row_grouped_s<R, 2>(args, groups, nx, ny, s)))
}
template <typename R>
cudaError_t launch_col_grouped(const ColArgs<R>* args, int shape, int groups, int nx, int ny, cudaStream_t s) {
  SGPE_SHAPE_SWITCH(shape, (launch_col_grouped_s<R, 0>(args, groups, nx, ny, s)),
                    (launch_col_grouped_s<R, 1>(args, groups, nx, ny, s)),
                    (launch_col_grouped_s<R, 2>(args, groups, nx, ny, s)))
}

// Per-shape geometry queries (0 if the size or shape is unsupported).
template <typename R, int S> struct ShapeQuery {
  int* row_e;
  int* col_e;
  int* cols;
  template <int N> cudaError_t run() const {
    if constexpr (RowCfg<R, N, S>::VALID) *row_e = RowCfg<R, N, S>::E;
    if constexpr (ColCfg<R, N, S>::VALID) {
      *col_e = ColCfg<R, N, S>::E;
      *cols = ColCfg<R, N, S>::COLS;
    }
    return cudaSuccess;
  }
};
template <typename R> void shape_geometry(int n, int shape, int* row_e, int* col_e, int* cols) {
  *row_e = *col_e = *cols = 0;
  switch (shape) {
    case 0: dispatch_n(n, ShapeQuery<R, 0>{row_e, col_e, cols}); break;
    case 1: dispatch_n(n, ShapeQuery<R, 1>{row_e, col_e, cols}); break;
    case 2: dispatch_n(n, ShapeQuery<R, 2>{row_e, col_e, cols}); break;
    default: break;
  }
}
// Points per thread of the row (x) and column (y) transforms.
template <typename R> int row_points_per_thread(int nx, int shape = 0) {
  int re, ce, c;
  shape_geometry<R>(nx, shape, &re, &ce, &c);
  return re;
}
template <typename R> int col_points_per_thread(int ny, int shape = 0) {
  int re, ce, c;
  shape_geometry<R>(ny, shape, &re, &ce, &c);
  return ce;
}
// Column-tile width used for a column length ny.
template <typename R> int col_tile_width(int ny, int shape = 0) {
  int re, ce, c;
  shape_geometry<R>(ny, shape, &re, &ce, &c);
  return c;
}

template <typename R> cudaError_t launch_scale(const ScaleArgs<R>& a, cudaStream_t s) {
  long long blocks = (a.n + 255) / 256;
  if (blocks > 4 * 152) blocks = 4 * 152;
  if (blocks < 1) blocks = 1;
  scale_kernel<R><<<int(blocks), 256, 0, s>>>(a);
  return cudaGetLastError();
}

template <typename R> cudaError_t launch_copy(const CopyArgs<R>& a, cudaStream_t s) {
  long long n = (long long)a.nx * a.ny;
  long long blocks = (n + 255) / 256;
  if (blocks > 8 * 152) blocks = 8 * 152;
  if (blocks < 1) blocks = 1;
  copy_kernel<R><<<int(blocks), 256, 0, s>>>(a);
  return cudaGetLastError();
}

// The kernels are instantiated in separate translation units (one per
// precision and pass) so the build compiles them in parallel.
#ifndef SGPE_INSTANTIATE
#define SGPE_EXTERN_SHAPE(R, S)                                                                                  \
  extern template cudaError_t launch_row_ops_s<R, true, S>(const RowArgs<R>&, int, int, cudaStream_t);            \
  extern template cudaError_t launch_row_ops_s<R, false, S>(const RowArgs<R>&, int, int, cudaStream_t);           \
  extern template cudaError_t launch_col_s<R, S>(const ColArgs<R>&, int, cudaStream_t);                           \
  extern template cudaError_t launch_row_grouped_s<R, S>(const RowArgs<R>*, int, int, int, cudaStream_t);         \
  extern template cudaError_t launch_col_grouped_s<R, S>(const ColArgs<R>*, int, int, int, cudaStream_t);
SGPE_EXTERN_SHAPE(float, 0)
SGPE_EXTERN_SHAPE(float, 1)
SGPE_EXTERN_SHAPE(float, 2)
SGPE_EXTERN_SHAPE(double, 0)
SGPE_EXTERN_SHAPE(double, 1)
SGPE_EXTERN_SHAPE(double, 2)
#undef SGPE_EXTERN_SHAPE
extern template cudaError_t launch_row_ops_s<DF, true, 0>(const RowArgs<DF>&, int, int, cudaStream_t);
extern template cudaError_t launch_row_ops_s<DF, false, 0>(const RowArgs<DF>&, int, int, cudaStream_t);
extern template cudaError_t launch_col_s<DF, 0>(const ColArgs<DF>&, int, cudaStream_t);
#endif

// Row pass: the separable kernels unless the step uses generic operator
// fields (the transform-only modes take the separable kernels, which do
// not read the operators).
template <typename R> cudaError_t launch_row(const RowArgs<R>& a, int nx, int ny, cudaStream_t s) {
  if (a.tc) {
    if (a.mode == kRowStep && !a.op.sep) return cudaErrorInvalidValue;  // not instantiated
    return launch_row_tc(a, nx, ny, s);
  }
  if (a.mode == kRowStep && !a.op.sep) return launch_row_ops<R, false>(a, nx, ny, s);
  return launch_row_ops<R, true>(a, nx, ny, s);
}

}  // namespace sgpe
