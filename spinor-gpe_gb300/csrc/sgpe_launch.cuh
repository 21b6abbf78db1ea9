// Launch configuration and size dispatch for the split-step kernels.
//
// Line lengths are compile-time: every power of two from 32 to 4096 along
// either axis is instantiated for complex64 (float) and complex128 (double).
#pragma once
#include "sgpe_kernels.cuh"

namespace sgpe {

// Points per thread E and the preferred column-tile width per precision.
// complex64: E = 16, 8 columns (64-byte row segments per column tile);
// complex128: E = 8, 4 columns (also 64-byte segments).
template <typename R> struct Tune;
template <> struct Tune<float> {
  static constexpr int E = 16, COLS = 8, ROW_THREADS = 256;
};
template <> struct Tune<double> {
  static constexpr int E = 8, COLS = 4, ROW_THREADS = 256;
};

constexpr int cmin(int a, int b) { return a < b ? a : b; }
constexpr int cmax(int a, int b) { return a > b ? a : b; }

template <typename R, int N> struct RowCfg {
  static constexpr int E = cmin(N, Tune<R>::E);
  static constexpr int T = N / E;
  // at least one warp per block, at most 16 rows
  static constexpr int ROWS = cmax(cmax(cmin(Tune<R>::ROW_THREADS / T, 16), 1), 32 / T);
  static constexpr int THREADS = T * ROWS;
  static constexpr size_t SMEM = 2ull * ROWS * (N + N / E) * sizeof(Cx<R>);
};

template <typename R, int N> struct ColCfg {
  static constexpr int E = cmin(N, Tune<R>::E);
  static constexpr int T = N / E;
  static constexpr int COLS = cmax(cmin(Tune<R>::COLS, 1024 / T), 32 / T);
  static constexpr int THREADS = T * COLS;
  static constexpr size_t SMEM = size_t(COLS) * (N + N / E + 2) * sizeof(Cx<R>);
};

inline bool size_supported(int n) {
  return n >= 32 && n <= 4096 && (n & (n - 1)) == 0;
}

// Calls F::template run<N>() for the compile-time N equal to n.
template <class F> inline cudaError_t dispatch_n(int n, F&& f) {
  switch (n) {
    case 32: return f.template run<32>();
    case 64: return f.template run<64>();
    case 128: return f.template run<128>();
    case 256: return f.template run<256>();
    case 512: return f.template run<512>();
    case 1024: return f.template run<1024>();
    case 2048: return f.template run<2048>();
    case 4096: return f.template run<4096>();
    default: return cudaErrorInvalidValue;
  }
}

template <typename R> struct RowLauncher {
  const RowArgs<R>* a;
  int ny;
  cudaStream_t s;
  template <int N> cudaError_t run() const {
    using Cfg = RowCfg<R, N>;
    if (ny % Cfg::ROWS != 0) return cudaErrorInvalidValue;
    auto k = row_kernel<R, N, Cfg::E, Cfg::ROWS>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(Cfg::SMEM));
    if (e != cudaSuccess) return e;
    k<<<ny / Cfg::ROWS, Cfg::THREADS, Cfg::SMEM, s>>>(*a);
    return cudaGetLastError();
  }
};

template <typename R> struct ColLauncher {
  const ColArgs<R>* a;
  int ny;
  cudaStream_t s;
  template <int N> cudaError_t run() const {
    using Cfg = ColCfg<R, N>;
    const int nx = a->nx;
    if (nx % Cfg::COLS != 0 || (nx / 2) % Cfg::COLS != 0) return cudaErrorInvalidValue;
    auto k = col_kernel<R, N, Cfg::E, Cfg::COLS>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(Cfg::SMEM));
    if (e != cudaSuccess) return e;
    k<<<dim3(nx / Cfg::COLS, 2), Cfg::THREADS, Cfg::SMEM, s>>>(*a);
    return cudaGetLastError();
  }
};

template <typename R> struct ColsQuery {
  int* out;
  template <int N> cudaError_t run() const {
    *out = ColCfg<R, N>::COLS;
    return cudaSuccess;
  }
};

template <typename R> cudaError_t launch_row(const RowArgs<R>& a, int nx, int ny, cudaStream_t s) {
  return dispatch_n(nx, RowLauncher<R>{&a, ny, s});
}

template <typename R> cudaError_t launch_col(const ColArgs<R>& a, int ny, cudaStream_t s) {
  return dispatch_n(ny, ColLauncher<R>{&a, ny, s});
}

// Column-tile width used for a column length ny (0 if unsupported).
template <typename R> int col_tile_width(int ny) {
  int c = 0;
  if (dispatch_n(ny, ColsQuery<R>{&c}) != cudaSuccess) return 0;
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
extern template cudaError_t launch_row<float>(const RowArgs<float>&, int, int, cudaStream_t);
extern template cudaError_t launch_row<double>(const RowArgs<double>&, int, int, cudaStream_t);
extern template cudaError_t launch_col<float>(const ColArgs<float>&, int, cudaStream_t);
extern template cudaError_t launch_col<double>(const ColArgs<double>&, int, cudaStream_t);
#endif

}  // namespace sgpe
