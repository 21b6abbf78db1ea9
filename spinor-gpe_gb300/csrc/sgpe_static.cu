// Allocation-free centred 2-D transform (sgpe_fft2_static).
//
// Who needs it: callers that cannot call cudaMalloc (or anything that
// allocates device memory) at the point where they want a transform --
// hosts whose device memory is owned by their own pool allocator, which has
// taken the device's free memory and must not be bypassed; real-time loops
// that cannot afford an allocation's latency or its implicit
// synchronisation; foreign-language hosts that hold only raw device
// pointers.  sgpe_fft2 needs a plan, and creating a plan allocates; this
// entry point needs nothing but the caller's input and output buffers.
//
// Its scratch (the field between the x and y passes and the per-stage
// twiddle tables) is the file-scope array below, SGPE_FFT2_STATIC_BYTES
// (2.25 MiB) on every GPU that loads the library, held until the process
// exits.  Host code cannot use the array's name as a device address (it is a
// host-side stand-in); the device address is looked up once per device with
// cudaGetSymbolAddress, with that device current, on the first call made on
// it, and kept per device index.  The runtime API's primary context is the
// one supported: a caller that makes another driver context current, or
// resets the device, must not rely on the kept address.  That first call on a
// device should come before any stream capture is started on it.  Under
// CUDA's default lazy module loading the first launch of each kernel loads
// its module, which allocates device memory; the transform kernels of each
// (grid size, precision, direction) are separate kernels, so a caller that
// cannot allocate later makes one warm-up call per combination it will use
// (or sets CUDA_MODULE_LOADING=EAGER).
//
// All calls share the one array and leave their data in it.  Nothing in it
// has to start at zero: each call writes every element of the intermediate
// field before reading it, and writes the twiddle tables unless the previous
// call on that device had the same grid and precision (the tables are then
// already in place, in stream order).  Calls whose work overlaps on the GPU
// (different streams without ordering, or different host threads) race on
// the array; order them on one stream.
#include <atomic>
#include <cmath>
#include <mutex>
#include <string>

#include "sgpe_launch.cuh"
#include "spinor_gb300.h"

namespace sgpe_detail {
int set_error(int code, const std::string& msg);  // sgpe_api.cu
}

namespace {

static __device__ __align__(256) unsigned char g_fft2_scratch[SGPE_FFT2_STATIC_BYTES];

constexpr int kMaxDevices = 64;
std::atomic<void*> g_scratch_dev[kMaxDevices];
// Per device: the (grid, precision) whose twiddle tables the array holds
// (0: none or unknown).  g_tw_mutex orders the check-and-rebuild.
std::atomic<unsigned long long> g_tw_key[kMaxDevices];
std::mutex g_tw_mutex;

// Device address of the scratch array on the current device (set-up on the
// first call per device).
int scratch_address(int* dev_out, void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return sgpe_detail::set_error(SGPE_ERR_CUDA, std::string("fft2_static: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return sgpe_detail::set_error(SGPE_ERR_ARG, "fft2_static: device index too large");
  void* p = g_scratch_dev[dev].load(std::memory_order_acquire);
  if (p == nullptr) {
    e = cudaGetSymbolAddress(&p, g_fft2_scratch);
    if (e != cudaSuccess)
      return sgpe_detail::set_error(SGPE_ERR_CUDA, std::string("fft2_static: cudaGetSymbolAddress: ") +
                                                       cudaGetErrorString(e));
    g_scratch_dev[dev].store(p, std::memory_order_release);  // the same value from any racing thread
  }
  *dev_out = dev;
  *out = p;
  return SGPE_OK;
}

// Per-stage twiddle table of an (n, e) transform in the order the FFT engine
// reads it (sgpe_fft.cuh): stage (ns, r_s) holds exp(-2 pi i k r/(ns r_s)) at
// (r - 1) ns + k.  FP64 sincospi of the exactly reduced fraction, rounded once.
__device__ __forceinline__ void set_twiddle(float2& w, double re, double im) { w = make_float2(float(re), float(im)); }
__device__ __forceinline__ void set_twiddle(double2& w, double re, double im) { w = make_double2(re, im); }
#if SGPE_TW_COMP
__device__ __forceinline__ void set_twiddle(float4& w, double re, double im) {
  const float hr = float(re), hi = float(im);
  w = make_float4(hr, hi, float(re - double(hr)), float(im - double(hi)));
}
#endif

template <typename R>
__global__ void twiddle_kernel(sgpe::TwE<R>* out, int n, int e, int total) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  int off = 0, ns = 1;
  while (ns < n) {
    const int rs = sgpe::stage_radix(n, e, ns);
    const int cnt = (rs - 1) * ns;
    if (i < off + cnt) {
      const int r = (i - off) / ns + 1, k = (i - off) % ns;
      const long long len = (long long)ns * rs;
      const long long m = ((long long)k * r) % len;
      double sn, cs;
      sincospi(2.0 * double(m) / double(len), &sn, &cs);
      set_twiddle(out[i], cs, -sn);
      return;
    }
    off += cnt;
    ns *= rs;
  }
}

size_t round_up(size_t b) { return (b + 255) & ~size_t(255); }

template <typename R>
int run(int ny, int nx, const void* i0, const void* i1, void* o0, void* o1, int inverse, double scale,
        cudaStream_t s) {
  using C = sgpe::Cx<R>;
  const int ex = sgpe::row_points_per_thread<R>(nx), ey = sgpe::col_points_per_thread<R>(ny);
  const int cols = sgpe::col_tile_width<R>(ny);
  if (ex == 0 || ey == 0 || cols == 0 || nx % cols != 0 || (nx / 2) % cols != 0)
    return sgpe_detail::set_error(SGPE_ERR_ARG, "fft2_static: unsupported grid size");
  const int twx = sgpe::tw_offset(nx, ex, nx), twy = sgpe::tw_offset(ny, ey, ny);
  using W = sgpe::TwE<R>;
  const size_t field = round_up(sizeof(C) * (size_t)nx * ny);
  const size_t need = 2 * field + round_up(sizeof(W) * (twx > 0 ? twx : 1)) + round_up(sizeof(W) * (twy > 0 ? twy : 1));
  if (need > size_t(SGPE_FFT2_STATIC_BYTES))
    return sgpe_detail::set_error(
        SGPE_ERR_ARG, "fft2_static: a " + std::to_string(ny) + "x" + std::to_string(nx) + " complex" +
                          std::to_string(8 * sizeof(C)) + " transform needs " + std::to_string(need) +
                          " bytes of scratch; the static scratch holds " + std::to_string(SGPE_FFT2_STATIC_BYTES) +
                          " (use sgpe_fft2 with a plan for larger grids)");
  void* base = nullptr;
  int dev = 0;
  int rc = scratch_address(&dev, &base);
  if (rc != SGPE_OK) return rc;
  unsigned char* b = static_cast<unsigned char*>(base);
  C* mid0 = reinterpret_cast<C*>(b);
  C* mid1 = reinterpret_cast<C*>(b + field);
  W* tw_x = reinterpret_cast<W*>(b + 2 * field);
  W* tw_y = reinterpret_cast<W*>(b + 2 * field + round_up(sizeof(W) * (twx > 0 ? twx : 1)));
  cudaError_t e = cudaSuccess;
  {
    // twiddle tables of this grid and precision, unless the previous call
    // on this device left them in place (launch status read from the launch
    // calls themselves, so an error left pending by the caller's own earlier
    // work is neither reported here nor cleared)
    const unsigned long long key =
        (static_cast<unsigned long long>(ny) << 32) | (static_cast<unsigned long long>(nx) << 8) | sizeof(R);
    std::lock_guard<std::mutex> lock(g_tw_mutex);
    if (g_tw_key[dev].load() != key) {
      g_tw_key[dev].store(0);
      auto build = [&](W* out, int n, int ep, int total) -> cudaError_t {
        if (total <= 0) return cudaSuccess;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((total + 255) / 256);
        cfg.blockDim = dim3(256);
        cfg.stream = s;
        return cudaLaunchKernelEx(&cfg, twiddle_kernel<R>, out, n, ep, total);
      };
      e = build(tw_x, nx, ex, twx);
      if (e == cudaSuccess) e = build(tw_y, ny, ey, twy);
      if (e != cudaSuccess)
        return sgpe_detail::set_error(SGPE_ERR_CUDA, std::string("fft2_static: ") + cudaGetErrorString(e));
      g_tw_key[dev].store(key);
    }
  }

  sgpe::RowArgs<R> r{};
  r.tw = reinterpret_cast<const C*>(tw_x);
  sgpe::ColArgs<R> c{};
  c.tw = reinterpret_cast<const C*>(tw_y);
  c.nx = nx;
  c.scale = R(1);
  if (!inverse) {  // x transform into the scratch, then y transform with centring
    r.in[0] = static_cast<const C*>(i0);
    r.in[1] = static_cast<const C*>(i1);
    r.out[0] = mid0;
    r.out[1] = mid1;
    r.mode = sgpe::kRowForward;
    r.scale = R(1);
    e = sgpe::launch_row<R>(r, nx, ny, s);
    if (e == cudaSuccess) {
      c.in[0] = mid0;
      c.in[1] = mid1;
      c.out[0] = static_cast<C*>(o0);
      c.out[1] = static_cast<C*>(o1);
      c.fwd = 1;
      c.out_shift = 1;
      c.scale = R(scale);
      e = sgpe::launch_col<R>(c, ny, s);
    }
  } else {  // un-centring y transform into the scratch, then x transform
    c.in[0] = static_cast<const C*>(i0);
    c.in[1] = static_cast<const C*>(i1);
    c.out[0] = mid0;
    c.out[1] = mid1;
    c.inv = 1;
    c.in_shift = 1;
    e = sgpe::launch_col<R>(c, ny, s);
    if (e == cudaSuccess) {
      r.in[0] = mid0;
      r.in[1] = mid1;
      r.out[0] = static_cast<C*>(o0);
      r.out[1] = static_cast<C*>(o1);
      r.mode = sgpe::kRowInverse;
      r.scale = R(scale);
      e = sgpe::launch_row<R>(r, nx, ny, s);
    }
  }
  if (e != cudaSuccess) return sgpe_detail::set_error(SGPE_ERR_CUDA, std::string("fft2_static: ") + cudaGetErrorString(e));
  return SGPE_OK;
}

}  // namespace

extern "C" int sgpe_fft2_static(int ny, int nx, int dtype_bits, const void* in0, const void* in1, void* out0,
                                void* out1, int inverse, double scale, void* stream) {
  if (!in0 || !in1 || !out0 || !out1) return sgpe_detail::set_error(SGPE_ERR_ARG, "fft2_static: null data pointer");
  if (!sgpe::size_supported(nx) || !sgpe::size_supported(ny))
    return sgpe_detail::set_error(SGPE_ERR_ARG, "fft2_static: unsupported grid size (powers of two in [32, 4096], 192, 384, 768)");
  if (dtype_bits != 64 && dtype_bits != 128)
    return sgpe_detail::set_error(SGPE_ERR_ARG, "fft2_static: dtype_bits must be 64 or 128");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  return dtype_bits == 64 ? run<float>(ny, nx, in0, in1, out0, out1, inverse, scale, s)
                          : run<double>(ny, nx, in0, in1, out0, out1, inverse, scale, s);
}
