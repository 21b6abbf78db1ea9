// C ABI of the split-step solver: plan life cycle, operator upload and the
// sequencing of column/row passes that makes up the Strang steps of
// spinor_gpe/pspinor/tensor_propagator.py:214-271.
//
// State machine of a plan:
//   EMPTY --load_psik--> KSPACE (natural-order psik in the state buffers)
//   KSPACE/MIXED --single_step--> MIXED (x-forward-transformed state after a
//                                        row pass; see sgpe_kernels.cuh)
// store_psik materialises psik from MIXED (column pass + renormalisation)
// without changing the state.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <complex>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include <cuda.h>
#include <cudaTypedefs.h>

#include "sgpe_analysis.cuh"
#include "sgpe_energy.cuh"
#include "sgpe_launch.cuh"
#include "sgpe_queue.cuh"
#include "spinor_gb300.h"

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char* where) {
  return fail(SGPE_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

struct DevField {
  void* p = nullptr;
  int sx = 0, sy = 0;
};

// FP64 host copy of a field (kept for the kinetic factors, which are
// combined pairwise into the merged tables of the fused column pass).
struct HostField {
  std::vector<double> v;  // interleaved (re, im)
  int sx = 0, sy = 0;
};

// Separable form of a sub-step's operators, used by the kernels' fast
// paths: every factor as a full-length 1-D table (x-tables of nx values,
// y-tables of ny values; uniform values expanded), so the kernels index them
// with compile-time strides.  Built when the fields allow it:
//  kinetic  exp(-i K_c t/2) = kx_c(x) ky_c(ky),
//  potential exp(-i V_c t) = px_c(x) py_c(y),
//  coupling  c uniform, s conj(e) and s e x-tables.
struct SepOps {
  DevField kx[2], ky[2];
  bool kin = false, kin_real = false;
  DevField px[2], py[2], s01x, s10x;
  bool pot = false, cpl = false;
  // The real-space operators of the separable row kernels, one 2x2 matrix
  // per point: coupling, potential and coupling C P C = pb(y) A(x) with
  // A = C diag(pa_0, kappa pa_1) C (m[0..3], fused_c), or without coupling
  // the potential alone, pb(y) diag(pa_0, kappa pa_1) (dg[0..1], fused_d);
  // x-tables built in FP64 and rounded once, when the potential's y factors
  // of the components differ by a constant (pb_1 = kappa pb_0)
  DevField m[4], dg[2], mb;
  bool fused_c = false, fused_d = false, mb_real = false;
};

// True when every value of the field has a zero imaginary part.
bool imag_zero(const HostField& f) {
  for (size_t i = 1; i < f.v.size(); i += 2)
    if (f.v[i] != 0.0) return false;
  return true;
}

struct SubOps {
  DevField kin_a[2], kin_b[2], pot_a[2], pot_b[2], cc, cs, ce, s01, s10;
  bool has_s01 = false;
  bool pot_real = false, cc_real = false, kin_real = false;
  HostField s01_host, s10_host;  // FP64 off-diagonals when has_s01
  SepOps sep;
  HostField kin_host[2][2];  // [comp][a, b]
  double zr = 0.0, zi = 0.0;
  std::vector<void*> allocs;
  bool set = false;
};

// FP64 energy fields of one slot (sgpe_set_energy_fields).
struct EnergyFields {
  DevField kin_a[2], kin_b[2], pot_a[2], pot_b[2], cpl;
  std::vector<void*> allocs;
  bool set = false;
};

// Kinetic factors of two consecutive sub-steps multiplied together in FP64
// (exp(-i K t_prev/2) exp(-i K t_next/2)) and rounded once: one table pass
// in the column kernel instead of two.
struct PairOps {
  DevField a[2], b[2];
  SepOps sep;             // kinetic part only
  bool real = false;
  std::vector<void*> allocs;
  bool set = false;
};

enum Form { kEmpty = 0, kKspace = 1, kMixed = 2 };

// Makes `dev` current and restores the caller's device on scope exit (no
// driver call when it is already current).
struct DeviceGuard {
  int prev = -1;
  bool ok = false;
  explicit DeviceGuard(int dev) {
    int cur = -1;
    if (cudaGetDevice(&cur) != cudaSuccess) return;
    if (cur == dev) {
      ok = true;
    } else if (cudaSetDevice(dev) == cudaSuccess) {
      prev = cur;
      ok = true;
    }
  }
  ~DeviceGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

}  // namespace

namespace sgpe_detail {
// Sets this thread's sgpe_last_error message (used by other translation units).
int set_error(int code, const std::string& msg) { return fail(code, msg); }
}  // namespace sgpe_detail

struct sgpe_plan {
  int ny = 0, nx = 0, bits = 0, device = 0;
  size_t elem = 0;           // bytes per complex element
  void* s[2] = {nullptr, nullptr};
  void* scratch[2] = {nullptr, nullptr};
  double* part = nullptr;    // column-pass partial sums [2][ntile][2]
  double* fin = nullptr;     // their sums (3 doubles) and the pass's arrival
  unsigned* count = nullptr; // counter, behind the partials in `part`
  // the last column block forms the sums once and row blocks read them
  // (double-float plans, where every row block re-summing the partials in
  // double-float arithmetic cost ~10% of the row pass); complex64 and
  // complex128 row blocks sum the partials themselves while their other
  // warps transform, which costs less than a serial tail on the column pass
  bool final_sums = false;
  int ntile = 0;             // column tiles of the current kernels
  int ntile_fp32 = 0;        // ... of the FP32 DFT kernels
  int tc = 0;                // radix-16 stages on the tensor cores (split-BF16)
  int row_shape = 0;         // kernel shapes of the row (x) and column (y)
  int col_shape = 0;         // passes (sgpe_launch.cuh); twiddles follow them
  uint32_t* tcb = nullptr;   // their B fragments (device)
  void* tw_x = nullptr;
  void* tw_y = nullptr;
  // complex128 twiddle tables of a double-float plan, for its complex128
  // transforms (sgpe_fft2, the energy functional); made on first use
  void* tw64_x = nullptr;
  void* tw64_y = nullptr;
  SubOps sub[2];
  PairOps pair[2][2];        // [prev][next]
  EnergyFields efield[2];
  void* epsi[2] = {nullptr, nullptr};   // real-space spinor for the energy
  double* epart = nullptr;              // energy block partials [2][kEnergyBlocks][6]
  double* apart = nullptr;              // analysis block partials
  void* tmaps = nullptr;     // two CUtensorMap of the state (column-pass tiles)
  bool tmaps_valid = false;  // encoded for the current column shape
  int* derr = nullptr;       // device error word (bounded waits that gave up)
  double g[3] = {0, 0, 0};
  double atom_num = 1.0, dv_r = 1.0, dv_k = 1.0;
  int coupling = 0;
  bool physics = false;
  int form = kEmpty;
  int prev_sub = 0;
  // Device slot that receives the populations of the current (mixed) state
  // when they are next computed: set by sgpe_full_steps for its last step.
  double* pending_pops = nullptr;
  // CUDA graphs of steady-state full steps (mixed form, previous sub-step
  // outer, no populations): the six launches of a step have fixed arguments,
  // so one graph launch replaces them.  graph[0]: 1 step, graph[1]: kGraphSteps.
  cudaStream_t cap_stream = nullptr;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  bool graphs_enabled = true;
  // incremented whenever captured launches would go stale (new physics or
  // operators); batches compare it with the value at their capture
  unsigned long long epoch = 0;
};

namespace {
constexpr int kGraphSteps = 8;
}

// A set of plans stepped together: their steady-state steps are captured as
// independent branches of one CUDA graph, so the solves' kernels run
// concurrently (sgpe_batch_steps).
// Plans of one grid size and precision whose steady-state passes run as
// grouped launches (one kernel for the same pass of every member).
struct BatchGroup {
  std::vector<int> members;  // indices into sgpe_batch::plans
  int nx = 0, ny = 0, bits = 0;
  int row_shape = 0, col_shape = 0;  // the members' kernel shapes (equal)
  void* col_args = nullptr;  // device ColArgs[3][G]: (0 -> 0), (0 -> 1), (1 -> 0)
  void* row_args = nullptr;  // device RowArgs[2][G]: sub-steps 0, 1
  cudaStream_t stream = nullptr;
  cudaEvent_t join = nullptr;
};

struct sgpe_batch {
  std::vector<sgpe_plan*> plans;
  int device = 0;
  cudaStream_t root = nullptr;
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> joins;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};  // 1 step, kGraphSteps steps
  std::vector<unsigned long long> epoch[2];        // plans' epochs at capture
  std::vector<BatchGroup> groups;                  // shared by both graphs
  std::vector<unsigned long long> groups_epoch;    // plans' epochs when built
  bool groups_built = false;
  bool grouping = true;                            // SGPE_BATCH_GROUPING=0 disables
  // Work-queue mode (sgpe_batch_set_queue): the steps run as one persistent
  // launch of the queue kernel per graph (sgpe_queue.cuh) instead of
  // grouped launches in parallel branches.
  bool queue = false;
  bool q_built = false;
  bool q_direct = false;             // the launch could not be captured: launched directly
  int q_grid = 0;                    // resident blocks of the queue kernel
  void* q_solves = nullptr;          // device QueueSolve[n]
  void* q_col = nullptr;             // device ColArgs<float>[n][3]
  void* q_row = nullptr;             // device RowArgs<float>[n][2]
  int* q_first = nullptr;            // device [2][n + 1]: first column / row item of each solve
  unsigned* q_words = nullptr;       // device: error word, claim, abort, done[n][6 * kGraphSteps]
  void* q_tw[sgpe::kQueueClasses] = {};  // twiddle tables of the queue shapes per line length
  std::vector<unsigned long long> q_epoch;  // plans' epochs when the arguments were built
};

namespace {

// One twiddle-table entry from an FP64 value: rounded once, or as FP32 head
// and tail (SGPE_TW_COMP).
template <class W> W twiddle_entry(double re, double im);
template <> inline float2 twiddle_entry<float2>(double re, double im) { return make_float2(float(re), float(im)); }
template <> inline double2 twiddle_entry<double2>(double re, double im) { return make_double2(re, im); }
template <> inline float4 twiddle_entry<float4>(double re, double im) {
  const float hr = float(re), hi = float(im);
  return make_float4(hr, hi, float(re - double(hr)), float(im - double(hi)));
}

// Calls f(R{}) with R the arithmetic type of a plan's precision: float
// (complex64), double (complex128) or sgpe::DF (double-float).
template <class F> auto by_prec(int bits, F&& f) {
  if (bits == 64) return f(float{});
  if (bits == 128) return f(double{});
  return f(sgpe::DF{});
}
// ... with R the type of the plan's psik buffers (complex64 or complex128;
// a double-float plan takes complex128 buffers).
template <class F> auto by_iface(int bits, F&& f) {
  if (bits == 64) return f(float{});
  return f(double{});
}

// Per-stage twiddle table of an (n, e) transform, in the order the FFT
// engine reads it (sgpe_fft.cuh: tw_offset): for each stage (ns, r_s),
// entries exp(-2 pi i k r / (ns r_s)) at (r - 1) * ns + k.  Angles are
// reduced exactly in integers and evaluated in FP64, then rounded once.
template <typename R> void* upload_twiddles(int n, int e, cudaError_t* err) {
  using W = sgpe::TwE<R>;
  std::vector<W> h;
  const double two_pi = 6.283185307179586476925286766559;
  for (int ns = 1; ns < n;) {
    const int rs = sgpe::stage_radix(n, e, ns);
    const long long len = (long long)ns * rs;
    for (int r = 1; r < rs; ++r)
      for (int k = 0; k < ns; ++k) {
        const long long m = ((long long)k * r) % len;
        const double ang = two_pi * double(m) / double(len);
        h.push_back(twiddle_entry<W>(std::cos(ang), -std::sin(ang)));
      }
    ns *= rs;
  }
  if (h.empty()) h.push_back(twiddle_entry<W>(1.0, 0.0));
  void* d = nullptr;
  *err = cudaMalloc(&d, sizeof(W) * h.size());
  if (*err != cudaSuccess) return nullptr;
  *err = cudaMemcpy(d, h.data(), sizeof(W) * h.size(), cudaMemcpyHostToDevice);
  return d;
}

// Default kernel shape of a pass (axis 0: rows along x, 1: columns along y)
// for a side n, from single-solve step times of square grids measured on
// GB300 with sgpe_autotune (real and imaginary time ranked alike): fewer
// points per thread win where a grid is too small to give every SM enough
// warps, and for complex128 wherever the FP64 butterflies of few blocks set
// the pace.  Step times (us), shape (0,0) -> default:
//   complex64   32^2 24 -> 15, 64^2 26 -> 15, 128^2 27 -> 16,
//              256^2 29 -> 21, 512^2 69 -> 40;
//   complex128  64^2 234 -> 85, 128^2 258 -> 96, 256^2 325 -> 178 (real
//               time; imaginary time ranks alike).
int default_shape(int bits, int axis, int n) {
  struct Entry {
    int n, row, col;
  };
  static const Entry f32[] = {{32, 2, 1}, {64, 2, 2}, {128, 2, 1}, {256, 2, 0}, {512, 1, 0}};
  static const Entry f64[] = {{32, 2, 1}, {64, 2, 1}, {128, 2, 1}, {256, 2, 0}, {512, 0, 0}};
  if (bits == SGPE_DTYPE_DF) return 0;
  for (const Entry& x : (bits == 64 ? f32 : f64))
    if (x.n == n) return axis == 0 ? x.row : x.col;
  return 0;
}

int shape_count(int bits, int axis, int n) {
  if (!sgpe::size_supported(n)) return 0;
  if (bits == 64) return axis == 0 ? sgpe::row_shape_count<float>(n) : sgpe::col_shape_count<float>(n);
  if (bits == SGPE_DTYPE_DF) return axis == 0 ? sgpe::row_shape_count<sgpe::DF>(n) : sgpe::col_shape_count<sgpe::DF>(n);
  return axis == 0 ? sgpe::row_shape_count<double>(n) : sgpe::col_shape_count<double>(n);
}

// cuTensorMapEncodeTiled from the driver, looked up once through the
// runtime (no link-time dependency on libcuda); null if unavailable.
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static const PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
  }();
  return fn;
}

void free_sub(SubOps& so) {
  for (void* p : so.allocs) cudaFree(p);
  so = SubOps();
}

int upload_field(sgpe_plan* p, const sgpe_field& f, DevField* out, SubOps* so, const char* name) {
  if (f.data == nullptr || f.n < 1 || f.sx < 0 || f.sy < 0)
    return fail(SGPE_ERR_ARG, std::string("field ") + name + ": null data, empty or negative stride");
  const long long last = (long long)(p->nx - 1) * f.sx + (long long)(p->ny - 1) * f.sy;
  if (last >= f.n) return fail(SGPE_ERR_ARG, std::string("field ") + name + ": strides exceed its data");
  void* d = nullptr;
  cudaError_t e = cudaMalloc(&d, p->elem * f.n);
  if (e != cudaSuccess) return fail(SGPE_ERR_OOM, std::string("field ") + name + ": " + cudaGetErrorString(e));
  so->allocs.push_back(d);
  if (p->bits == 64) {
    std::vector<float> h(2 * (size_t)f.n);
    for (size_t i = 0; i < h.size(); ++i) h[i] = float(f.data[i]);
    e = cudaMemcpy(d, h.data(), p->elem * f.n, cudaMemcpyHostToDevice);
  } else if (p->bits == SGPE_DTYPE_DF) {
    // (re.hi, re.lo, im.hi, im.lo): the FP64 value as head + tail
    std::vector<float> h(4 * (size_t)f.n);
    for (size_t i = 0; i < 2 * (size_t)f.n; ++i) {
      const float hd = float(f.data[i]);
      h[2 * i] = hd;
      h[2 * i + 1] = float(f.data[i] - double(hd));
    }
    e = cudaMemcpy(d, h.data(), p->elem * f.n, cudaMemcpyHostToDevice);
  } else {
    e = cudaMemcpy(d, f.data, p->elem * f.n, cudaMemcpyHostToDevice);
  }
  if (e != cudaSuccess) return cuda_fail(e, "field upload");
  out->p = d;
  out->sx = f.sx;
  out->sy = f.sy;
  return SGPE_OK;
}

int upload_host_field(sgpe_plan* p, const HostField& hf, DevField* out, std::vector<void*>* allocs) {
  sgpe_field f;
  f.data = hf.v.data();
  f.n = int(hf.v.size() / 2);
  f.sx = hf.sx;
  f.sy = hf.sy;
  SubOps tmp;
  int rc = upload_field(p, f, out, &tmp, "merged kinetic");
  for (void* q : tmp.allocs) allocs->push_back(q);
  tmp.allocs.clear();
  return rc;
}

HostField host_copy(const sgpe_field& f) {
  HostField h;
  h.v.assign(f.data, f.data + 2 * (size_t)f.n);
  h.sx = f.sx;
  h.sy = f.sy;
  return h;
}

// Element-wise product of two broadcast fields, evaluated in FP64 (with
// the second factor conjugated when conj_b).
HostField multiply_fields(const HostField& fa, const HostField& fb, int nx, int ny, bool conj_b = false) {
  HostField r;
  if (fa.sx == fb.sx && fa.sy == fb.sy) {
    r.sx = fa.sx;
    r.sy = fa.sy;
  } else if (fa.sx == 0 && fa.sy == 0) {
    r.sx = fb.sx;
    r.sy = fb.sy;
  } else if (fb.sx == 0 && fb.sy == 0) {
    r.sx = fa.sx;
    r.sy = fa.sy;
  } else {
    r.sx = 1;
    r.sy = nx;
  }
  const int xs = r.sx ? nx : 1, ys = r.sy ? ny : 1;
  long long n = 0;
  for (int y = 0; y < ys; ++y)
    for (int x = 0; x < xs; ++x) n = std::max(n, (long long)x * r.sx + (long long)y * r.sy + 1);
  r.v.assign(2 * n, 0.0);
  for (int y = 0; y < ys; ++y)
    for (int x = 0; x < xs; ++x) {
      const long long ia = (long long)x * fa.sx + (long long)y * fa.sy;
      const long long ib = (long long)x * fb.sx + (long long)y * fb.sy;
      const long long ir = (long long)x * r.sx + (long long)y * r.sy;
      const double ar = fa.v[2 * ia], ai = fa.v[2 * ia + 1];
      const double br = fb.v[2 * ib], bi = conj_b ? -fb.v[2 * ib + 1] : fb.v[2 * ib + 1];
      r.v[2 * ir] = ar * br - ai * bi;
      r.v[2 * ir + 1] = ar * bi + ai * br;
    }
  return r;
}

// The values of a field that does not vary along y as an x-table of nx
// values (axis 0), or along x as a y-table of ny values (axis 1); false when
// the field varies along the other axis.
bool expand_1d(const HostField& f, int axis, int nx, int ny, HostField* out) {
  if (axis == 0 ? f.sy != 0 : f.sx != 0) return false;
  const int n = axis == 0 ? nx : ny, stride = axis == 0 ? f.sx : f.sy;
  out->sx = axis == 0 ? 1 : 0;
  out->sy = axis == 0 ? 0 : 1;
  out->v.assign(2 * (size_t)n, 0.0);
  for (int i = 0; i < n; ++i) {
    const long long k = (long long)i * stride;
    out->v[2 * i] = f.v[2 * k];
    out->v[2 * i + 1] = f.v[2 * k + 1];
  }
  return true;
}

// A product of two broadcast factors fa * fb as (x-table, y-table) when one
// factor does not vary along y and the other not along x (either order).
// The kernels multiply the two tables in the order (x, y); complex products
// are commutative bit for bit (cmul uses fma(a.x, b.x, -a.y b.y) and
// fma(a.x, b.y, a.y b.x)), so the result equals the product fa * fb.
bool split_xy(const HostField& fa, const HostField& fb, int nx, int ny, HostField* x, HostField* y) {
  if (expand_1d(fa, 0, nx, ny, x) && expand_1d(fb, 1, nx, ny, y)) return true;
  return expand_1d(fb, 0, nx, ny, x) && expand_1d(fa, 1, nx, ny, y);
}

HostField host_field(const sgpe_field& f) {
  HostField h;
  h.v.assign(f.data, f.data + 2 * (size_t)f.n);
  h.sx = f.sx;
  h.sy = f.sy;
  return h;
}

// Kinetic part of SepOps from the FP64 factors of each component.
int build_sep_kin(sgpe_plan* p, const HostField (&a)[2], const HostField (&b)[2], SepOps* so,
                  std::vector<void*>* allocs) {
  HostField x[2], y[2];
  for (int c = 0; c < 2; ++c)
    if (!split_xy(a[c], b[c], p->nx, p->ny, &x[c], &y[c])) return SGPE_OK;  // not separable: generic path
  for (int c = 0; c < 2; ++c) {
    int rc = upload_host_field(p, x[c], &so->kx[c], allocs);
    if (rc == SGPE_OK) rc = upload_host_field(p, y[c], &so->ky[c], allocs);
    if (rc != SGPE_OK) return rc;
  }
  so->kin = true;
  return SGPE_OK;
}

// The fused real-space tables of SepOps.  With c the uniform coupling
// diagonal, s01/s10 the off-diagonal x-tables (s01 == nullptr: no coupling
// tables), pa_c/pb_c the potential's x and y factors and pb_1(y) =
// kappa pb_0(y) (checked to 1e-14 over every y),
//   C diag(pa_0 pb_0, pa_1 pb_1) C = pb_0(y) A(x),
//   A00 = c^2 d0 + s01 s10 d1,  A01 = c s01 (d0 + d1),
//   A10 = c s10 (d0 + d1),      A11 = s10 s01 d0 + c^2 d1,
// and without coupling diag(pa_0 pb_0, pa_1 pb_1) = pb_0(y) diag(d0, d1),
// d0 = pa_0(x), d1 = kappa pa_1(x), all in FP64.  Leaves both fused flags
// false when the y factors are not proportional.
int build_fused(sgpe_plan* p, const HostField (&px)[2], const HostField (&py)[2], const HostField* s01,
                const HostField* s10, double cr, double ci, SepOps* so, std::vector<void*>* allocs) {
  typedef std::complex<double> cd;
  const int nx = p->nx, ny = p->ny;
  auto at = [](const HostField& f, int i) { return cd(f.v[2 * i], f.v[2 * i + 1]); };
  const cd b00 = at(py[0], 0);
  if (std::abs(b00) == 0.0) return SGPE_OK;
  const cd kappa = at(py[1], 0) / b00;
  for (int y = 0; y < ny; ++y) {
    const cd b0 = at(py[0], y), b1 = at(py[1], y);
    if (std::abs(b1 - kappa * b0) > 1e-14 * std::abs(b1) + 1e-300) return SGPE_OK;
  }
  auto table = [&](HostField* f) {
    f->sx = 1;
    f->sy = 0;
    f->v.assign(2 * (size_t)nx, 0.0);
  };
  auto put = [](HostField* f, int x, cd v) {
    f->v[2 * x] = v.real();
    f->v[2 * x + 1] = v.imag();
  };
  const cd c(cr, ci);
  HostField m[4], dg[2];
  for (auto& f : m) table(&f);
  for (auto& f : dg) table(&f);
  for (int x = 0; x < nx; ++x) {
    const cd d0 = at(px[0], x), d1 = kappa * at(px[1], x);
    put(&dg[0], x, d0);
    put(&dg[1], x, d1);
    if (s01 != nullptr) {
      const cd a01 = at(*s01, x), a10 = at(*s10, x);
      put(&m[0], x, c * c * d0 + a01 * a10 * d1);
      put(&m[1], x, c * a01 * (d0 + d1));
      put(&m[2], x, c * a10 * (d0 + d1));
      put(&m[3], x, a10 * a01 * d0 + c * c * d1);
    }
  }
  int rc = upload_host_field(p, py[0], &so->mb, allocs);
  for (int k = 0; k < 2 && rc == SGPE_OK; ++k) rc = upload_host_field(p, dg[k], &so->dg[k], allocs);
  if (rc != SGPE_OK) return rc;
  so->mb_real = imag_zero(py[0]);
  so->fused_d = true;
  if (s01 != nullptr) {
    for (int k = 0; k < 4 && rc == SGPE_OK; ++k) rc = upload_host_field(p, m[k], &so->m[k], allocs);
    if (rc != SGPE_OK) return rc;
    so->fused_c = true;
  }
  return SGPE_OK;
}

constexpr int kEnergyBlocks = 304;

// FP64 upload of a field (energy fields keep double precision).
int upload_field64(sgpe_plan* p, const sgpe_field& f, DevField* out, std::vector<void*>* allocs, const char* name) {
  if (f.data == nullptr || f.n < 1 || f.sx < 0 || f.sy < 0)
    return fail(SGPE_ERR_ARG, std::string("field ") + name + ": null data, empty or negative stride");
  const long long last = (long long)(p->nx - 1) * f.sx + (long long)(p->ny - 1) * f.sy;
  if (last >= f.n) return fail(SGPE_ERR_ARG, std::string("field ") + name + ": strides exceed its data");
  void* d = nullptr;
  cudaError_t e = cudaMalloc(&d, sizeof(double2) * f.n);
  if (e != cudaSuccess) return fail(SGPE_ERR_OOM, std::string("field ") + name + ": " + cudaGetErrorString(e));
  allocs->push_back(d);
  e = cudaMemcpy(d, f.data, sizeof(double2) * f.n, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(e, "energy field upload");
  out->p = d;
  out->sx = f.sx;
  out->sy = f.sy;
  return SGPE_OK;
}

void free_efield(EnergyFields& ef) {
  for (void* q : ef.allocs) cudaFree(q);
  ef = EnergyFields();
}

sgpe::Field<double> typed64(const DevField& f) {
  return sgpe::Field<double>{static_cast<const double2*>(f.p), f.sx, f.sy};
}

void free_pair(PairOps& po) {
  for (void* q : po.allocs) cudaFree(q);
  po = PairOps();
}

// Merged kinetic tables for (prev, next), built on first use.
int ensure_pair(sgpe_plan* p, int prev, int next) {
  PairOps& po = p->pair[prev][next];
  if (po.set) return SGPE_OK;
  HostField ma[2], mb[2];
  for (int c = 0; c < 2; ++c) {
    ma[c] = multiply_fields(p->sub[prev].kin_host[c][0], p->sub[next].kin_host[c][0], p->nx, p->ny);
    mb[c] = multiply_fields(p->sub[prev].kin_host[c][1], p->sub[next].kin_host[c][1], p->nx, p->ny);
    int rc = upload_host_field(p, ma[c], &po.a[c], &po.allocs);
    if (rc == SGPE_OK) rc = upload_host_field(p, mb[c], &po.b[c], &po.allocs);
    if (rc != SGPE_OK) {
      free_pair(po);
      return rc;
    }
  }
  const int rc = build_sep_kin(p, ma, mb, &po.sep, &po.allocs);
  if (rc != SGPE_OK) {
    free_pair(po);
    return rc;
  }
  po.real = imag_zero(ma[0]) && imag_zero(ma[1]) && imag_zero(mb[0]) && imag_zero(mb[1]);
  po.set = true;
  return SGPE_OK;
}

template <typename R> sgpe::Field<R> typed(const DevField& f) {
  return sgpe::Field<R>{static_cast<const sgpe::Cx<R>*>(f.p), f.sx, f.sy};
}

template <typename R>
sgpe::KinOp<R> kin_from(const DevField (&a)[2], const DevField (&b)[2], const SepOps& sep, bool real) {
  sgpe::KinOp<R> k;
  for (int c = 0; c < 2; ++c) {
    k.a[c] = typed<R>(sep.kin ? sep.kx[c] : a[c]);
    k.b[c] = typed<R>(sep.kin ? sep.ky[c] : b[c]);
  }
  k.sep = sep.kin ? 1 : 0;
  k.real = real ? 1 : 0;
  return k;
}

template <typename R> sgpe::KinOp<R> kin_op(const SubOps& so) {
  return kin_from<R>(so.kin_a, so.kin_b, so.sep, so.kin_real);
}

template <typename R> sgpe::KinOp<R> kin_pair(const PairOps& po) { return kin_from<R>(po.a, po.b, po.sep, po.real); }

// The separable row kernels carry the fused point-wise code (SepOps::m /
// dg); any other operator takes the generic broadcast-field kernels.
bool fused_sep(const SubOps& so, int coupling) { return coupling ? so.sep.fused_c : so.sep.fused_d; }

template <typename R> sgpe::RealOp<R> real_op(const SubOps& so, int coupling) {
  sgpe::RealOp<R> o;
  const bool sep = fused_sep(so, coupling);
  for (int c = 0; c < 2; ++c) {
    o.pa[c] = typed<R>(so.pot_a[c]);
    o.pb[c] = typed<R>(so.pot_b[c]);
  }
  o.cc = typed<R>(so.cc);
  o.cs = typed<R>(so.cs);
  o.ce = typed<R>(so.ce);
  o.has_s01 = so.has_s01 ? 1 : 0;
  o.s01 = typed<R>(so.has_s01 ? so.s01 : so.cs);
  o.s10 = typed<R>(so.has_s01 ? so.s10 : so.cs);
  o.sep = sep ? 1 : 0;
  o.diag = coupling ? 0 : 1;
  if (sep) {
    if (coupling) {
      for (int k = 0; k < 4; ++k) o.m[k] = typed<R>(so.sep.m[k]);
    } else {
      o.m[0] = o.m[1] = o.m[2] = typed<R>(so.sep.dg[0]);  // m[1], m[2] unread
      o.m[3] = typed<R>(so.sep.dg[1]);
    }
    o.mb = typed<R>(so.sep.mb);
    o.real_mb = so.sep.mb_real ? 1 : 0;
  }
  o.real_pot = so.pot_real ? 1 : 0;
  o.real_cc = so.cc_real ? 1 : 0;
  o.zr = R(so.zr);
  o.zi = R(so.zi);
  return o;
}

template <typename R> sgpe::Cx<R>* st(void* p) { return static_cast<sgpe::Cx<R>*>(p); }
template <typename R> const sgpe::Cx<R>* cst(const void* p) { return static_cast<const sgpe::Cx<R>*>(p); }

// Column pass over the state (in place) ending a sub-step and starting `sub`.
// want_u: the populations of the state entering the pass are needed, so the
// two kinetic half steps are applied separately (sum after the first).
// Arguments of the column pass that starts sub-step `sub` (from the plan's
// current form and previous sub-step); false if a merged table could not be
// allocated.
template <typename R> bool col_step_args(sgpe_plan* p, int sub, bool want_u, sgpe::ColArgs<R>* out) {
  sgpe::ColArgs<R>& a = *out;
  a = sgpe::ColArgs<R>{};
  a.in[0] = cst<R>(p->s[0]);
  a.in[1] = cst<R>(p->s[1]);
  a.out[0] = st<R>(p->s[0]);
  a.out[1] = st<R>(p->s[1]);
  a.tw = cst<R>(p->tw_y);
  a.tc = p->tc;
  a.tcb = p->tcb;
  a.shape = p->col_shape;
  a.tmap = (p->tmaps_valid && !p->tc) ? p->tmaps : nullptr;  // in place, no shifts
  a.err = p->derr;
  a.nx = p->nx;
  a.fwd = (p->form == kMixed);
  a.inv = 1;
  if (p->form != kMixed) {
    a.nk = 1;
    a.k1 = kin_op<R>(p->sub[sub]);
  } else if (want_u) {
    a.nk = 2;
    a.k1 = kin_op<R>(p->sub[p->prev_sub]);
    a.k2 = kin_op<R>(p->sub[sub]);
  } else {
    if (ensure_pair(p, p->prev_sub, sub) != SGPE_OK) return false;
    a.nk = 1;
    a.k1 = kin_pair<R>(p->pair[p->prev_sub][sub]);
  }
  a.scale = R(1);
  a.part = reinterpret_cast<R*>(p->part);
  a.fin = p->final_sums ? p->fin : nullptr;
  a.count = p->count;
  return true;
}

template <typename R> cudaError_t col_pass_step(sgpe_plan* p, int sub, double* pops, cudaStream_t s) {
  sgpe::ColArgs<R> a;
  if (!col_step_args<R>(p, sub, pops != nullptr, &a)) return cudaErrorMemoryAllocation;
  return sgpe::launch_col<R>(a, p->ny, s);
}

// Arguments of the row pass of sub-step `sub`.
template <typename R> sgpe::RowArgs<R> row_step_args(sgpe_plan* p, int sub, double* pops) {
  sgpe::RowArgs<R> a{};
  a.in[0] = cst<R>(p->s[0]);
  a.in[1] = cst<R>(p->s[1]);
  a.out[0] = st<R>(p->s[0]);
  a.out[1] = st<R>(p->s[1]);
  a.tw = cst<R>(p->tw_x);
  a.tc = p->tc;
  a.tcb = p->tcb;
  a.shape = p->row_shape;
  a.err = p->derr;
  a.mode = sgpe::kRowStep;
  a.scale = R(1);
  a.part = reinterpret_cast<R*>(p->part);
  a.ntile = p->ntile;
  a.fin = p->final_sums ? p->fin : nullptr;
  a.norm_num = p->atom_num / (double(p->nx) * double(p->ny) * p->dv_r);
  a.g_uu = R(p->g[0]);
  a.g_dd = R(p->g[1]);
  a.g_ud = R(p->g[2]);
  a.coupling = p->coupling;
  a.op = real_op<R>(p->sub[sub], p->coupling);
  a.pops = pops;
  a.atom_num = p->atom_num;
  return a;
}

template <typename R> cudaError_t row_pass_step(sgpe_plan* p, int sub, double* pops, cudaStream_t s) {
  const sgpe::RowArgs<R> a = row_step_args<R>(p, sub, pops);
  return sgpe::launch_row<R>(a, p->nx, p->ny, s);
}

template <typename R> int substep(sgpe_plan* p, int sub, double* pops, cudaStream_t s) {
  const bool fused = (p->form == kMixed);
  if (fused && pops == nullptr) pops = p->pending_pops;
  p->pending_pops = nullptr;
  cudaError_t e = col_pass_step<R>(p, sub, fused ? pops : nullptr, s);
  if (e != cudaSuccess) return cuda_fail(e, "column pass");
  e = row_pass_step<R>(p, sub, fused ? pops : nullptr, s);
  if (e != cudaSuccess) return cuda_fail(e, "row pass");
  p->form = kMixed;
  p->prev_sub = sub;
  return SGPE_OK;
}

// Conversion copies of the double-float state (sgpe::DfCopyArgs).
__global__ void __launch_bounds__(256) df_copy_kernel(const sgpe::DfCopyArgs a) {
  __shared__ double s_alpha;
  if (threadIdx.x < 32) {
    double alpha = 1.0;
    if (a.part != nullptr) {
      double s0, s1, sw;
      sgpe::sum_partials(a.part, a.ntile, threadIdx.x, &s0, &s1, &sw);
      alpha = sqrt(a.atom_num / (a.dv * (s0 + s1)));
      if (threadIdx.x == 0 && a.pops != nullptr && blockIdx.x == 0) {
        a.pops[0] = a.atom_num * s0 / (s0 + s1);
        a.pops[1] = a.atom_num * s1 / (s0 + s1);
      }
    }
    if (threadIdx.x == 0) s_alpha = alpha;
  }
  __syncthreads();
  const double alpha = s_alpha;
  const long long n = (long long)a.nx * a.ny;
  const long long stride = (long long)gridDim.x * blockDim.x;
  const int sx = a.shift ? a.nx / 2 : 0, sy = a.shift ? a.ny / 2 : 0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int y = int(i / a.nx), x = int(i - (long long)y * a.nx);
    const long long src = (long long)((y + sy) % a.ny) * a.nx + (x + sx) % a.nx;
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      if (a.to_df) {
        static_cast<sgpe::DFC*>(a.out[c])[i] = sgpe::to_dfc(static_cast<const double2*>(a.in[c])[src]);
      } else {
        const double2 z = sgpe::from_dfc(static_cast<const sgpe::DFC*>(a.in[c])[src]);
        static_cast<double2*>(a.out[c])[i] = make_double2(z.x * alpha, z.y * alpha);
      }
    }
  }
}

// Double-float state to complex128 psik: in k-space form a converting copy;
// in mixed form the column pass into the plan's scratch (centred order),
// then the conversion with the final renormalisation and populations.
int store_df(sgpe_plan* p, void* o0, void* o1, double* pops, cudaStream_t s) {
  using R = sgpe::DF;
  sgpe::DfCopyArgs d{};
  d.out[0] = o0;
  d.out[1] = o1;
  d.nx = p->nx;
  d.ny = p->ny;
  d.to_df = 0;
  if (p->form == kKspace) {
    d.in[0] = p->s[0];
    d.in[1] = p->s[1];
    d.shift = 1;
  } else {
    for (int c = 0; c < 2; ++c) {
      if (p->scratch[c] == nullptr) {
        const cudaError_t e = cudaMalloc(&p->scratch[c], p->elem * p->nx * p->ny);
        if (e != cudaSuccess) return fail(SGPE_ERR_OOM, std::string("store scratch: ") + cudaGetErrorString(e));
      }
    }
    sgpe::ColArgs<R> a{};
    a.in[0] = cst<R>(p->s[0]);
    a.in[1] = cst<R>(p->s[1]);
    a.out[0] = st<R>(p->scratch[0]);
    a.out[1] = st<R>(p->scratch[1]);
    a.tw = cst<R>(p->tw_y);
    a.shape = p->col_shape;
    a.nx = p->nx;
    a.fwd = 1;
    a.inv = 0;
    a.out_shift = 1;
    a.nk = 1;
    a.k1 = kin_op<R>(p->sub[p->prev_sub]);
    a.scale = R(1);
    a.part = reinterpret_cast<R*>(p->part);
    const cudaError_t e = sgpe::launch_col<R>(a, p->ny, s);
    if (e != cudaSuccess) return cuda_fail(e, "store (column pass)");
    d.in[0] = p->scratch[0];
    d.in[1] = p->scratch[1];
    d.shift = 0;
    d.part = reinterpret_cast<const R*>(p->part);
    d.ntile = p->ntile;
    d.atom_num = p->atom_num;
    d.dv = p->dv_k;
    d.pops = pops != nullptr ? pops : p->pending_pops;
    p->pending_pops = nullptr;
  }
  df_copy_kernel<<<8 * 152, 256, 0, s>>>(d);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? SGPE_OK : cuda_fail(e, "store (double-float conversion)");
}

template <typename R> int store(sgpe_plan* p, void* o0, void* o1, double* pops, cudaStream_t s) {
  if (p->form == kKspace) {
    sgpe::CopyArgs<R> c{};
    c.in[0] = cst<R>(p->s[0]);
    c.in[1] = cst<R>(p->s[1]);
    c.out[0] = st<R>(o0);
    c.out[1] = st<R>(o1);
    c.nx = p->nx;
    c.ny = p->ny;
    c.shift = 1;
    c.scale = R(1);
    cudaError_t e = sgpe::launch_copy<R>(c, s);
    return e == cudaSuccess ? SGPE_OK : cuda_fail(e, "store (copy)");
  }
  sgpe::ColArgs<R> a{};
  a.in[0] = cst<R>(p->s[0]);
  a.in[1] = cst<R>(p->s[1]);
  a.out[0] = st<R>(o0);
  a.out[1] = st<R>(o1);
  a.tw = cst<R>(p->tw_y);
  a.tc = p->tc;
  a.tcb = p->tcb;
  a.shape = p->col_shape;
  a.nx = p->nx;
  a.fwd = 1;
  a.inv = 0;
  a.out_shift = 1;
  a.nk = 1;
  a.k1 = kin_op<R>(p->sub[p->prev_sub]);
  a.scale = R(1);
  a.part = reinterpret_cast<R*>(p->part);
  cudaError_t e = sgpe::launch_col<R>(a, p->ny, s);
  if (e != cudaSuccess) return cuda_fail(e, "store (column pass)");
  sgpe::ScaleArgs<R> sa{};
  sa.d[0] = st<R>(o0);
  sa.d[1] = st<R>(o1);
  sa.n = (long long)p->nx * p->ny;
  sa.part = reinterpret_cast<const R*>(p->part);
  sa.ntile = p->ntile;
  sa.atom_num = p->atom_num;
  sa.dv = p->dv_k;
  sa.pops = pops != nullptr ? pops : p->pending_pops;
  p->pending_pops = nullptr;
  e = sgpe::launch_scale<R>(sa, s);
  return e == cudaSuccess ? SGPE_OK : cuda_fail(e, "store (scale)");
}

template <> int store<sgpe::DF>(sgpe_plan* p, void* o0, void* o1, double* pops, cudaStream_t s) {
  return store_df(p, o0, o1, pops, s);
}

// Twiddle tables for transforms in the arithmetic of R: the plan's own, or,
// for the complex128 transforms of a double-float plan, complex128 tables of
// kernel shape 0 made on first use.
template <typename R> int transform_tables(sgpe_plan* p, const void** tx, const void** ty) {
  if (!(std::is_same<R, double>::value && p->bits == SGPE_DTYPE_DF)) {
    *tx = p->tw_x;
    *ty = p->tw_y;
    return SGPE_OK;
  }
  if (p->tw64_x == nullptr) {
    cudaError_t e = cudaSuccess;
    void* x = upload_twiddles<double>(p->nx, sgpe::row_points_per_thread<double>(p->nx, 0), &e);
    void* y = e == cudaSuccess ? upload_twiddles<double>(p->ny, sgpe::col_points_per_thread<double>(p->ny, 0), &e)
                               : nullptr;
    if (e != cudaSuccess) {
      if (x) cudaFree(x);
      if (y) cudaFree(y);
      return fail(SGPE_ERR_OOM, std::string("complex128 twiddle tables: ") + cudaGetErrorString(e));
    }
    p->tw64_x = x;
    p->tw64_y = y;
  }
  *tx = p->tw64_x;
  *ty = p->tw64_y;
  return SGPE_OK;
}

template <typename R> int fft2(sgpe_plan* p, const void* i0, const void* i1, void* o0, void* o1,
                               int inverse, double scale, cudaStream_t s) {
  if (p->scratch[0] == nullptr) {
    for (int c = 0; c < 2; ++c) {
      cudaError_t e = cudaMalloc(&p->scratch[c], p->elem * p->nx * p->ny);
      if (e != cudaSuccess) return fail(SGPE_ERR_OOM, std::string("fft2 scratch: ") + cudaGetErrorString(e));
    }
  }
  const void* twx = nullptr;
  const void* twy = nullptr;
  const int trc = transform_tables<R>(p, &twx, &twy);
  if (trc != SGPE_OK) return trc;
  // the complex128 transforms of a double-float plan run in shape 0
  const bool own = (p->bits != SGPE_DTYPE_DF);
  sgpe::RowArgs<R> r{};
  r.tw = cst<R>(twx);
  r.tc = p->tc;
  r.tcb = p->tcb;
  r.shape = own ? p->row_shape : 0;
  sgpe::ColArgs<R> c{};
  c.tw = cst<R>(twy);
  c.tc = p->tc;
  c.tcb = p->tcb;
  c.shape = own ? p->col_shape : 0;
  c.nx = p->nx;
  c.scale = R(1);
  cudaError_t e;
  if (!inverse) {
    r.in[0] = cst<R>(i0);
    r.in[1] = cst<R>(i1);
    r.out[0] = st<R>(p->scratch[0]);
    r.out[1] = st<R>(p->scratch[1]);
    r.mode = sgpe::kRowForward;
    r.scale = R(1);
    e = sgpe::launch_row<R>(r, p->nx, p->ny, s);
    if (e != cudaSuccess) return cuda_fail(e, "fft2 row pass");
    c.in[0] = cst<R>(p->scratch[0]);
    c.in[1] = cst<R>(p->scratch[1]);
    c.out[0] = st<R>(o0);
    c.out[1] = st<R>(o1);
    c.fwd = 1;
    c.out_shift = 1;
    c.scale = R(scale);
    e = sgpe::launch_col<R>(c, p->ny, s);
    if (e != cudaSuccess) return cuda_fail(e, "fft2 column pass");
  } else {
    c.in[0] = cst<R>(i0);
    c.in[1] = cst<R>(i1);
    c.out[0] = st<R>(p->scratch[0]);
    c.out[1] = st<R>(p->scratch[1]);
    c.inv = 1;
    c.in_shift = 1;
    e = sgpe::launch_col<R>(c, p->ny, s);
    if (e != cudaSuccess) return cuda_fail(e, "ifft2 column pass");
    r.in[0] = cst<R>(p->scratch[0]);
    r.in[1] = cst<R>(p->scratch[1]);
    r.out[0] = st<R>(o0);
    r.out[1] = st<R>(o1);
    r.mode = sgpe::kRowInverse;
    r.scale = R(scale);
    e = sgpe::launch_row<R>(r, p->nx, p->ny, s);
    if (e != cudaSuccess) return cuda_fail(e, "ifft2 row pass");
  }
  return SGPE_OK;
}

bool ready(sgpe_plan* p) { return p->physics && p->sub[0].set && p->sub[1].set; }

template <typename R>
int energy_impl(sgpe_plan* p, int slot, const void* k0, const void* k1, double* out, cudaStream_t s) {
  const EnergyFields& ef = p->efield[slot];
  const long long n = (long long)p->nx * p->ny;
  for (int c = 0; c < 2; ++c) {
    if (p->epsi[c] == nullptr) {
      cudaError_t e = cudaMalloc(&p->epsi[c], p->elem * n);
      if (e != cudaSuccess) return fail(SGPE_ERR_OOM, std::string("energy buffer: ") + cudaGetErrorString(e));
    }
  }
  if (p->epart == nullptr) {
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&p->epart), sizeof(double) * 2 * kEnergyBlocks * sgpe::kEnergySums);
    if (e != cudaSuccess) return fail(SGPE_ERR_OOM, std::string("energy partials: ") + cudaGetErrorString(e));
  }
  sgpe::EnergyArgs<R> a{};
  a.n = n;
  a.nx = p->nx;
  a.g_uu = p->g[0];
  a.g_dd = p->g[1];
  a.g_ud = p->g[2];
  a.h = typed64(ef.cpl);
  // k-space pass on psik
  a.a[0] = cst<R>(k0);
  a.a[1] = cst<R>(k1);
  for (int c = 0; c < 2; ++c) {
    a.w[c] = typed64(ef.kin_a[c]);
    a.wb[c] = typed64(ef.kin_b[c]);
  }
  a.part = p->epart;
  sgpe::energy_k_kernel<R><<<kEnergyBlocks, 256, 0, s>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "energy (k pass)");
  // psi = ifft_2d(psik): unnormalised inverse over N points, times 2 pi/(dx dy)
  const double dxdy = p->dv_r;
  const int rc = fft2<R>(p, k0, k1, p->epsi[0], p->epsi[1], 1, 6.283185307179586476925286766559 / (double(n) * dxdy), s);
  if (rc != SGPE_OK) return rc;
  a.a[0] = cst<R>(p->epsi[0]);
  a.a[1] = cst<R>(p->epsi[1]);
  for (int c = 0; c < 2; ++c) {
    a.w[c] = typed64(ef.pot_a[c]);
    a.wb[c] = typed64(ef.pot_b[c]);
  }
  a.part = p->epart + kEnergyBlocks * sgpe::kEnergySums;
  sgpe::energy_r_kernel<R><<<kEnergyBlocks, 256, 0, s>>>(a);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "energy (real-space pass)");
  sgpe::energy_finalize_kernel<<<1, 32, 0, s>>>(p->epart, p->epart + kEnergyBlocks * sgpe::kEnergySums,
                                                kEnergyBlocks, p->dv_k, p->dv_r, out);
  e = cudaGetLastError();
  return e == cudaSuccess ? SGPE_OK : cuda_fail(e, "energy (finalise)");
}

// Tensor maps of the two state components for the column pass's TMA tiles
// (ColArgs::tmap): the component as a 2-D array of working-precision
// scalars {2 nx, ny} (row stride nx complex values), box {2 COLS, min(ny,
// 256)} for the current column shape.  Left invalid (plain loads) when the
// encoder is unavailable or refuses the layout.
template <typename R> void update_col_tmaps(sgpe_plan* p) {
  p->tmaps_valid = false;
  if (!SGPE_COL_TMA) return;  // the kernels are built without the TMA tiles
  if (p->bits == SGPE_DTYPE_DF) return;  // plain loads for double-float tiles
  const PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  const int cols = sgpe::col_tile_width<R>(p->ny, p->col_shape);
  if (enc == nullptr || cols == 0) return;
  if (p->tmaps == nullptr && cudaMalloc(&p->tmaps, 2 * sizeof(CUtensorMap)) != cudaSuccess) {
    p->tmaps = nullptr;
    return;
  }
  CUtensorMap maps[2];
  const cuuint64_t dims[2] = {cuuint64_t(2) * p->nx, cuuint64_t(p->ny)};
  const cuuint64_t strides[1] = {cuuint64_t(p->nx) * p->elem};
  const cuuint32_t box[2] = {cuuint32_t(2 * cols), cuuint32_t(std::min(p->ny, 256))};
  const cuuint32_t estr[2] = {1, 1};
  const CUtensorMapDataType dt = sizeof(R) == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
  for (int c = 0; c < 2; ++c)
    if (enc(&maps[c], dt, 2, p->s[c], dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return;
  if (cudaMemcpy(p->tmaps, maps, sizeof(maps), cudaMemcpyHostToDevice) != cudaSuccess) return;
  p->tmaps_valid = true;
}

void drop_graphs(sgpe_plan* p) {
  ++p->epoch;
  for (auto& g : p->graph) {
    if (g) cudaGraphExecDestroy(g);
    g = nullptr;
  }
}

// One eager full step (outer, inner, outer).
template <typename R> int eager_step(sgpe_plan* p, double* pops, cudaStream_t s) {
  int rc = substep<R>(p, 0, pops, s);
  if (rc == SGPE_OK) rc = substep<R>(p, 1, nullptr, s);
  if (rc == SGPE_OK) rc = substep<R>(p, 0, nullptr, s);
  return rc;
}

// Capture `steps` steady-state full steps into an executable graph.  The plan
// must be in mixed form after an outer sub-step with no pending populations;
// the capture leaves that state unchanged.
template <typename R> int capture_steps(sgpe_plan* p, int steps, cudaGraphExec_t* out) {
  if (p->cap_stream == nullptr) {
    cudaError_t e = cudaStreamCreateWithFlags(&p->cap_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_fail(e, "graph stream");
  }
  // merged kinetic tables must exist before capture (they allocate)
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b)
      if (ensure_pair(p, a, b) != SGPE_OK) return SGPE_ERR_OOM;
  cudaError_t e = cudaStreamBeginCapture(p->cap_stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return cuda_fail(e, "begin capture");
  int rc = SGPE_OK;
  for (int i = 0; i < steps && rc == SGPE_OK; ++i) rc = eager_step<R>(p, nullptr, p->cap_stream);
  cudaGraph_t graph = nullptr;
  e = cudaStreamEndCapture(p->cap_stream, &graph);
  if (rc != SGPE_OK) {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  if (e != cudaSuccess) return cuda_fail(e, "end capture");
  e = cudaGraphInstantiate(out, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return cuda_fail(e, "graph instantiate");
  return SGPE_OK;
}

// Switch the plan's kernel shapes: new twiddle tables for an axis whose
// shape changes, the column-tile count, and the captured graphs dropped.
// The mixed state is the same in every shape, so this is valid between any
// two calls.
template <typename R> int apply_shapes(sgpe_plan* p, int rs, int cs) {
  if (rs < 0 || rs >= shape_count(p->bits, 0, p->nx) || cs < 0 || cs >= shape_count(p->bits, 1, p->ny))
    return fail(SGPE_ERR_ARG, "kernel shape out of range for this grid (sgpe_shape_count)");
  if (p->tc && (rs != 0 || cs != 0)) return fail(SGPE_ERR_STATE, "the tensor-core DFT mode runs shape 0 only");
  if (rs == p->row_shape && cs == p->col_shape) return SGPE_OK;
  const int cols = sgpe::col_tile_width<R>(p->ny, cs);
  if (cols == 0 || p->nx % cols != 0 || (p->nx / 2) % cols != 0)
    return fail(SGPE_ERR_ARG, "nx incompatible with the column tile width of that shape");
  DeviceGuard g(p->device);
  cudaError_t e = cudaSuccess;
  void* tx = nullptr;
  void* ty = nullptr;
  if (rs != p->row_shape) tx = upload_twiddles<R>(p->nx, sgpe::row_points_per_thread<R>(p->nx, rs), &e);
  if (e == cudaSuccess && cs != p->col_shape)
    ty = upload_twiddles<R>(p->ny, sgpe::col_points_per_thread<R>(p->ny, cs), &e);
  if (e != cudaSuccess) {
    if (tx) cudaFree(tx);
    if (ty) cudaFree(ty);
    return fail(SGPE_ERR_OOM, std::string("twiddle tables: ") + cudaGetErrorString(e));
  }
  drop_graphs(p);
  // cudaFree waits for launches still reading the old tables
  if (tx) {
    cudaFree(p->tw_x);
    p->tw_x = tx;
  }
  if (ty) {
    cudaFree(p->tw_y);
    p->tw_y = ty;
  }
  p->row_shape = rs;
  p->col_shape = cs;
  p->ntile_fp32 = p->nx / cols;
  p->ntile = p->ntile_fp32;
  update_col_tmaps<R>(p);
  return SGPE_OK;
}

int apply_shapes_any(sgpe_plan* p, int rs, int cs) {
  return by_prec(p->bits, [&](auto t) { return apply_shapes<decltype(t)>(p, rs, cs); });
}

template <typename R> int full_steps_impl(sgpe_plan* p, int n_steps, double* pops, cudaStream_t s) {
  int i = 0;
  while (i < n_steps) {
    double* slot = (pops != nullptr && i > 0) ? pops + 2 * (i - 1) : nullptr;
    const bool steady = p->graphs_enabled && slot == nullptr && p->pending_pops == nullptr &&
                        p->form == kMixed && p->prev_sub == 0 && (pops == nullptr || i > 0);
    if (steady && pops == nullptr) {
      const int k = (n_steps - i >= kGraphSteps) ? 1 : 0;
      if (p->graph[k] == nullptr) {
        const int rc = capture_steps<R>(p, k ? kGraphSteps : 1, &p->graph[k]);
        if (rc != SGPE_OK) return rc;
      }
      const cudaError_t e = cudaGraphLaunch(p->graph[k], s);
      if (e != cudaSuccess) return cuda_fail(e, "graph launch");
      i += k ? kGraphSteps : 1;
      continue;
    }
    const int rc = eager_step<R>(p, slot, s);
    if (rc != SGPE_OK) return rc;
    ++i;
  }
  return SGPE_OK;
}

}  // namespace

extern "C" {

int sgpe_version(void) { return 100; }

const char* sgpe_last_error(void) { return g_last_error.c_str(); }

int sgpe_plan_create(sgpe_plan** out, int ny, int nx, int dtype_bits, int device) {
  if (out == nullptr) return fail(SGPE_ERR_ARG, "plan output pointer is null");
  *out = nullptr;
  if (!sgpe::size_supported(nx) || !sgpe::size_supported(ny))
    return fail(SGPE_ERR_ARG, "grid sizes must be powers of two in [32, 4096] or 192, 384, 768, got ny=" + std::to_string(ny) +
                                  " nx=" + std::to_string(nx));
  if (dtype_bits != 64 && dtype_bits != 128 && dtype_bits != SGPE_DTYPE_DF)
    return fail(SGPE_ERR_ARG, "dtype_bits must be 64, 128 or SGPE_DTYPE_DF (48)");
  DeviceGuard g(device);
  if (!g.ok) return fail(SGPE_ERR_ARG, "cannot select device " + std::to_string(device));
  sgpe_plan* p = new sgpe_plan();
  p->ny = ny;
  p->nx = nx;
  p->bits = dtype_bits;
  p->device = device;
  p->elem = dtype_bits == 64 ? sizeof(float2) : dtype_bits == 128 ? sizeof(double2) : sizeof(sgpe::DFC);
  // SGPE_DISABLE_GRAPHS (any value) makes this plan launch every step
  // eagerly; used to check graph replay against eager launches.
  p->graphs_enabled = std::getenv("SGPE_DISABLE_GRAPHS") == nullptr;
  // SGPE_FINAL_SUMS=0/1 overrides the precision's choice (measurements)
  const char* fs = std::getenv("SGPE_FINAL_SUMS");
  p->final_sums = fs != nullptr ? fs[0] == '1' : dtype_bits == SGPE_DTYPE_DF;
  p->row_shape = default_shape(dtype_bits, 0, nx);
  p->col_shape = default_shape(dtype_bits, 1, ny);
  int cols = by_prec(dtype_bits, [&](auto t) { return sgpe::col_tile_width<decltype(t)>(ny, p->col_shape); });
  if (cols == 0 || nx % cols != 0 || (nx / 2) % cols != 0) {
    // the default shape's tile does not divide nx: shape 0
    p->col_shape = 0;
    cols = by_prec(dtype_bits, [&](auto t) { return sgpe::col_tile_width<decltype(t)>(ny); });
  }
  if (cols == 0 || nx % cols != 0 || (nx / 2) % cols != 0) {
    delete p;
    return fail(SGPE_ERR_ARG, "nx incompatible with the column tile width");
  }
  p->ntile = nx / cols;
  p->ntile_fp32 = p->ntile;
  cudaError_t e = cudaSuccess;
  for (int c = 0; c < 2 && e == cudaSuccess; ++c) e = cudaMalloc(&p->s[c], p->elem * (size_t)nx * ny);
  // room for one tile per column: every kernel configuration fits
  const size_t red_bytes = sizeof(double) * 4 * (size_t)nx + 64;  // + final sums and counter
  if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&p->part), red_bytes);
  if (e == cudaSuccess) e = cudaMemset(p->part, 0, red_bytes);
  if (e == cudaSuccess) {
    p->fin = p->part + 4 * (size_t)nx;
    p->count = reinterpret_cast<unsigned*>(p->fin + 4);
  }
  if (e == cudaSuccess) {
    by_prec(dtype_bits, [&](auto t) {
      using R = decltype(t);
      p->tw_x = upload_twiddles<R>(nx, sgpe::row_points_per_thread<R>(nx, p->row_shape), &e);
      if (e == cudaSuccess) p->tw_y = upload_twiddles<R>(ny, sgpe::col_points_per_thread<R>(ny, p->col_shape), &e);
      return 0;
    });
  }
  if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&p->derr), sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(p->derr, 0, sizeof(int));
  if (e != cudaSuccess) {
    sgpe_plan_destroy(p);
    return fail(SGPE_ERR_OOM, std::string("plan allocation: ") + cudaGetErrorString(e));
  }
  if (dtype_bits == 64) update_col_tmaps<float>(p);
  else if (dtype_bits == 128) update_col_tmaps<double>(p);
  *out = p;
  return SGPE_OK;
}

int sgpe_plan_destroy(sgpe_plan* p) {
  if (p == nullptr) return SGPE_OK;
  DeviceGuard g(p->device);
  drop_graphs(p);
  if (p->cap_stream) cudaStreamDestroy(p->cap_stream);
  for (int c = 0; c < 2; ++c) {
    if (p->s[c]) cudaFree(p->s[c]);
    if (p->scratch[c]) cudaFree(p->scratch[c]);
  }
  if (p->part) cudaFree(p->part);
  if (p->tw_x) cudaFree(p->tw_x);
  if (p->tw_y) cudaFree(p->tw_y);
  if (p->tw64_x) cudaFree(p->tw64_x);
  if (p->tw64_y) cudaFree(p->tw64_y);
  free_sub(p->sub[0]);
  free_sub(p->sub[1]);
  for (int i = 0; i < 2; ++i)
    for (int k = 0; k < 2; ++k) free_pair(p->pair[i][k]);
  free_efield(p->efield[0]);
  free_efield(p->efield[1]);
  for (int c = 0; c < 2; ++c)
    if (p->epsi[c]) cudaFree(p->epsi[c]);
  if (p->epart) cudaFree(p->epart);
  if (p->tcb) cudaFree(p->tcb);
  if (p->apart) cudaFree(p->apart);
  if (p->tmaps) cudaFree(p->tmaps);
  if (p->derr) cudaFree(p->derr);
  delete p;
  return SGPE_OK;
}

}  // extern "C"

namespace {
__global__ void __launch_bounds__(256) tc_bfrag_kernel(uint32_t* bfrag) {
  sgpe::tc_fill_bfrag(bfrag, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}

// One block waits, with the pass kernels' bounded wait, on an mbarrier phase
// that expects 16 bytes no copy will deliver; out[0] = 1 if every thread
// gave up, out[1] = the nanoseconds thread 0 waited.
__global__ void __launch_bounds__(64) wait_check_kernel(unsigned long long* out) {
  __shared__ __align__(8) uint64_t bar;
  __shared__ int gave_up;
  if (threadIdx.x == 0) {
    gave_up = 0;
    sgpe::mbar_init(&bar, 1);
  }
  __syncthreads();
  if (threadIdx.x == 0) sgpe::mbar_arrive_expect_tx(&bar, 16);
  const unsigned long long t0 = sgpe::global_ns();
  const bool done = sgpe::mbar_wait_bounded(&bar, 0);
  const unsigned long long t1 = sgpe::global_ns();
  if (!done) atomicAdd(&gave_up, 1);
  __syncthreads();
  if (threadIdx.x == 0) {
    out[0] = gave_up == int(blockDim.x) ? 1ull : 0ull;
    out[1] = t1 - t0;
  }
}
}  // namespace

extern "C" {

int sgpe_set_dft_mode(sgpe_plan* p, int mode) {
  if (p == nullptr) return fail(SGPE_ERR_ARG, "null plan");
  if (mode != 0 && mode != 1) return fail(SGPE_ERR_ARG, "dft mode must be 0 (FP32) or 1 (split-BF16 tensor cores)");
  if (mode == 1) {
    if (p->bits != 64) return fail(SGPE_ERR_ARG, "the tensor-core DFT16 variant is complex64 only");
    if (!sgpe::tc_size_supported(p->nx) || !sgpe::tc_size_supported(p->ny))
      return fail(SGPE_ERR_ARG, "the tensor-core DFT16 variant supports sides 64, 256, 1024 and 2048");
  }
  if (p->form == kMixed && p->pending_pops != nullptr)
    return fail(SGPE_ERR_STATE, "populations of the last step are pending; read the state first");
  if (mode == 1) {
    // the tensor-core kernels are built on shape 0 (radix-16 stages)
    const int rc = apply_shapes_any(p, 0, 0);
    if (rc != SGPE_OK) return rc;
  }
  if (mode == 1 && p->tcb == nullptr) {
    DeviceGuard g(p->device);
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&p->tcb), sizeof(uint32_t) * sgpe::kTcBfragWords);
    if (e == cudaSuccess) {
      tc_bfrag_kernel<<<8, 256>>>(p->tcb);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
      if (p->tcb) cudaFree(p->tcb);
      p->tcb = nullptr;
      return cuda_fail(e, "tensor-core DFT tables");
    }
  }
  p->tc = mode;
  p->ntile = mode ? p->nx / sgpe::tc_col_tile_width(p->ny) : p->ntile_fp32;
  drop_graphs(p);
  return SGPE_OK;
}

int sgpe_set_physics(sgpe_plan* p, double g_uu, double g_dd, double g_ud, double atom_num, double dv_r,
                     double dv_k, int is_coupling) {
  if (p == nullptr) return fail(SGPE_ERR_ARG, "null plan");
  if (!(atom_num > 0) || !(dv_r > 0) || !(dv_k > 0))
    return fail(SGPE_ERR_ARG, "atom_num, dv_r and dv_k must be positive");
  p->g[0] = g_uu;
  p->g[1] = g_dd;
  p->g[2] = g_ud;
  p->atom_num = atom_num;
  p->dv_r = dv_r;
  p->dv_k = dv_k;
  p->coupling = is_coupling ? 1 : 0;
  p->physics = true;
  drop_graphs(p);
  return SGPE_OK;
}

int sgpe_set_substep(sgpe_plan* p, int sub, const sgpe_substep_ops* ops) {
  if (p == nullptr || ops == nullptr) return fail(SGPE_ERR_ARG, "null plan or operators");
  if (sub != 0 && sub != 1) return fail(SGPE_ERR_ARG, "sub must be 0 (outer) or 1 (inner)");
  DeviceGuard g(p->device);
  SubOps so;
  int rc = SGPE_OK;
  const char* names[2] = {"0", "1"};
  for (int c = 0; c < 2 && rc == SGPE_OK; ++c) {
    rc = upload_field(p, ops->kin_a[c], &so.kin_a[c], &so, (std::string("kin_a") + names[c]).c_str());
    if (rc == SGPE_OK) rc = upload_field(p, ops->kin_b[c], &so.kin_b[c], &so, "kin_b");
    if (rc == SGPE_OK) rc = upload_field(p, ops->pot_a[c], &so.pot_a[c], &so, "pot_a");
    if (rc == SGPE_OK) rc = upload_field(p, ops->pot_b[c], &so.pot_b[c], &so, "pot_b");
  }
  if (rc == SGPE_OK) rc = upload_field(p, ops->cpl_c, &so.cc, &so, "cpl_c");
  if (rc == SGPE_OK) rc = upload_field(p, ops->cpl_s, &so.cs, &so, "cpl_s");
  if (rc == SGPE_OK) rc = upload_field(p, ops->cpl_e, &so.ce, &so, "cpl_e");
  if (rc == SGPE_OK) {
    // s conj(e) and s e in FP64, when the products stay compact (1-D or
    // uniform) or the factors are full fields anyway
    const HostField hs = host_copy(ops->cpl_s), he = host_copy(ops->cpl_e);
    HostField m01 = multiply_fields(hs, he, p->nx, p->ny, true);
    HostField m10 = multiply_fields(hs, he, p->nx, p->ny, false);
    const bool product_full = (m01.sx == 1 && m01.sy == p->nx);
    const bool factor_full = (hs.sx == 1 && hs.sy == p->nx) || (he.sx == 1 && he.sy == p->nx);
    if (!product_full || factor_full) {
      rc = upload_host_field(p, m01, &so.s01, &so.allocs);
      if (rc == SGPE_OK) rc = upload_host_field(p, m10, &so.s10, &so.allocs);
      so.has_s01 = (rc == SGPE_OK);
      so.s01_host = m01;
      so.s10_host = m10;
    }
  }
  if (rc != SGPE_OK) {
    free_sub(so);
    return rc;
  }
  for (int c = 0; c < 2; ++c) {
    const sgpe_field* src[2] = {&ops->kin_a[c], &ops->kin_b[c]};
    for (int k = 0; k < 2; ++k) {
      so.kin_host[c][k].v.assign(src[k]->data, src[k]->data + 2 * (size_t)src[k]->n);
      so.kin_host[c][k].sx = src[k]->sx;
      so.kin_host[c][k].sy = src[k]->sy;
    }
  }
  // factors with zero imaginary parts (imaginary time)
  so.kin_real = true;
  for (int c = 0; c < 2; ++c)
    for (int k = 0; k < 2; ++k) so.kin_real = so.kin_real && imag_zero(so.kin_host[c][k]);
  so.pot_real = true;
  for (int c = 0; c < 2; ++c)
    so.pot_real = so.pot_real && imag_zero(host_field(ops->pot_a[c])) && imag_zero(host_field(ops->pot_b[c]));
  so.cc_real = imag_zero(host_field(ops->cpl_c));
  // separable fast-path tables
  {
    const HostField ka[2] = {so.kin_host[0][0], so.kin_host[1][0]};
    const HostField kb[2] = {so.kin_host[0][1], so.kin_host[1][1]};
    rc = build_sep_kin(p, ka, kb, &so.sep, &so.allocs);
    HostField px[2], py[2];
    bool pot = (rc == SGPE_OK);
    for (int c = 0; c < 2 && pot; ++c)
      pot = split_xy(host_field(ops->pot_a[c]), host_field(ops->pot_b[c]), p->nx, p->ny, &px[c], &py[c]);
    for (int c = 0; c < 2 && pot && rc == SGPE_OK; ++c) {
      rc = upload_host_field(p, px[c], &so.sep.px[c], &so.allocs);
      if (rc == SGPE_OK) rc = upload_host_field(p, py[c], &so.sep.py[c], &so.allocs);
    }
    so.sep.pot = pot && rc == SGPE_OK;
    HostField s01x, s10x;
    const bool cc_uniform = ops->cpl_c.sx == 0 && ops->cpl_c.sy == 0;
    if (rc == SGPE_OK && cc_uniform && so.has_s01 && expand_1d(so.s01_host, 0, p->nx, p->ny, &s01x) &&
        expand_1d(so.s10_host, 0, p->nx, p->ny, &s10x)) {
      rc = upload_host_field(p, s01x, &so.sep.s01x, &so.allocs);
      if (rc == SGPE_OK) rc = upload_host_field(p, s10x, &so.sep.s10x, &so.allocs);
      so.sep.cpl = (rc == SGPE_OK);
    }
    if (rc == SGPE_OK && so.sep.pot) {
      const HostField hc = host_field(ops->cpl_c);
      rc = build_fused(p, px, py, so.sep.cpl ? &s01x : nullptr, so.sep.cpl ? &s10x : nullptr, hc.v[0],
                       hc.v[1], &so.sep, &so.allocs);
    }
    if (rc != SGPE_OK) {
      free_sub(so);
      return rc;
    }
  }
  so.zr = ops->int_z_re;
  so.zi = ops->int_z_im;
  so.set = true;
  free_sub(p->sub[sub]);
  p->sub[sub] = std::move(so);
  drop_graphs(p);
  for (int i = 0; i < 2; ++i) {
    free_pair(p->pair[sub][i]);
    free_pair(p->pair[i][sub]);
  }
  return SGPE_OK;
}

int sgpe_load_psik(sgpe_plan* p, const void* k0, const void* k1, void* stream) {
  if (p == nullptr || k0 == nullptr || k1 == nullptr) return fail(SGPE_ERR_ARG, "null plan or psik pointer");
  DeviceGuard g(p->device);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e;
  if (p->bits == SGPE_DTYPE_DF) {
    sgpe::DfCopyArgs d{};
    d.in[0] = k0;
    d.in[1] = k1;
    d.out[0] = p->s[0];
    d.out[1] = p->s[1];
    d.nx = p->nx;
    d.ny = p->ny;
    d.shift = 1;
    d.to_df = 1;
    df_copy_kernel<<<8 * 152, 256, 0, s>>>(d);
    e = cudaGetLastError();
  } else if (p->bits == 64) {
    sgpe::CopyArgs<float> c{};
    c.in[0] = cst<float>(k0);
    c.in[1] = cst<float>(k1);
    c.out[0] = st<float>(p->s[0]);
    c.out[1] = st<float>(p->s[1]);
    c.nx = p->nx;
    c.ny = p->ny;
    c.shift = 1;
    c.scale = 1.0f;
    e = sgpe::launch_copy<float>(c, s);
  } else {
    sgpe::CopyArgs<double> c{};
    c.in[0] = cst<double>(k0);
    c.in[1] = cst<double>(k1);
    c.out[0] = st<double>(p->s[0]);
    c.out[1] = st<double>(p->s[1]);
    c.nx = p->nx;
    c.ny = p->ny;
    c.shift = 1;
    c.scale = 1.0;
    e = sgpe::launch_copy<double>(c, s);
  }
  if (e != cudaSuccess) return cuda_fail(e, "load_psik");
  p->form = kKspace;
  p->pending_pops = nullptr;
  return SGPE_OK;
}

int sgpe_store_psik(sgpe_plan* p, void* o0, void* o1, double* pops, void* stream) {
  if (p == nullptr || o0 == nullptr || o1 == nullptr) return fail(SGPE_ERR_ARG, "null plan or psik pointer");
  if (p->form == kEmpty) return fail(SGPE_ERR_STATE, "no state loaded");
  DeviceGuard g(p->device);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  return by_prec(p->bits, [&](auto t) { return store<decltype(t)>(p, o0, o1, pops, s); });
}

int sgpe_single_step(sgpe_plan* p, int sub, void* stream) {
  if (p == nullptr) return fail(SGPE_ERR_ARG, "null plan");
  if (sub != 0 && sub != 1) return fail(SGPE_ERR_ARG, "sub must be 0 (outer) or 1 (inner)");
  if (p->form == kEmpty) return fail(SGPE_ERR_STATE, "no state loaded");
  if (!ready(p)) return fail(SGPE_ERR_STATE, "physics or sub-step operators not set");
  DeviceGuard g(p->device);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  return by_prec(p->bits, [&](auto t) { return substep<decltype(t)>(p, sub, nullptr, s); });
}

int sgpe_full_steps(sgpe_plan* p, int n_steps, double* pops, void* stream) {
  if (p == nullptr) return fail(SGPE_ERR_ARG, "null plan");
  if (n_steps < 0) return fail(SGPE_ERR_ARG, "n_steps must be non-negative");
  if (p->form == kEmpty) return fail(SGPE_ERR_STATE, "no state loaded");
  if (!ready(p)) return fail(SGPE_ERR_STATE, "physics or sub-step operators not set");
  DeviceGuard g(p->device);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int rc = by_prec(p->bits, [&](auto t) { return full_steps_impl<decltype(t)>(p, n_steps, pops, s); });
  if (rc != SGPE_OK) return rc;
  if (pops != nullptr && n_steps > 0) p->pending_pops = pops + 2 * (n_steps - 1);
  return SGPE_OK;
}

int sgpe_set_energy_fields(sgpe_plan* p, int slot, const sgpe_energy_fields* f) {
  if (p == nullptr || f == nullptr) return fail(SGPE_ERR_ARG, "null plan or fields");
  if (slot != 0 && slot != 1) return fail(SGPE_ERR_ARG, "slot must be 0 or 1");
  DeviceGuard g(p->device);
  EnergyFields ef;
  int rc = SGPE_OK;
  for (int c = 0; c < 2 && rc == SGPE_OK; ++c) {
    rc = upload_field64(p, f->kin_a[c], &ef.kin_a[c], &ef.allocs, "energy kin_a");
    if (rc == SGPE_OK) rc = upload_field64(p, f->kin_b[c], &ef.kin_b[c], &ef.allocs, "energy kin_b");
    if (rc == SGPE_OK) rc = upload_field64(p, f->pot_a[c], &ef.pot_a[c], &ef.allocs, "energy pot_a");
    if (rc == SGPE_OK) rc = upload_field64(p, f->pot_b[c], &ef.pot_b[c], &ef.allocs, "energy pot_b");
  }
  if (rc == SGPE_OK) rc = upload_field64(p, f->cpl, &ef.cpl, &ef.allocs, "energy cpl");
  if (rc != SGPE_OK) {
    free_efield(ef);
    return rc;
  }
  ef.set = true;
  free_efield(p->efield[slot]);
  p->efield[slot] = std::move(ef);
  return SGPE_OK;
}

int sgpe_energy(sgpe_plan* p, int slot, const void* k0, const void* k1, double* out, void* stream) {
  if (p == nullptr || k0 == nullptr || k1 == nullptr || out == nullptr)
    return fail(SGPE_ERR_ARG, "null plan, psik or output pointer");
  if (slot != 0 && slot != 1) return fail(SGPE_ERR_ARG, "slot must be 0 or 1");
  if (!p->efield[slot].set) return fail(SGPE_ERR_STATE, "energy fields of this slot not set");
  if (!p->physics) return fail(SGPE_ERR_STATE, "physics not set");
  DeviceGuard g(p->device);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  return by_iface(p->bits, [&](auto t) { return energy_impl<decltype(t)>(p, slot, k0, k1, out, s); });
}

}  // extern "C"

namespace {
template <typename R>
int analysis_impl(sgpe_plan* p, const void* const* in, void* const* out, double* sums, cudaStream_t s) {
  using C = sgpe::Cx<R>;
  sgpe::AnalysisArgs<R> a{};
  for (int c = 0; c < 2; ++c) {
    a.psi[c] = static_cast<const C*>(in[c]);
    a.psik[c] = static_cast<const C*>(in[2 + c]);
    a.dens[c] = static_cast<R*>(out[c]);
    a.densk[c] = static_cast<R*>(out[2 + c]);
    a.phase[c] = static_cast<R*>(out[4 + c]);
  }
  a.n = (long long)p->nx * p->ny;
  a.part = p->apart;
  a.sums = sums;
  sgpe::analysis_dens_kernel<R><<<sgpe::kAnalysisBlocks, 256, 0, s>>>(a);
  sgpe::analysis_finalize_kernel<<<1, 32, 0, s>>>(p->apart, sgpe::kAnalysisBlocks, sums);
  sgpe::analysis_phase_kernel<R><<<sgpe::kAnalysisBlocks, 256, 0, s>>>(a);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? SGPE_OK : cuda_fail(e, "analysis");
}
}  // namespace

extern "C" {

int sgpe_analysis(sgpe_plan* p, const void* psi0, const void* psi1, const void* psik0, const void* psik1,
                  void* dens0, void* dens1, void* densk0, void* densk1, void* phase0, void* phase1,
                  double* sums_dev, void* stream) {
  if (p == nullptr || !psi0 || !psi1 || !psik0 || !psik1 || !dens0 || !dens1 || !densk0 || !densk1 || !phase0 ||
      !phase1 || !sums_dev)
    return fail(SGPE_ERR_ARG, "null plan or data pointer");
  DeviceGuard g(p->device);
  if (p->apart == nullptr) {
    const cudaError_t e =
        cudaMalloc(reinterpret_cast<void**>(&p->apart), sizeof(double) * sgpe::kAnalysisBlocks * sgpe::kAnalysisSums);
    if (e != cudaSuccess) return fail(SGPE_ERR_OOM, std::string("analysis partials: ") + cudaGetErrorString(e));
  }
  const void* in[4] = {psi0, psi1, psik0, psik1};
  void* out[6] = {dens0, dens1, densk0, densk1, phase0, phase1};
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  return by_iface(p->bits, [&](auto t) { return analysis_impl<decltype(t)>(p, in, out, sums_dev, s); });
}

int sgpe_time_passes(sgpe_plan* p, int n_steps, double* col_ms, double* row_ms, void* stream) {
  if (p == nullptr || col_ms == nullptr || row_ms == nullptr || n_steps < 1)
    return fail(SGPE_ERR_ARG, "null plan/outputs or n_steps < 1");
  if (p->form == kEmpty) return fail(SGPE_ERR_STATE, "no state loaded");
  if (!ready(p)) return fail(SGPE_ERR_STATE, "physics or sub-step operators not set");
  DeviceGuard g(p->device);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // reach the steady state (mixed form after an outer sub-step) eagerly
  if (!(p->form == kMixed && p->prev_sub == 0 && p->pending_pops == nullptr)) {
    const int rc = by_prec(p->bits, [&](auto t) { return eager_step<decltype(t)>(p, nullptr, s); });
    if (rc != SGPE_OK) return rc;
  }
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b)
      if (ensure_pair(p, a, b) != SGPE_OK) return SGPE_ERR_OOM;
  if (p->cap_stream == nullptr) {
    cudaError_t e = cudaStreamCreateWithFlags(&p->cap_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_fail(e, "graph stream");
  }
  // Capture n_steps steps with timing events around every pass (external
  // event-record nodes), so that the measured intervals are device time
  // between back-to-back graph nodes.
  const int n_pass = 3 * n_steps;
  std::vector<cudaEvent_t> ev(4 * n_pass, nullptr);
  cudaError_t e = cudaSuccess;
  for (auto& x : ev)
    if (e == cudaSuccess) e = cudaEventCreate(&x);
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t cs = p->cap_stream;
  if (e == cudaSuccess) e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    for (int i = 0; i < n_pass && e == cudaSuccess; ++i) {
      const int sub = (i % 3 == 1) ? 1 : 0;
      e = cudaEventRecordWithFlags(ev[4 * i + 0], cs, cudaEventRecordExternal);
      if (e == cudaSuccess)
        e = by_prec(p->bits, [&](auto t) { return col_pass_step<decltype(t)>(p, sub, nullptr, cs); });
      if (e == cudaSuccess) e = cudaEventRecordWithFlags(ev[4 * i + 1], cs, cudaEventRecordExternal);
      if (e == cudaSuccess) e = cudaEventRecordWithFlags(ev[4 * i + 2], cs, cudaEventRecordExternal);
      if (e == cudaSuccess)
        e = by_prec(p->bits, [&](auto t) { return row_pass_step<decltype(t)>(p, sub, nullptr, cs); });
      if (e == cudaSuccess) e = cudaEventRecordWithFlags(ev[4 * i + 3], cs, cudaEventRecordExternal);
      p->form = kMixed;
      p->prev_sub = sub;
    }
    const cudaError_t e2 = cudaStreamEndCapture(cs, &graph);
    if (e == cudaSuccess) e = e2;
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
  if (e == cudaSuccess) e = cudaGraphLaunch(exec, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  double tc = 0.0, tr = 0.0;
  for (int i = 0; i < n_pass && e == cudaSuccess; ++i) {
    float a = 0.f, b = 0.f;
    e = cudaEventElapsedTime(&a, ev[4 * i + 0], ev[4 * i + 1]);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&b, ev[4 * i + 2], ev[4 * i + 3]);
    tc += a;
    tr += b;
  }
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  for (auto& x : ev)
    if (x) cudaEventDestroy(x);
  if (e != cudaSuccess) return cuda_fail(e, "time_passes");
  *col_ms = tc / n_pass;
  *row_ms = tr / n_pass;
  return SGPE_OK;
}

int sgpe_check_bounded_wait(int* gave_up, double* waited_ms) {
  if (gave_up == nullptr || waited_ms == nullptr) return fail(SGPE_ERR_ARG, "null output");
  unsigned long long* d = nullptr;
  cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&d), 2 * sizeof(unsigned long long));
  if (e != cudaSuccess) return cuda_fail(e, "bounded-wait check");
  unsigned long long h[2] = {0, 0};
  wait_check_kernel<<<1, 64>>>(d);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return cuda_fail(e, "bounded-wait check");
  *gave_up = int(h[0]);
  *waited_ms = double(h[1]) * 1e-6;
  return SGPE_OK;
}

int sgpe_device_status(sgpe_plan* p, int* status) {
  if (p == nullptr || status == nullptr) return fail(SGPE_ERR_ARG, "null plan or status");
  DeviceGuard g(p->device);
  int h = 0;
  const cudaError_t e = cudaMemcpy(&h, p->derr, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "device status");
  *status = h;
  if (h != 0) return fail(SGPE_ERR_CUDA, "a pass kernel gave up waiting for its bulk copies (device error word " +
                                             std::to_string(h) + "); results of that pass are not reliable");
  return SGPE_OK;
}

int sgpe_shape_count(int dtype_bits, int axis, int n) {
  if ((dtype_bits != 64 && dtype_bits != 128 && dtype_bits != SGPE_DTYPE_DF) || (axis != 0 && axis != 1)) return 0;
  return shape_count(dtype_bits, axis, n);
}

int sgpe_set_shapes(sgpe_plan* p, int row_shape, int col_shape) {
  if (p == nullptr) return fail(SGPE_ERR_ARG, "null plan");
  if (p->form == kMixed && p->pending_pops != nullptr)
    return fail(SGPE_ERR_STATE, "populations of the last step are pending; read the state first");
  return apply_shapes_any(p, row_shape, col_shape);
}

int sgpe_get_shapes(const sgpe_plan* p, int* row_shape, int* col_shape) {
  if (p == nullptr || row_shape == nullptr || col_shape == nullptr) return fail(SGPE_ERR_ARG, "null argument");
  *row_shape = p->row_shape;
  *col_shape = p->col_shape;
  return SGPE_OK;
}

int sgpe_autotune(sgpe_plan* p, int n_steps, int* row_shape, int* col_shape, double* step_us, void* stream) {
  if (p == nullptr || row_shape == nullptr || col_shape == nullptr || n_steps < 1)
    return fail(SGPE_ERR_ARG, "null plan/outputs or n_steps < 1");
  if (p->form == kEmpty) return fail(SGPE_ERR_STATE, "no state loaded");
  if (!ready(p)) return fail(SGPE_ERR_STATE, "physics or sub-step operators not set");
  if (p->form == kMixed && p->pending_pops != nullptr)
    return fail(SGPE_ERR_STATE, "populations of the last step are pending; read the state first");
  DeviceGuard g(p->device);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  constexpr int M = sgpe::kMaxShapes;
  if (step_us != nullptr)
    for (int i = 0; i < M * M; ++i) step_us[i] = -1.0;
  const int nr = shape_count(p->bits, 0, p->nx), nc = shape_count(p->bits, 1, p->ny);
  const int r0 = p->row_shape, c0 = p->col_shape;
  *row_shape = r0;
  *col_shape = c0;
  if (p->tc || (nr <= 1 && nc <= 1)) return SGPE_OK;
  // the state is saved and every candidate starts from it; the plan ends
  // with the saved state in the chosen shapes
  const size_t bytes = p->elem * (size_t)p->nx * p->ny;
  for (int c = 0; c < 2; ++c) {
    if (p->scratch[c] == nullptr) {
      cudaError_t e = cudaMalloc(&p->scratch[c], bytes);
      if (e != cudaSuccess) return fail(SGPE_ERR_OOM, std::string("autotune scratch: ") + cudaGetErrorString(e));
    }
  }
  const int form0 = p->form, prev0 = p->prev_sub;
  auto restore = [&](void* const* from, void* const* to) {
    cudaError_t e = cudaSuccess;
    for (int c = 0; c < 2 && e == cudaSuccess; ++c) e = cudaMemcpyAsync(to[c], from[c], bytes, cudaMemcpyDeviceToDevice, s);
    return e;
  };
  cudaError_t e = restore(p->s, p->scratch);
  cudaEvent_t ev[2] = {nullptr, nullptr};
  for (auto& x : ev)
    if (e == cudaSuccess) e = cudaEventCreate(&x);
  std::vector<double> t(M * M, -1.0);
  int rc = e == cudaSuccess ? SGPE_OK : cuda_fail(e, "autotune set-up");
  for (int round = 0; round < 2 && rc == SGPE_OK; ++round)
    for (int r = 0; r < nr && rc == SGPE_OK; ++r)
      for (int c = 0; c < nc && rc == SGPE_OK; ++c) {
        if (apply_shapes_any(p, r, c) != SGPE_OK) continue;  // tile width does not divide nx
        e = restore(p->scratch, p->s);
        if (e != cudaSuccess) {
          rc = cuda_fail(e, "autotune restore");
          break;
        }
        p->form = form0;
        p->prev_sub = prev0;
        p->pending_pops = nullptr;
        // warm-up: reaches the steady state and captures both step graphs
        rc = by_prec(p->bits, [&](auto t) { return full_steps_impl<decltype(t)>(p, kGraphSteps + 2, nullptr, s); });
        if (rc != SGPE_OK) break;
        e = cudaEventRecord(ev[0], s);
        if (e == cudaSuccess) {
          rc = by_prec(p->bits, [&](auto t) { return full_steps_impl<decltype(t)>(p, n_steps, nullptr, s); });
          if (rc != SGPE_OK) break;
          e = cudaEventRecord(ev[1], s);
        }
        if (e == cudaSuccess) e = cudaEventSynchronize(ev[1]);
        float ms = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, ev[0], ev[1]);
        if (e != cudaSuccess) {
          rc = cuda_fail(e, "autotune timing");
          break;
        }
        const double us = 1e3 * ms / n_steps;
        double& slot = t[r * M + c];
        slot = (slot < 0 || us < slot) ? us : slot;
      }
  for (auto& x : ev)
    if (x) cudaEventDestroy(x);
  // fastest shapes; the plan's own stay unless another is >2% faster
  int br = r0, bc = c0;
  double bt = t[r0 * M + c0];
  for (int i = 0; i < M * M; ++i)
    if (t[i] > 0 && (bt < 0 || t[i] < bt)) {
      bt = t[i];
      br = i / M;
      bc = i % M;
    }
  if (t[r0 * M + c0] > 0 && t[r0 * M + c0] <= 1.02 * bt) {
    br = r0;
    bc = c0;
  }
  if (rc != SGPE_OK) {
    br = r0;
    bc = c0;
  }
  const int rc2 = apply_shapes_any(p, br, bc);
  e = restore(p->scratch, p->s);
  p->form = form0;
  p->prev_sub = prev0;
  p->pending_pops = nullptr;
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (rc != SGPE_OK) return rc;
  if (rc2 != SGPE_OK) return rc2;
  if (e != cudaSuccess) return cuda_fail(e, "autotune restore");
  *row_shape = br;
  *col_shape = bc;
  if (step_us != nullptr)
    for (int i = 0; i < M * M; ++i) step_us[i] = t[i];
  return SGPE_OK;
}

int sgpe_batch_create(sgpe_batch** out, sgpe_plan* const* plans, int n_plans) {
  if (out == nullptr || plans == nullptr || n_plans < 1) return fail(SGPE_ERR_ARG, "null output/plans or no plans");
  *out = nullptr;
  for (int i = 0; i < n_plans; ++i) {
    if (plans[i] == nullptr) return fail(SGPE_ERR_ARG, "null plan in batch");
    if (plans[i]->device != plans[0]->device) return fail(SGPE_ERR_ARG, "batch plans must share a device");
    for (int k = 0; k < i; ++k)
      if (plans[k] == plans[i]) return fail(SGPE_ERR_ARG, "a plan appears twice in the batch");
  }
  DeviceGuard g(plans[0]->device);
  sgpe_batch* b = new sgpe_batch();
  b->plans.assign(plans, plans + n_plans);
  b->device = plans[0]->device;
  const char* env = std::getenv("SGPE_BATCH_GROUPING");
  b->grouping = !(env != nullptr && env[0] == '0');
  cudaError_t e = cudaStreamCreateWithFlags(&b->root, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
  b->joins.assign(n_plans, nullptr);
  for (int i = 0; i < n_plans && e == cudaSuccess; ++i) e = cudaEventCreateWithFlags(&b->joins[i], cudaEventDisableTiming);
  for (int i = 0; i < n_plans && e == cudaSuccess; ++i)
    if (plans[i]->cap_stream == nullptr) e = cudaStreamCreateWithFlags(&plans[i]->cap_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    sgpe_batch_destroy(b);
    return cuda_fail(e, "batch create");
  }
  *out = b;
  return SGPE_OK;
}

namespace {
void free_groups(sgpe_batch* b) {
  for (BatchGroup& g : b->groups) {
    if (g.col_args) cudaFree(g.col_args);
    if (g.row_args) cudaFree(g.row_args);
    if (g.join) cudaEventDestroy(g.join);
    if (g.stream) cudaStreamDestroy(g.stream);
  }
  b->groups.clear();
  b->groups_built = false;
}
}  // namespace

namespace {
void free_queue_args(sgpe_batch* b) {
  for (void* x : {b->q_solves, b->q_col, b->q_row, static_cast<void*>(b->q_first)})
    if (x) cudaFree(x);
  b->q_solves = b->q_col = b->q_row = nullptr;
  b->q_first = nullptr;
  b->q_built = false;
}
}  // namespace

int sgpe_batch_destroy(sgpe_batch* b) {
  if (b == nullptr) return SGPE_OK;
  DeviceGuard g(b->device);
  for (auto& x : b->graph)
    if (x) cudaGraphExecDestroy(x);
  free_groups(b);
  free_queue_args(b);
  if (b->q_words) cudaFree(b->q_words);
  for (void* t : b->q_tw)
    if (t) cudaFree(t);
  for (auto& ev : b->joins)
    if (ev) cudaEventDestroy(ev);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->root) cudaStreamDestroy(b->root);
  delete b;
  return SGPE_OK;
}

extern "C++" {
namespace {
// Device argument arrays of a group's steady-state passes (the same
// arguments the plans' own steps use, so results are identical).
template <typename R> int upload_group_args(sgpe_batch* b, BatchGroup& g) {
  const size_t G = g.members.size();
  std::vector<sgpe::ColArgs<R>> col(3 * G);
  std::vector<sgpe::RowArgs<R>> row(2 * G);
  const int prevs[3] = {0, 0, 1}, subs[3] = {0, 1, 0};
  for (size_t i = 0; i < G; ++i) {
    sgpe_plan* p = b->plans[g.members[i]];
    const int saved = p->prev_sub;
    bool ok = true;
    for (int v = 0; v < 3 && ok; ++v) {
      p->prev_sub = prevs[v];
      ok = col_step_args<R>(p, subs[v], false, &col[v * G + i]);
    }
    p->prev_sub = saved;
    if (!ok) return fail(SGPE_ERR_OOM, "batch: merged kinetic tables");
    for (int sub = 0; sub < 2; ++sub) row[sub * G + i] = row_step_args<R>(p, sub, nullptr);
  }
  cudaError_t e = cudaMalloc(&g.col_args, sizeof(sgpe::ColArgs<R>) * col.size());
  if (e == cudaSuccess) e = cudaMalloc(&g.row_args, sizeof(sgpe::RowArgs<R>) * row.size());
  if (e == cudaSuccess)
    e = cudaMemcpy(g.col_args, col.data(), sizeof(sgpe::ColArgs<R>) * col.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(g.row_args, row.data(), sizeof(sgpe::RowArgs<R>) * row.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && g.stream == nullptr) e = cudaStreamCreateWithFlags(&g.stream, cudaStreamNonBlocking);
  if (e == cudaSuccess && g.join == nullptr) e = cudaEventCreateWithFlags(&g.join, cudaEventDisableTiming);
  return e == cudaSuccess ? SGPE_OK : cuda_fail(e, "batch group arguments");
}

// `steps` steady-state full steps of a group as grouped launches on its
// stream: per sub-step one column-pass and one row-pass launch for all
// members.
template <typename R> int launch_group_steps(const BatchGroup& g, int steps) {
  const int G = int(g.members.size());
  const auto* col = static_cast<const sgpe::ColArgs<R>*>(g.col_args);
  const auto* row = static_cast<const sgpe::RowArgs<R>*>(g.row_args);
  const int cv[3] = {0, 1, 2}, rs[3] = {0, 1, 0};
  for (int k = 0; k < steps; ++k)
    for (int t = 0; t < 3; ++t) {
      cudaError_t e = sgpe::launch_col_grouped<R>(col + cv[t] * G, g.col_shape, G, g.nx, g.ny, g.stream);
      if (e == cudaSuccess)
        e = sgpe::launch_row_grouped<R>(row + rs[t] * G, g.row_shape, G, g.nx, g.ny, g.stream);
      if (e != cudaSuccess) return cuda_fail(e, "batch grouped pass");
    }
  return SGPE_OK;
}

// Plans that can share grouped launches: equal size, precision and kernel
// shapes, and separable real-space operators in both sub-steps (the grouped row kernels
// carry the separable point-wise code).
void build_groups(sgpe_batch* b) {
  std::vector<bool> taken(b->plans.size(), false);
  for (size_t i = 0; i < b->plans.size(); ++i) {
    if (taken[i]) continue;
    sgpe_plan* p = b->plans[i];
    auto sep = [](const sgpe_plan* q) {
      if (q->tc) return false;  // the grouped kernels carry the FP32 DFTs
      if (q->bits == SGPE_DTYPE_DF) return false;  // no grouped double-float kernels
      for (int sub = 0; sub < 2; ++sub)
        if (!fused_sep(q->sub[sub], q->coupling)) return false;
      return true;
    };
    if (!b->grouping || !sep(p)) continue;
    BatchGroup g;
    g.nx = p->nx;
    g.ny = p->ny;
    g.bits = p->bits;
    g.row_shape = p->row_shape;
    g.col_shape = p->col_shape;
    for (size_t k = i; k < b->plans.size(); ++k) {
      const sgpe_plan* q = b->plans[k];
      if (!taken[k] && q->nx == p->nx && q->ny == p->ny && q->bits == p->bits && q->row_shape == p->row_shape &&
          q->col_shape == p->col_shape && sep(q))
        g.members.push_back(int(k));
    }
    if (g.members.size() < 2) continue;
    for (int k : g.members) taken[k] = true;
    b->groups.push_back(g);
  }
}

// Capture `steps` steady-state steps of every plan as parallel branches:
// one branch per group of grouped launches, one per remaining plan.
int capture_batch(sgpe_batch* b, int steps, cudaGraphExec_t* out) {
  for (sgpe_plan* p : b->plans)
    for (int x = 0; x < 2; ++x)
      for (int y = 0; y < 2; ++y)
        if (ensure_pair(p, x, y) != SGPE_OK) return SGPE_ERR_OOM;
  // The groups' argument arrays are shared by the 1-step and the 8-step
  // graph.  They are rebuilt only when some plan's operators changed; the
  // other graph, which points at the old arrays, is dropped first.
  std::vector<unsigned long long> now;
  for (const sgpe_plan* p : b->plans) now.push_back(p->epoch);
  if (!b->groups_built || b->groups_epoch != now) {
    for (auto& x : b->graph)
      if (x != nullptr && &x != out) {
        cudaGraphExecDestroy(x);
        x = nullptr;
      }
    free_groups(b);  // cudaFree waits for launches still reading them
    build_groups(b);
    for (BatchGroup& g : b->groups) {
      const int rc = g.bits == 64 ? upload_group_args<float>(b, g) : upload_group_args<double>(b, g);
      if (rc != SGPE_OK) {
        free_groups(b);
        return rc;
      }
    }
    b->groups_epoch = now;
    b->groups_built = true;
  }
  std::vector<bool> grouped(b->plans.size(), false);
  for (const BatchGroup& g : b->groups)
    for (int k : g.members) grouped[k] = true;
  cudaError_t e = cudaStreamBeginCapture(b->root, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return cuda_fail(e, "batch begin capture");
  if (e == cudaSuccess) e = cudaEventRecord(b->fork, b->root);
  int rc = SGPE_OK;
  for (size_t i = 0; i < b->groups.size() && e == cudaSuccess && rc == SGPE_OK; ++i) {
    BatchGroup& g = b->groups[i];
    e = cudaStreamWaitEvent(g.stream, b->fork, 0);
    if (e == cudaSuccess) rc = g.bits == 64 ? launch_group_steps<float>(g, steps) : launch_group_steps<double>(g, steps);
    if (e == cudaSuccess && rc == SGPE_OK) e = cudaEventRecord(g.join, g.stream);
    if (e == cudaSuccess && rc == SGPE_OK) e = cudaStreamWaitEvent(b->root, g.join, 0);
  }
  for (size_t i = 0; i < b->plans.size() && e == cudaSuccess && rc == SGPE_OK; ++i) {
    if (grouped[i]) continue;
    sgpe_plan* p = b->plans[i];
    e = cudaStreamWaitEvent(p->cap_stream, b->fork, 0);
    for (int k = 0; k < steps && e == cudaSuccess && rc == SGPE_OK; ++k)
      rc = by_prec(p->bits, [&](auto t) { return eager_step<decltype(t)>(p, nullptr, p->cap_stream); });
    if (e == cudaSuccess && rc == SGPE_OK) e = cudaEventRecord(b->joins[i], p->cap_stream);
    if (e == cudaSuccess && rc == SGPE_OK) e = cudaStreamWaitEvent(b->root, b->joins[i], 0);
  }
  cudaGraph_t graph = nullptr;
  const cudaError_t e2 = cudaStreamEndCapture(b->root, &graph);
  if (e == cudaSuccess) e = e2;
  if (rc != SGPE_OK || e != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    return rc != SGPE_OK ? rc : cuda_fail(e, "batch capture");
  }
  e = cudaGraphInstantiate(out, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return cuda_fail(e, "batch graph instantiate");
  std::vector<unsigned long long>& ep = b->epoch[steps == 1 ? 0 : 1];
  ep.clear();
  for (sgpe_plan* p : b->plans) ep.push_back(p->epoch);
  return SGPE_OK;
}

// Why plan p cannot run in the queue kernel (nullptr: it can): complex64
// FP32 transforms with the fused separable operators, sides among the
// queue's line lengths, and tiles that divide the grid.
const char* queue_unsupported(const sgpe_plan* p) {
  if (p->bits != 64) return "the work queue runs complex64 plans only";
  if (p->tc) return "the work queue runs the FP32 transforms only";
  for (int sub = 0; sub < 2; ++sub)
    if (!fused_sep(p->sub[sub], p->coupling)) return "the work queue needs separable operators";
  if (sgpe::queue_class(p->nx) < 0 || sgpe::queue_class(p->ny) < 0)
    return "the work queue takes sides 128, 192, 256, 384, 512, 768 and 1024";
  if (p->nx % sgpe::queue_cols(p->ny) != 0 || p->ny % sgpe::queue_rows(p->nx) != 0)
    return "the work queue's tiles do not divide this grid";
  return nullptr;
}

// Device arguments of the queue kernel: per solve the column-pass arguments
// of the three sub-steps and the row-pass arguments of the two sub-step
// kinds (the plans' own, with the queue shapes' twiddle tables and tile
// counts), and the first item of each solve in a column and a row phase.
int queue_build(sgpe_batch* b) {
  free_queue_args(b);
  const int n = int(b->plans.size());
  std::vector<sgpe::ColArgs<float>> col(3 * n);
  std::vector<sgpe::RowArgs<float>> row(2 * n);
  std::vector<sgpe::QueueSolve> sv(n);
  std::vector<int> first(2 * (n + 1), 0);
  const int prevs[3] = {0, 0, 1}, subs[3] = {0, 1, 0};
  cudaError_t e = cudaSuccess;
  for (int i = 0; i < n && e == cudaSuccess; ++i) {
    sgpe_plan* p = b->plans[i];
    const int cx = sgpe::queue_class(p->nx), cy = sgpe::queue_class(p->ny);
    for (int c : {cx, cy})
      if (b->q_tw[c] == nullptr && e == cudaSuccess) {
        const int len = sgpe::queue_size(c);
        b->q_tw[c] = upload_twiddles<float>(len, sgpe::queue_e(len), &e);
      }
    if (e != cudaSuccess) break;
    const int tiles = p->nx / sgpe::queue_cols(p->ny);
    const int rows = p->ny / sgpe::queue_rows(p->nx);
    const int saved = p->prev_sub;
    bool ok = true;
    for (int v = 0; v < 3 && ok; ++v) {
      p->prev_sub = prevs[v];
      ok = col_step_args<float>(p, subs[v], false, &col[3 * i + v]);
      col[3 * i + v].tw = static_cast<const float2*>(b->q_tw[cy]);
      col[3 * i + v].tmap = nullptr;
    }
    p->prev_sub = saved;
    if (!ok) return fail(SGPE_ERR_OOM, "work queue: merged kinetic tables");
    for (int sub = 0; sub < 2; ++sub) {
      row[2 * i + sub] = row_step_args<float>(p, sub, nullptr);
      row[2 * i + sub].tw = static_cast<const float2*>(b->q_tw[cx]);
      row[2 * i + sub].ntile = tiles;
    }
    sv[i].cls_x = cx;
    sv[i].cls_y = cy;
    sv[i].col_tiles = tiles;
    sv[i].row_items = rows;
    first[i + 1] = first[i] + 2 * tiles;
    first[(n + 1) + i + 1] = first[(n + 1) + i] + rows;
  }
  if (e != cudaSuccess) return cuda_fail(e, "work queue twiddles");
  e = cudaMalloc(&b->q_col, sizeof(sgpe::ColArgs<float>) * col.size());
  if (e == cudaSuccess) e = cudaMalloc(&b->q_row, sizeof(sgpe::RowArgs<float>) * row.size());
  if (e == cudaSuccess) e = cudaMalloc(&b->q_solves, sizeof(sgpe::QueueSolve) * sv.size());
  if (e == cudaSuccess) e = cudaMalloc(&b->q_first, sizeof(int) * first.size());
  if (e == cudaSuccess) {
    for (int i = 0; i < n; ++i) {
      sv[i].col = static_cast<const sgpe::ColArgs<float>*>(b->q_col) + 3 * i;
      sv[i].row = static_cast<const sgpe::RowArgs<float>*>(b->q_row) + 2 * i;
    }
    e = cudaMemcpy(b->q_col, col.data(), sizeof(sgpe::ColArgs<float>) * col.size(), cudaMemcpyHostToDevice);
  }
  if (e == cudaSuccess)
    e = cudaMemcpy(b->q_row, row.data(), sizeof(sgpe::RowArgs<float>) * row.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(b->q_solves, sv.data(), sizeof(sgpe::QueueSolve) * sv.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(b->q_first, first.data(), sizeof(int) * first.size(), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    free_queue_args(b);
    return cuda_fail(e, "work queue arguments");
  }
  b->q_built = true;
  b->q_epoch.clear();
  for (const sgpe_plan* p : b->plans) b->q_epoch.push_back(p->epoch);
  return SGPE_OK;
}

// Enqueue `steps` steps as one launch of the queue kernel on s: reset the
// claim counter, the abort flag and the finished-item counters, then launch.
cudaError_t queue_enqueue(sgpe_batch* b, int steps, cudaStream_t s) {
  const int n = int(b->plans.size());
  sgpe::QueueArgs q{};
  q.solves = static_cast<const sgpe::QueueSolve*>(b->q_solves);
  q.col_first = b->q_first;
  q.row_first = b->q_first + (n + 1);
  q.n = n;
  q.phases = 6 * steps;
  q.err = reinterpret_cast<int*>(b->q_words);
  q.claim = b->q_words + 1;
  q.abort = reinterpret_cast<int*>(b->q_words + 2);
  q.done = b->q_words + 3;
  cudaError_t e =
      cudaMemsetAsync(b->q_words + 1, 0, sizeof(unsigned) * (2 + size_t(n) * 6 * kGraphSteps), s);
  if (e == cudaSuccess) e = sgpe::launch_batch_queue(q, b->q_grid, s);
  return e;
}

// Capture `steps` queue steps as a graph (the cooperative launch as a
// kernel node); when the capture is refused the steps are launched directly.
int capture_queue(sgpe_batch* b, int steps, cudaGraphExec_t* out) {
  cudaError_t e = cudaStreamBeginCapture(b->root, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return cuda_fail(e, "queue begin capture");
  const cudaError_t el = queue_enqueue(b, steps, b->root);
  cudaGraph_t graph = nullptr;
  const cudaError_t e2 = cudaStreamEndCapture(b->root, &graph);
  if (el != cudaSuccess || e2 != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    cudaGetLastError();
    b->q_direct = true;
    return SGPE_OK;
  }
  e = cudaGraphInstantiate(out, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    cudaGetLastError();
    b->q_direct = true;
    return SGPE_OK;
  }
  std::vector<unsigned long long>& ep = b->epoch[steps == 1 ? 0 : 1];
  ep.clear();
  for (sgpe_plan* p : b->plans) ep.push_back(p->epoch);
  return SGPE_OK;
}

// True when some plan's physics or operators changed since graph k was
// captured.
bool batch_stale(const sgpe_batch* b, int k) {
  if (b->epoch[k].size() != b->plans.size()) return true;
  for (size_t i = 0; i < b->plans.size(); ++i)
    if (b->plans[i]->epoch != b->epoch[k][i]) return true;
  return false;
}
}  // namespace
}  // extern "C++"

int sgpe_batch_steps(sgpe_batch* b, int n_steps, void* stream) {
  if (b == nullptr) return fail(SGPE_ERR_ARG, "null batch");
  if (n_steps < 0) return fail(SGPE_ERR_ARG, "n_steps must be non-negative");
  for (sgpe_plan* p : b->plans) {
    if (p->form == kEmpty) return fail(SGPE_ERR_STATE, "a batch plan has no state loaded");
    if (!ready(p)) return fail(SGPE_ERR_STATE, "a batch plan has no physics or operators");
  }
  DeviceGuard g(b->device);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int done = 0;
  // bring every plan to the steady state with one eager step (on `s`)
  bool eager = false;
  for (sgpe_plan* p : b->plans)
    if (!(p->form == kMixed && p->prev_sub == 0 && p->pending_pops == nullptr)) eager = true;
  if (eager && n_steps > 0) {
    for (sgpe_plan* p : b->plans) {
      const int rc = by_prec(p->bits, [&](auto t) { return eager_step<decltype(t)>(p, nullptr, s); });
      if (rc != SGPE_OK) return rc;
    }
    done = 1;
  }
  if (b->queue && done < n_steps) {
    std::vector<unsigned long long> now;
    for (const sgpe_plan* p : b->plans) now.push_back(p->epoch);
    if (!b->q_built || b->q_epoch != now) {
      for (auto& x : b->graph)
        if (x != nullptr) {
          cudaGraphExecDestroy(x);
          x = nullptr;
        }
      for (sgpe_plan* p : b->plans)
        for (int x = 0; x < 2; ++x)
          for (int y = 0; y < 2; ++y)
            if (ensure_pair(p, x, y) != SGPE_OK) return fail(SGPE_ERR_OOM, "work queue: merged kinetic tables");
      cudaError_t e = cudaStreamSynchronize(s);  // launches still reading the old arguments
      if (e != cudaSuccess) return cuda_fail(e, "work queue rebuild");
      const int rc = queue_build(b);
      if (rc != SGPE_OK) return rc;
    }
  }
  while (done < n_steps) {
    const int k = (n_steps - done >= kGraphSteps) ? 1 : 0;
    if (b->graph[k] != nullptr && batch_stale(b, k)) {
      cudaGraphExecDestroy(b->graph[k]);
      b->graph[k] = nullptr;
    }
    if (b->queue && b->q_direct) {
      const cudaError_t e = queue_enqueue(b, k ? kGraphSteps : 1, s);
      if (e != cudaSuccess) return cuda_fail(e, "work queue launch");
      done += k ? kGraphSteps : 1;
      continue;
    }
    if (b->graph[k] == nullptr) {
      const int rc = b->queue ? capture_queue(b, k ? kGraphSteps : 1, &b->graph[k])
                              : capture_batch(b, k ? kGraphSteps : 1, &b->graph[k]);
      if (rc != SGPE_OK) return rc;
      if (b->queue && b->q_direct) continue;
    }
    const cudaError_t e = cudaGraphLaunch(b->graph[k], s);
    if (e != cudaSuccess) return cuda_fail(e, "batch graph launch");
    done += k ? kGraphSteps : 1;
  }
  return SGPE_OK;
}

int sgpe_batch_set_queue(sgpe_batch* b, int on) {
  if (b == nullptr) return fail(SGPE_ERR_ARG, "null batch");
  DeviceGuard g(b->device);
  if (on) {
    for (const sgpe_plan* p : b->plans)
      if (const char* why = queue_unsupported(p)) return fail(SGPE_ERR_ARG, why);
    if (b->q_grid == 0) b->q_grid = sgpe::queue_resident_blocks();
    if (b->q_grid <= 0) return fail(SGPE_ERR_CUDA, "work queue: no resident blocks on this device");
    if (b->q_words == nullptr) {
      const size_t words = 3 + b->plans.size() * 6 * kGraphSteps;
      cudaError_t e = cudaMalloc(&b->q_words, sizeof(unsigned) * words);
      if (e == cudaSuccess) e = cudaMemset(b->q_words, 0, sizeof(unsigned) * words);
      if (e != cudaSuccess) return cuda_fail(e, "work queue counters");
    }
  }
  if (bool(on) != b->queue) {
    for (auto& x : b->graph)
      if (x != nullptr) {
        cudaGraphExecDestroy(x);
        x = nullptr;
      }
    b->queue = bool(on);
    b->q_direct = false;
  }
  return SGPE_OK;
}

int sgpe_batch_device_status(sgpe_batch* b, int* status) {
  if (b == nullptr || status == nullptr) return fail(SGPE_ERR_ARG, "null batch or status");
  *status = 0;
  if (b->q_words == nullptr) return SGPE_OK;
  DeviceGuard g(b->device);
  int w = 0;
  const cudaError_t e = cudaMemcpy(&w, b->q_words, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "batch status read");
  *status = w;
  if (w != 0) return fail(SGPE_ERR_CUDA, "a work-queue wait gave up (the batch's states are not reliable)");
  return SGPE_OK;
}

int sgpe_check_queue_wait(int* gave_up, double* waited_ms) {
  if (gave_up == nullptr || waited_ms == nullptr) return fail(SGPE_ERR_ARG, "null output");
  const cudaError_t e = sgpe::check_queue_wait(gave_up, waited_ms);
  return e == cudaSuccess ? SGPE_OK : cuda_fail(e, "queue wait check");
}

int sgpe_fft2(sgpe_plan* p, const void* i0, const void* i1, void* o0, void* o1, int inverse, double scale,
              void* stream) {
  if (p == nullptr || !i0 || !i1 || !o0 || !o1) return fail(SGPE_ERR_ARG, "null plan or data pointer");
  DeviceGuard g(p->device);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  return by_iface(p->bits, [&](auto t) { return fft2<decltype(t)>(p, i0, i1, o0, o1, inverse, scale, s); });
}

}  // extern "C"
