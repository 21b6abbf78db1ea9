/*
 * spinor_gb300.h -- C ABI of the GB300 split-step solver for the
 * pseudospin-1/2 Gross-Pitaevskii equation.
 *
 * The library replaces the torch propagation path of spinor-gpe
 * (spinor_gpe/pspinor/tensor_propagator.py, spinor_gpe/pspinor/tensor_tools.py).
 * It exposes plain C: opaque plan handles, plain pointers and sizes, an int
 * status on every call (0 = success) and a thread-local message from
 * sgpe_last_error().  No exception crosses this boundary.
 *
 * Conventions
 *  - A spinor is two components, each an (ny, nx) row-major array with x
 *    contiguous (spinor_gpe/pspinor/pspinor.py:194, 350-351).
 *  - psik arguments are in the centred (fftshift) k order of the original
 *    (spinor_gpe/pspinor/tensor_tools.py:218-226).
 *  - Element type is interleaved complex: float pairs for dtype_bits = 64
 *    (complex64), double pairs for dtype_bits = 128 (complex128).
 *  - Device pointers live on the plan's device; "stream" is a cudaStream_t
 *    passed as void* (NULL = legacy default stream).  All work is enqueued
 *    asynchronously on that stream; nothing synchronises the host except the
 *    set-up calls marked "synchronous".
 *  - A plan is used by one host thread at a time.
 */
#ifndef SPINOR_GB300_H
#define SPINOR_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define SGPE_OK 0
#define SGPE_ERR_ARG 1     /* invalid argument or unsupported size */
#define SGPE_ERR_STATE 2   /* call not valid in the plan's current state */
#define SGPE_ERR_CUDA 3    /* CUDA runtime error (message has the detail) */
#define SGPE_ERR_OOM 4     /* device allocation failed */

typedef struct sgpe_plan sgpe_plan;

/* A complex operator field in FP64 on the host, interleaved (re, im).
 * value(x, y) = data[x*sx + y*sy]; sx = sy = 0 is a uniform value, (1, 0) a
 * table along x, (0, 1) a table along y, (1, nx) a full (ny, nx) field.
 * n is the number of complex elements in data.  The library rounds the
 * values once to the plan's precision. */
typedef struct sgpe_field {
  const double* data;
  int n;
  int sx;
  int sy;
} sgpe_field;

/* Operators of one Strang sub-step (outer = 0, inner = 1).
 * Replaces the pre-computed operator dicts eng_out / eng_in of the original
 * (spinor_gpe/pspinor/tensor_propagator.py:138-149; operators built by
 * tensor_tools.evolution_op :546-560 and coupling_op :563-591).
 *  kin_a[c] * kin_b[c] = exp(-i K_c t/2) in NATURAL (unshifted) k order,
 *  pot_a[c] * pot_b[c] = exp(-i V_c t) in real space,
 *  cpl_c = cos(Omega t/4), cpl_s = -i sin(Omega t/4), cpl_e = exp(i theta),
 *  interaction operator exp(z E_c) with z = int_z_re + i int_z_im = -i t/2.
 * t is the (complex, in imaginary time) sub-step duration. */
typedef struct sgpe_substep_ops {
  sgpe_field kin_a[2];
  sgpe_field kin_b[2];
  sgpe_field pot_a[2];
  sgpe_field pot_b[2];
  sgpe_field cpl_c;
  sgpe_field cpl_s;
  sgpe_field cpl_e;
  double int_z_re;
  double int_z_im;
} sgpe_substep_ops;

/* Library version (major*10000 + minor*100 + patch). */
int sgpe_version(void);

/* Message of the last failing call on this thread ("" if none). */
const char* sgpe_last_error(void);

/* dtype_bits of the double-float precision: the state, the operator tables
 * and every transform in pairs of FP32 values (head + tail, about 48
 * significant bits, 16 bytes per complex value), on the FP32 pipes; psik is
 * loaded and stored as complex128 and the energy, analysis and sgpe_fft2 of
 * such a plan take complex128 buffers.  Kernel shape 0 only; not grouped in
 * batches; no tensor-core DFT. */
#define SGPE_DTYPE_DF 48

/* Create a plan for an (ny, nx) grid.  Sizes on each axis: powers of two
 * 32..4096, or 192, 384, 768 (3 * 2^k, with a radix-3 stage).  dtype_bits:
 * 64 (complex64), 128 (complex128) or SGPE_DTYPE_DF (double-float).
 * Allocates the device state on `device`.  Synchronous.
 * Replaces: TensorPropagator.__init__ tensor uploads
 * (spinor_gpe/pspinor/tensor_propagator.py:111-122). */
int sgpe_plan_create(sgpe_plan** plan, int ny, int nx, int dtype_bits, int device);

/* Release a plan and its device memory.  Synchronous. */
int sgpe_plan_destroy(sgpe_plan* plan);

/* Interaction strengths, atom number, volume elements and the coupling
 * switch (spinor_gpe/pspinor/tensor_propagator.py:110-113, 119-121). */
int sgpe_set_physics(sgpe_plan* plan, double g_uu, double g_dd, double g_ud,
                     double atom_num, double dv_r, double dv_k, int is_coupling);

/* Upload the operators of sub-step `sub` (0 = outer, 1 = inner).
 * Synchronous.  Replaces: tensor_propagator.py:138-149. */
int sgpe_set_substep(sgpe_plan* plan, int sub, const sgpe_substep_ops* ops);

/* Load a spinor (device pointers, centred k order) as the plan state.
 * Replaces: assignment of TensorPropagator.psik (tensor_propagator.py:118). */
int sgpe_load_psik(sgpe_plan* plan, const void* psik0, const void* psik1, void* stream);

/* Write the current state as psik (device pointers, centred k order),
 * renormalised to the atom number in k-space as the original leaves it after
 * every sub-step (tensor_propagator.py:271).  If pops_dev is non-NULL, the two
 * component populations (tensor_tools.calc_pops, :466-484) of that state are
 * written there as doubles.  The plan state is not changed. */
int sgpe_store_psik(sgpe_plan* plan, void* psik0, void* psik1, double* pops_dev, void* stream);

/* One Strang sub-step with the operators of `sub`.
 * Replaces: TensorPropagator.single_step (tensor_propagator.py:224-271). */
int sgpe_single_step(sgpe_plan* plan, int sub, void* stream);

/* n_steps full steps (outer, inner, outer sub-steps each).  If pops_dev is
 * non-NULL it receives the populations after step i as pops_dev[2*i + c].
 * Those of steps 0 .. n_steps-2 are written during the call; those of the
 * last step are written by the next call that evaluates the state (the next
 * sgpe_store_psik with pops_dev = NULL, or the first sub-step of the next
 * sgpe_single_step / sgpe_full_steps), so pops_dev must stay valid until
 * then.  sgpe_load_psik discards that pending write.
 * Without populations, steady-state steps are replayed from CUDA graphs the
 * plan captures on first use (one graph launch per 8 steps); changing the
 * physics or operators discards them.
 * Replaces: TensorPropagator.full_step (tensor_propagator.py:214-222) and the
 * step loop of prop_loop (:185-194). */
int sgpe_full_steps(sgpe_plan* plan, int n_steps, double* pops_dev, void* stream);

/* Normalised, centred 2-D transforms of a two-component field (device
 * pointers, out-of-place; in and out must not overlap).
 *   inverse = 0: out_c = scale * fftshift(fft2(in_c))       (fft_2d, tensor_tools.py:201-228)
 *   inverse = 1: out_c = scale * ifft2_unnormalised(ifftshift(in_c))
 *                (ifft_2d, tensor_tools.py:231-258, with scale = 1/(nx ny norm))
 * Does not touch the propagation state. */
int sgpe_fft2(sgpe_plan* plan, const void* in0, const void* in1, void* out0, void* out1,
              int inverse, double scale, void* stream);

/* Energy fields (FP64, real parts used; each energy is the sum of two
 * broadcast fields a + b, so separable energies stay 1-D tables):
 *  kin_a[c] + kin_b[c] = K_c(kx, ky) in centred k order (the order of psik),
 *  pot_a[c] + pot_b[c] = V_c(x, y),
 *  cpl = h(x, y), the coupling energy density being 2 Re(conj(psi_0) h psi_1);
 *  h = (Omega/2) exp(-i theta) is the upper off-diagonal of the coupling
 *  Hamiltonian the propagator applies. */
typedef struct sgpe_energy_fields {
  sgpe_field kin_a[2];
  sgpe_field kin_b[2];
  sgpe_field pot_a[2];
  sgpe_field pot_b[2];
  sgpe_field cpl;
} sgpe_energy_fields;

/* Store energy fields in slot 0 or 1 of the plan (e.g. the physical energy
 * and the original package's reporting convention).  Synchronous. */
int sgpe_set_energy_fields(sgpe_plan* plan, int slot, const sgpe_energy_fields* fields);

/* FP64 energy of the spinor psik (device pointers, centred k order) with the
 * fields of `slot`; writes 10 doubles to out_dev (device):
 *   [E_kin, E_pot, E_int, E_cpl, E_total, mu, N_k, N_r, S1, S2]
 * E_kin = sum_k K_c |psik_c|^2 dv_k (spectral), E_pot = sum V_c n_c dv_r,
 * E_int = sum (g_uu n0^2/2 + g_dd n1^2/2 + g_ud n0 n1) dv_r,
 * E_cpl = sum 2 Re(conj(psi_0) h psi_1) dv_r, mu = (E_kin + E_pot + E_cpl +
 * 2 E_int) / N_r, N_k / N_r the atom numbers in k / real space,
 * S1 = sum (g_uu n0^2 + g_dd n1^2) dv_r, S2 = sum g_ud n0 n1 dv_r, with
 * psi = ifft_2d(psik).  Replaces the host-side energy expectation value
 * (spinor_gpe/pspinor/tensor_propagator.py:273-324); the kinetic term is
 * spectral instead of finite differences of the unwrapped phase. */
int sgpe_energy(sgpe_plan* plan, int slot, const void* psik0, const void* psik1, double* out_dev, void* stream);

/* Post-analysis of a final spinor (the derived fields of the original's
 * PropResult, spinor_gpe/pspinor/prop_result.py:76-88), all device pointers
 * of the plan's grid and precision:
 *   dens_c = |psi_c|^2, densk_c = |psik_c|^2 (real, working precision),
 *   phase_c = angle(psi_c), 0 where dens_c < 1e-6 max dens_c
 *             (tensor_tools.py:514-539 without unwrapping),
 *   sums_dev[5] = [sum n0 n1, sum n0^2, sum n1^2, max n0, max n1] (FP64),
 * from which calc_separation = 1 - s0 / sqrt(s1 s2). */
int sgpe_analysis(sgpe_plan* plan, const void* psi0, const void* psi1, const void* psik0, const void* psik1,
                  void* dens0, void* dens1, void* densk0, void* densk1, void* phase0, void* phase1,
                  double* sums_dev, void* stream);

/* Initial-state set-up on the device for a separable trap V = vx(x) + vy(y)
 * (the O(Nx Ny) parts of the original's PSpinor set-up,
 * spinor_gpe/pspinor/pspinor.py:248-281): writes the Thomas-Fermi spinor
 *   psi_c = sqrt(max(mu - V, 0)) * amp_c * exp(i phi_c)
 * (amp: 2 complex values as (re, im) pairs; phi_c ~ U(-noise, noise) from a
 * counter-based hash of (seed, component, point); noise = 0: none) to
 * psi0/psi1 (complex64 or complex128, (ny, nx) row-major), then, if
 * atom_num > 0, renormalises to atom_num with volume element dv_r.
 * vx (nx), vy (ny) are FP64 device arrays; scratch holds 304 doubles. */
int sgpe_setup_spinor(int dtype_bits, int ny, int nx, const double* vx, const double* vy, double mu,
                      const double* amp, double noise, unsigned long long seed, double atom_num, double dv_r,
                      double* scratch, void* psi0, void* psi1, void* stream);

/* psi_c *= prod_j f(r_j / heal_c) exp(i w_j atan2(y - y_j, x - x_j)),
 * f(g) = g / sqrt(g^2 + 1), for the vortices vort[j] = (component, x_j, y_j,
 * w_j) (FP64 device array of n_vort x 4); x (nx), y (ny) the grid coordinates
 * (device), heal[2] host values.  Replaces seed_vortices
 * (spinor_gpe/pspinor/pspinor.py:680-745). */
int sgpe_imprint_vortices(int dtype_bits, int ny, int nx, const double* x, const double* y, const double* vort,
                          int n_vort, const double* heal, void* psi0, void* psi1, void* stream);

/* out = f_plus S(+shift) in + f_minus S(-shift) in for one (ny, nx)
 * component, S(s) the multiplication by exp(-2 pi i s fftfreq(nx)[ix]) along
 * x: the momentum split of shift_momentum (spinor_gpe/pspinor/pspinor.py:
 * 503-545, scipy.ndimage.fourier_shift of the centred transform). */
int sgpe_fourier_split_x(int dtype_bits, int ny, int nx, double shift, double f_plus, double f_minus,
                         const void* in, void* out, void* stream);

/* Measurement helper: n_steps full steps exactly as sgpe_full_steps (no
 * populations), captured into a CUDA graph with events around every column
 * pass and every row pass, launched once on `stream`.  Synchronises the
 * stream and returns the mean device duration of one column pass and of one
 * row pass in milliseconds.  Advances the state by n_steps steps (plus at
 * most one step to reach the graph's steady state).
 * Instrumentation of the native path; no counterpart in the original. */
int sgpe_time_passes(sgpe_plan* plan, int n_steps, double* col_ms, double* row_ms, void* stream);

/* A batch of plans stepped together (many independent solves, uneven grid
 * sizes and parameters).  The plans stay owned by the caller and must
 * outlive the batch and be on one device.  While the batch exists the plans
 * may still be stepped, read and loaded on their own; when a plan's physics
 * or operators are replaced, the batch re-captures its graphs at its next
 * step.  No counterpart in the original (which runs one solve per process). */
typedef struct sgpe_batch sgpe_batch;
int sgpe_batch_create(sgpe_batch** batch, sgpe_plan* const* plans, int n_plans);
int sgpe_batch_destroy(sgpe_batch* batch);

/* Advance every plan of the batch by n_steps full steps (no populations).
 * The solves' steady-state steps are captured once as independent branches
 * of a CUDA graph (one graph per 8 steps and one per step) and replayed on
 * `stream`, so their kernels run concurrently on the GPU.  Plans that are not
 * in the steady state first take one eager step.  Results are identical to
 * stepping each plan alone with sgpe_full_steps. */
int sgpe_batch_steps(sgpe_batch* batch, int n_steps, void* stream);

/* Work-queue mode of a batch (on = 1): its steps run as one persistent
 * (cooperative) launch per graph, fed from a device work queue: every pass
 * of every sub-step of every solve is split into items (column tiles, row
 * groups), blocks claim the items in one global order, and an item waits
 * (bounded, 1 s) until the previous pass of its solve has finished.  The
 * launch is captured in the batch's CUDA graphs (launched directly when
 * the driver refuses the capture).  Complex64 plans with separable
 * operators and sides 128, 192, 256, 384, 512, 768 or 1024 only
 * (SGPE_ERR_ARG otherwise).  The items use their own tile shapes, so
 * results agree with sgpe_full_steps per plan to complex64 rounding (not
 * bit for bit).  on = 0 returns to grouped launches.  No counterpart in
 * the original (one solve per process). */
int sgpe_batch_set_queue(sgpe_batch* batch, int on);

/* Error word of the batch's work queue: 0, or the code of a wait that gave
 * up (the batch's states are then not reliable; SGPE_ERR_CUDA).
 * Synchronous (a 4-byte device read). */
int sgpe_batch_device_status(sgpe_batch* batch, int* status);

/* Check of the work queue's bounded wait on the current device: one block
 * waits for a counter that nothing increments; gave_up = 1 when the wait
 * ended by its limit (about 1 s, returned in waited_ms). */
int sgpe_check_queue_wait(int* gave_up, double* waited_ms);

/* Arithmetic of the radix-16 DFT stages of the plan's transforms:
 * mode 0 (default) FP32 butterflies on the CUDA cores; mode 1 split-BF16
 * products on the tensor cores (each FP32 operand split into BF16 head and
 * tail, products hi.hi + hi.lo + lo.hi accumulated in FP32), a precision-
 * study variant for complex64 plans with sides 64, 256, 1024 or 2048.
 * Twiddles, point-wise operators and reductions are unchanged.  The state
 * is kept; must not be called while populations of a step are pending.
 * No counterpart in the original. */
int sgpe_set_dft_mode(sgpe_plan* plan, int mode);

/* Kernel shapes.  Each pass (axis 0: the row pass along x, axis 1: the
 * column pass along y) can run in one of several launch configurations for
 * the same side: shape 0 and, depending on the side and precision, shapes
 * with fewer points per thread or fewer lines per block (power-of-two sides
 * up to 512: more warps and blocks for small grids), with 32 points per
 * thread (complex64 rows of 1024), or with the other radix-3 plan (sides
 * 3 * 2^k).  All shapes compute the same steps; rounding differs with the
 * radix plan (every shape meets the parity tolerances).  A new plan takes
 * built-in defaults measured on GB300.
 * No counterpart in the original (whose transforms are cuFFT's).
 *
 * sgpe_shape_count: number of shapes for (dtype_bits, axis, side n), 0 if n
 * is unsupported.  sgpe_set_shapes: switch the plan's shapes (new twiddle
 * tables, graphs re-captured; the state is kept; the tensor-core DFT mode
 * runs shape 0 only).  sgpe_get_shapes: the current shapes. */
/* Device error word of the plan's pass kernels: 0, or 1 when a kernel gave
 * up a bounded wait for its bulk (TMA) copies and continued with plain loads
 * (the state of that pass is not reliable).  Synchronous (a 4-byte device
 * read); returns SGPE_ERR_CUDA with a message when the word is non-zero. */
int sgpe_device_status(sgpe_plan* plan, int* status);

/* Check of the bounded wait itself, on the current device: one block waits
 * on an mbarrier phase that no copy completes; gave_up = 1 when every
 * thread ended its wait by the limit (about 0.5 s, returned in waited_ms)
 * instead of hanging.  No counterpart in the original. */
int sgpe_check_bounded_wait(int* gave_up, double* waited_ms);

#define SGPE_MAX_SHAPES 3
int sgpe_shape_count(int dtype_bits, int axis, int n);
int sgpe_set_shapes(sgpe_plan* plan, int row_shape, int col_shape);
int sgpe_get_shapes(const sgpe_plan* plan, int* row_shape, int* col_shape);

/* Autotuner: times n_steps steady-state full steps in every pair of
 * shapes (twice, the faster kept), each pair starting from the plan's
 * current state, and leaves the plan in the fastest pair with that state
 * restored (the plan's own shapes stay unless another pair is more than 2%
 * faster).  step_us (optional, SGPE_MAX_SHAPES^2 entries, index
 * row_shape * SGPE_MAX_SHAPES + col_shape) receives the microseconds per
 * step, -1 for pairs not run.  Synchronises `stream`.  The plan must be
 * ready to step, with no populations pending. */
int sgpe_autotune(sgpe_plan* plan, int n_steps, int* row_shape, int* col_shape, double* step_us, void* stream);

/* Size in bytes of the device scratch array used by sgpe_fft2_static
 * (2.25 MiB, present on every GPU that loads the library). */
#define SGPE_FFT2_STATIC_BYTES (2359296)

/* Allocation-free variant of sgpe_fft2, without a plan.  No counterpart in
 * the original package.
 * For callers that must not allocate device memory where they need the
 * transform: hosts whose device memory belongs to their own pool allocator
 * (which has taken the device's free memory and must not be bypassed),
 * real-time loops that cannot take an allocation's latency or implicit
 * synchronisation, foreign-language hosts holding only raw device pointers.  It calls no cudaMalloc/cudaFree
 * and no allocating library routine; the caller passes inputs and outputs.
 * Scratch: a file-scope device array of SGPE_FFT2_STATIC_BYTES, enough for
 * grids of up to 65,536 points in complex128 and 131,072 in complex64
 * (e.g. 256x256 and 256x512); larger grids return SGPE_ERR_ARG with a
 * message -- use sgpe_fft2 with a plan for those.
 * Runs on the current CUDA device, in the runtime API's primary context.
 * The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress) and should be made before any stream capture on
 * that device is started.  Under CUDA's default lazy module loading the first
 * launch of a kernel loads its module, which allocates device memory, and
 * each (grid size, precision, direction) uses its own kernels: make one
 * warm-up call per combination before the code that cannot allocate, or set
 * CUDA_MODULE_LOADING=EAGER.  All calls share the array: calls that overlap
 * on the GPU (other streams or threads) race -- order them on one stream.
 * Arguments and results as sgpe_fft2. */
int sgpe_fft2_static(int ny, int nx, int dtype_bits, const void* in0, const void* in1, void* out0, void* out1,
                     int inverse, double scale, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* SPINOR_GB300_H */
