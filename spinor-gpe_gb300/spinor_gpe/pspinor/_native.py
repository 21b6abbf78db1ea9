"""ctypes binding of ``libspinor_gb300.so`` (declared in
``include/spinor_gb300.h``).

The library is the only compute path of this package: if it is missing or
cannot be loaded, importing the propagator raises instead of falling back to
any other implementation.
"""
import ctypes
import os

import numpy as np

# SGPE_LIB_PATH selects another build of the same library (tuning builds).
LIB_PATH = os.environ.get('SGPE_LIB_PATH') or os.path.join(
    os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
    'libspinor_gb300.so')

SGPE_OK = 0
SGPE_ERR_ARG = 1
SGPE_ERR_STATE = 2
SGPE_ERR_CUDA = 3
SGPE_ERR_OOM = 4

EXPORTED = ('sgpe_version', 'sgpe_last_error', 'sgpe_plan_create',
            'sgpe_plan_destroy', 'sgpe_set_physics', 'sgpe_set_substep',
            'sgpe_load_psik', 'sgpe_store_psik', 'sgpe_single_step',
            'sgpe_full_steps', 'sgpe_fft2', 'sgpe_time_passes',
            'sgpe_fft2_static', 'sgpe_set_energy_fields', 'sgpe_energy',
            'sgpe_batch_create', 'sgpe_batch_destroy', 'sgpe_batch_steps',
            'sgpe_set_dft_mode', 'sgpe_analysis', 'sgpe_setup_spinor',
            'sgpe_imprint_vortices', 'sgpe_fourier_split_x',
            'sgpe_shape_count', 'sgpe_set_shapes', 'sgpe_get_shapes',
            'sgpe_autotune', 'sgpe_device_status', 'sgpe_check_bounded_wait',
            'sgpe_batch_set_queue', 'sgpe_batch_device_status', 'sgpe_check_queue_wait')

SGPE_MAX_SHAPES = 3
# dtype_bits of the double-float precision (include/spinor_gb300.h)
SGPE_DTYPE_DF = 48


class SgpeError(RuntimeError):
    """A non-zero status from the native library."""

    def __init__(self, code, msg):
        super().__init__(f'sgpe error {code}: {msg}')
        self.code = code


class Field(ctypes.Structure):
    """``sgpe_field``: host FP64 complex data with broadcast strides."""
    _fields_ = [('data', ctypes.POINTER(ctypes.c_double)),
                ('n', ctypes.c_int), ('sx', ctypes.c_int),
                ('sy', ctypes.c_int)]


class SubstepOps(ctypes.Structure):
    """``sgpe_substep_ops``."""
    _fields_ = [('kin_a', Field * 2), ('kin_b', Field * 2),
                ('pot_a', Field * 2), ('pot_b', Field * 2),
                ('cpl_c', Field), ('cpl_s', Field), ('cpl_e', Field),
                ('int_z_re', ctypes.c_double), ('int_z_im', ctypes.c_double)]


class EnergyFields(ctypes.Structure):
    """``sgpe_energy_fields``."""
    _fields_ = [('kin_a', Field * 2), ('kin_b', Field * 2),
                ('pot_a', Field * 2), ('pot_b', Field * 2), ('cpl', Field)]


_VP = ctypes.c_void_p
_SIGS = {
    'sgpe_version': ([], ctypes.c_int),
    'sgpe_last_error': ([], ctypes.c_char_p),
    'sgpe_plan_create': ([ctypes.POINTER(_VP), ctypes.c_int, ctypes.c_int,
                          ctypes.c_int, ctypes.c_int], ctypes.c_int),
    'sgpe_plan_destroy': ([_VP], ctypes.c_int),
    'sgpe_set_physics': ([_VP] + [ctypes.c_double] * 6 + [ctypes.c_int],
                         ctypes.c_int),
    'sgpe_set_substep': ([_VP, ctypes.c_int, ctypes.POINTER(SubstepOps)],
                         ctypes.c_int),
    'sgpe_load_psik': ([_VP, _VP, _VP, _VP], ctypes.c_int),
    'sgpe_store_psik': ([_VP, _VP, _VP, _VP, _VP], ctypes.c_int),
    'sgpe_single_step': ([_VP, ctypes.c_int, _VP], ctypes.c_int),
    'sgpe_full_steps': ([_VP, ctypes.c_int, _VP, _VP], ctypes.c_int),
    'sgpe_fft2': ([_VP, _VP, _VP, _VP, _VP, ctypes.c_int, ctypes.c_double,
                   _VP], ctypes.c_int),
    'sgpe_time_passes': ([_VP, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                          ctypes.POINTER(ctypes.c_double), _VP], ctypes.c_int),
    'sgpe_set_energy_fields': ([_VP, ctypes.c_int, ctypes.POINTER(EnergyFields)],
                               ctypes.c_int),
    'sgpe_energy': ([_VP, ctypes.c_int, _VP, _VP, _VP, _VP], ctypes.c_int),
    'sgpe_batch_create': ([ctypes.POINTER(_VP), ctypes.POINTER(_VP), ctypes.c_int],
                          ctypes.c_int),
    'sgpe_batch_destroy': ([_VP], ctypes.c_int),
    'sgpe_batch_steps': ([_VP, ctypes.c_int, _VP], ctypes.c_int),
    'sgpe_batch_set_queue': ([_VP, ctypes.c_int], ctypes.c_int),
    'sgpe_batch_device_status': ([_VP, ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
    'sgpe_check_queue_wait': ([ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)],
                              ctypes.c_int),
    'sgpe_set_dft_mode': ([_VP, ctypes.c_int], ctypes.c_int),
    'sgpe_shape_count': ([ctypes.c_int, ctypes.c_int, ctypes.c_int], ctypes.c_int),
    'sgpe_device_status': ([_VP, ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
    'sgpe_check_bounded_wait': ([ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)],
                                ctypes.c_int),
    'sgpe_set_shapes': ([_VP, ctypes.c_int, ctypes.c_int], ctypes.c_int),
    'sgpe_get_shapes': ([_VP, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)],
                        ctypes.c_int),
    'sgpe_autotune': ([_VP, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                       ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double), _VP],
                      ctypes.c_int),
    'sgpe_analysis': ([_VP] + [_VP] * 10 + [_VP, _VP], ctypes.c_int),
    'sgpe_setup_spinor': ([ctypes.c_int, ctypes.c_int, ctypes.c_int, _VP, _VP,
                           ctypes.c_double, _VP, ctypes.c_double, ctypes.c_ulonglong,
                           ctypes.c_double, ctypes.c_double, _VP, _VP, _VP, _VP],
                          ctypes.c_int),
    'sgpe_imprint_vortices': ([ctypes.c_int, ctypes.c_int, ctypes.c_int, _VP, _VP,
                               _VP, ctypes.c_int, _VP, _VP, _VP, _VP], ctypes.c_int),
    'sgpe_fourier_split_x': ([ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                              ctypes.c_double, ctypes.c_double, _VP, _VP, _VP],
                             ctypes.c_int),
    'sgpe_fft2_static': ([ctypes.c_int, ctypes.c_int, ctypes.c_int, _VP, _VP,
                          _VP, _VP, ctypes.c_int, ctypes.c_double, _VP],
                         ctypes.c_int),
}

_LIB = None


def load():
    """Load the library once (raises if it is absent)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f'{LIB_PATH} is missing: build it with '
                '`python spinor-gpe_gb300/build_native.py` (needs nvcc); '
                'this solver has no fallback implementation.')
        lib = ctypes.CDLL(LIB_PATH)
        for name, (args, res) in _SIGS.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = res
        _LIB = lib
    return _LIB


def check(code):
    if code != SGPE_OK:
        msg = load().sgpe_last_error().decode(errors='replace')
        raise SgpeError(code, msg)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


c_ptr = _ptr
c_void_p = ctypes.c_void_p


def _stream(torch, device):
    """Handle of ``device``'s current CUDA stream, as the C ABI's ``stream``
    arguments take it.  Read through torch's raw-handle accessor when it has
    one (a few hundred nanoseconds, against several microseconds for a
    ``torch.cuda.Stream`` object); a Python loop with one ``full_step()``
    per step at small grids pays this on every call."""
    raw = getattr(torch._C, '_cuda_getCurrentRawStream', None)
    if raw is None or not torch.cuda.is_initialized():
        return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)
    if isinstance(device, int):
        idx = device
    else:
        idx = torch.device(device).index
    if idx is None:
        idx = torch.cuda.current_device()
    return raw(idx)


def make_field(arr):
    """``Field`` from a numpy ``FieldSpec`` (see ``operators.py``); the
    returned tuple keeps the backing array alive."""
    data = np.ascontiguousarray(arr.values, dtype=np.complex128)
    f = Field(data.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
              int(data.size), int(arr.sx), int(arr.sy))
    return f, data


class Plan:
    """Owner of one native plan (``sgpe_plan``) on a CUDA device."""

    def __init__(self, ny, nx, dtype_bits, device_index):
        lib = load()
        h = _VP()
        check(lib.sgpe_plan_create(ctypes.byref(h), int(ny), int(nx),
                                   int(dtype_bits), int(device_index)))
        self._h = h
        self.ny, self.nx, self.bits = ny, nx, dtype_bits
        self.device_index = device_index

    def close(self):
        if getattr(self, '_h', None) is not None and self._h.value:
            load().sgpe_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:   # interpreter shutdown
            pass

    def set_dft_mode(self, mode):
        """0: FP32 radix-16 DFTs; 1: split-BF16 tensor-core DFT16."""
        check(load().sgpe_set_dft_mode(self._h, int(mode)))

    def check_device_status(self):
        """Raise if a pass kernel recorded a failed bounded wait."""
        st = ctypes.c_int()
        check(load().sgpe_device_status(self._h, ctypes.byref(st)))

    def set_shapes(self, row_shape, col_shape):
        """Kernel shapes of the row and column passes (keeps the state)."""
        check(load().sgpe_set_shapes(self._h, int(row_shape), int(col_shape)))

    @property
    def shapes(self):
        """Current (row shape, column shape)."""
        r, c = ctypes.c_int(), ctypes.c_int()
        check(load().sgpe_get_shapes(self._h, ctypes.byref(r), ctypes.byref(c)))
        return r.value, c.value

    def autotune(self, torch, n_steps, device):
        """Time every pair of kernel shapes over n_steps steps from the
        current state and keep the fastest; returns ((row, col), {(row,
        col): microseconds per step}).  The state is unchanged."""
        r, c = ctypes.c_int(), ctypes.c_int()
        us = (ctypes.c_double * (SGPE_MAX_SHAPES * SGPE_MAX_SHAPES))()
        check(load().sgpe_autotune(self._h, int(n_steps), ctypes.byref(r),
                                   ctypes.byref(c), us, _stream(torch, device)))
        times = {(i // SGPE_MAX_SHAPES, i % SGPE_MAX_SHAPES): us[i]
                 for i in range(SGPE_MAX_SHAPES * SGPE_MAX_SHAPES) if us[i] > 0}
        return (r.value, c.value), times

    def set_physics(self, g_uu, g_dd, g_ud, atom_num, dv_r, dv_k,
                    is_coupling):
        check(load().sgpe_set_physics(self._h, g_uu, g_dd, g_ud, atom_num,
                                      dv_r, dv_k, int(bool(is_coupling))))

    def set_substep(self, sub, spec):
        """Upload a ``SubstepSpec`` (``operators.py``) as sub-step ``sub``."""
        ops = SubstepOps()
        keep = []

        def put(fs):
            f, d = make_field(fs)
            keep.append(d)
            return f
        for c in range(2):
            ops.kin_a[c] = put(spec.kin_a[c])
            ops.kin_b[c] = put(spec.kin_b[c])
            ops.pot_a[c] = put(spec.pot_a[c])
            ops.pot_b[c] = put(spec.pot_b[c])
        ops.cpl_c = put(spec.cpl_c)
        ops.cpl_s = put(spec.cpl_s)
        ops.cpl_e = put(spec.cpl_e)
        ops.int_z_re = float(spec.int_z.real)
        ops.int_z_im = float(spec.int_z.imag)
        check(load().sgpe_set_substep(self._h, int(sub), ctypes.byref(ops)))

    def load_psik(self, torch, psik):
        check(load().sgpe_load_psik(self._h, _ptr(psik[0]), _ptr(psik[1]),
                                    _stream(torch, psik[0].device)))

    def store_psik(self, torch, out, pops=None):
        check(load().sgpe_store_psik(
            self._h, _ptr(out[0]), _ptr(out[1]),
            _ptr(pops) if pops is not None else None,
            _stream(torch, out[0].device)))

    def single_step(self, torch, sub, device):
        check(load().sgpe_single_step(self._h, int(sub),
                                      _stream(torch, device)))

    def full_steps(self, torch, n_steps, device, pops=None):
        check(load().sgpe_full_steps(
            self._h, int(n_steps), _ptr(pops) if pops is not None else None,
            _stream(torch, device)))

    def time_passes(self, torch, n_steps, device):
        """Mean (column pass, row pass) durations in ms over n_steps full
        steps, from CUDA events on the current stream."""
        col = ctypes.c_double()
        row = ctypes.c_double()
        check(load().sgpe_time_passes(self._h, int(n_steps), ctypes.byref(col),
                                      ctypes.byref(row),
                                      _stream(torch, device)))
        return col.value, row.value

    def set_energy_fields(self, slot, kin, pot, cpl):
        """Upload FP64 energy fields: ``kin`` and ``pot`` are two (a, b)
        FieldSpec pairs per component (the energy is a + b), ``cpl`` the
        coupling field h."""
        ef = EnergyFields()
        keep = []

        def put(fs):
            f, d = make_field(fs)
            keep.append(d)
            return f
        for c in range(2):
            ef.kin_a[c] = put(kin[c][0])
            ef.kin_b[c] = put(kin[c][1])
            ef.pot_a[c] = put(pot[c][0])
            ef.pot_b[c] = put(pot[c][1])
        ef.cpl = put(cpl)
        check(load().sgpe_set_energy_fields(self._h, int(slot), ctypes.byref(ef)))

    def energy(self, torch, slot, psik, out):
        """FP64 energy of psik (device tensors) into ``out`` (10 doubles,
        device)."""
        check(load().sgpe_energy(self._h, int(slot), _ptr(psik[0]), _ptr(psik[1]),
                                 _ptr(out), _stream(torch, psik[0].device)))

    def analysis(self, torch, psi, psik, dens, densk, phase, sums):
        """Densities, masked phases and FP64 separation sums (device)."""
        check(load().sgpe_analysis(
            self._h, _ptr(psi[0]), _ptr(psi[1]), _ptr(psik[0]), _ptr(psik[1]),
            _ptr(dens[0]), _ptr(dens[1]), _ptr(densk[0]), _ptr(densk[1]),
            _ptr(phase[0]), _ptr(phase[1]), _ptr(sums),
            _stream(torch, psi[0].device)))

    def fft2(self, torch, inp, out, inverse, scale):
        check(load().sgpe_fft2(self._h, _ptr(inp[0]), _ptr(inp[1]),
                               _ptr(out[0]), _ptr(out[1]), int(inverse),
                               float(scale), _stream(torch, inp[0].device)))


class Batch:
    """Owner of a native batch of plans (``sgpe_batch``)."""

    def __init__(self, plans):
        lib = load()
        self._plans = list(plans)          # keep the plans alive
        arr = (_VP * len(self._plans))(*[p._h for p in self._plans])
        h = _VP()
        check(lib.sgpe_batch_create(ctypes.byref(h), arr, len(self._plans)))
        self._h = h

    def close(self):
        if getattr(self, '_h', None) is not None and self._h.value:
            load().sgpe_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:   # interpreter shutdown
            pass

    def steps(self, torch, n_steps, device):
        check(load().sgpe_batch_steps(self._h, int(n_steps),
                                      _stream(torch, device)))

    def set_queue(self, on):
        """Work-queue mode: the steps run as one persistent launch of the
        queue kernel per graph (complex64 plans with separable operators)."""
        check(load().sgpe_batch_set_queue(self._h, int(bool(on))))

    def check_device_status(self):
        """Raise if a work-queue wait gave up (synchronous)."""
        st = ctypes.c_int()
        check(load().sgpe_batch_device_status(self._h, ctypes.byref(st)))
