"""Drop-in ``TensorPropagator``: the spinor-gpe split-step propagator backed
by the native GB300 kernels.

Same constructor, methods and readable attributes as the original
(``spinor_gpe/pspinor/tensor_propagator.py:67-324``).  The time stepping runs
entirely in ``libspinor_gb300.so``: two fused sweeps over the state per
Strang sub-step, renormalisation and populations reduced on the device, no
host synchronisation inside a step loop.  There is no CPU path: a ``device``
that is not a CUDA device raises.

Differences a caller can observe:

* ``device`` defaults to ``'cuda'``; ``dtype`` (64 or 128, default 128) selects
  complex64 or complex128 arithmetic; ``dtype='double-float'`` keeps the
  state, the operator tables and every transform in pairs of FP32 values
  (about 48 significant bits on the FP32 pipes), with ``psik`` in
  complex128.
* ``psik`` is materialised on read from the device state (functional, as in
  the original, which rebinds ``self.psik`` every sub-step); assigning it loads
  a new state.
* ``eng_out`` / ``eng_in`` are dicts whose ``'kin'``, ``'pot'`` and ``'coupl'``
  entries are built on first access; ``single_step`` accepts only these two
  dicts.
* ``eng_expect`` evaluates the original's energy convention
  (``tensor_propagator.py:273-324``) with a spectral kinetic term instead of
  finite differences of the unwrapped phase (scikit-image is not used).
"""
import numpy as np
import torch

from .. import tuning
from . import _native
from . import operators as ops
from . import prop_result
from . import tensor_tools as ttools
from .plotting_tools import next_available_path

try:  # progress bar as in the original; optional
    from tqdm import tqdm as _tqdm
except ImportError:  # pragma: no cover
    def _tqdm(it, **_):
        return it

MAGIC_GAMMA = 1 / (2 + 2**(1 / 3))     # tensor_propagator.py:101


def _bits(dtype):
    if dtype in (64, 'complex64', torch.complex64, np.complex64):
        return 64
    if dtype in (128, 'complex128', torch.complex128, np.complex128):
        return 128
    if dtype in (_native.SGPE_DTYPE_DF, 'double-float', 'df'):
        return _native.SGPE_DTYPE_DF
    raise ValueError("dtype must be complex64, complex128 or 'double-float', "
                     f"got {dtype!r}")


def cuda_device(device):
    """torch.device for a CUDA device string; raises for anything else."""
    dev = torch.device(device)
    if dev.type != 'cuda':
        raise ValueError(
            f"device {device!r}: this propagator runs only on CUDA devices "
            "(the split step is implemented by the native GB300 kernels and "
            "has no CPU fallback); pass device='cuda'.")
    if not torch.cuda.is_available():
        raise RuntimeError('CUDA is not available in this process')
    if dev.index is None:
        dev = torch.device('cuda', torch.cuda.current_device())
    return dev


def _space_value(v):
    """A grid quantity: separable meshes as they are, the rest as arrays."""
    return v if isinstance(v, ops.SepField) else np.asarray(v)


class SubstepOperators(dict):
    """``eng_out`` / ``eng_in``: the operators of one sub-step.

    ``sub`` is 0 (outer) or 1 (inner).  The dense ``'kin'``, ``'pot'`` and
    ``'coupl'`` tensors of the original (tensor_propagator.py:138-149) are
    built from the FP64 specs on first access.
    """

    def __init__(self, owner, sub, spec):
        super().__init__()
        self.owner = owner
        self.sub = sub
        self.spec = spec

    def __missing__(self, key):
        p = self.owner
        ny, nx = p._shape
        cdt = p._ctype
        dev = p._device

        def dense(fa, fb=None):
            v = fa.dense(ny, nx)
            if fb is not None:
                v = v * fb.dense(ny, nx)
            return torch.as_tensor(v, dtype=cdt, device=dev)
        s = self.spec
        if key == 'kin':   # centred k order, like the original
            val = [torch.as_tensor(np.fft.fftshift(
                s.kin_a[c].dense(ny, nx) * s.kin_b[c].dense(ny, nx)),
                dtype=cdt, device=dev) for c in range(2)]
        elif key == 'pot':
            val = [dense(s.pot_a[c], s.pot_b[c]) for c in range(2)]
        elif key == 'coupl':
            cc, cs, ce = (s.cpl_c.dense(ny, nx), s.cpl_s.dense(ny, nx),
                          s.cpl_e.dense(ny, nx))
            val = [[torch.as_tensor(cc, dtype=cdt, device=dev),
                    torch.as_tensor(cs * np.conj(ce), dtype=cdt, device=dev)],
                   [torch.as_tensor(cs * ce, dtype=cdt, device=dev),
                    torch.as_tensor(cc, dtype=cdt, device=dev)]]
        else:
            raise KeyError(key)
        self[key] = val
        return val


class TensorPropagator:
    """GPU propagator of the pseudospin-1/2 GPE (see the module docstring).

    Parameters follow ``tensor_propagator.py:67-91``: ``spin`` (a
    ``PSpinor``), ``t_step``, ``n_steps``, ``device``, ``time`` ('imag' or
    'real'), ``is_sampling``, ``n_samples``; plus ``dtype`` (64 / 128 / 'double-float') and
    ``tensor_core_dft`` (complex64 only: radix-16 DFT stages as split-BF16
    products on the tensor cores, a precision-study variant),
    ``kernel_shapes`` (row and column kernel shapes, default: the shapes
    remembered for this grid by ``spinor_gpe.tuning``, else the library's
    built-in defaults) and ``autotune`` (time every pair of shapes on the
    initial state and keep the fastest, see ``autotune()``).
    """

    # pylint: disable=too-many-instance-attributes
    def __init__(self, spin, t_step, n_steps, device='cuda', time='imag',
                 is_sampling=False, n_samples=1, dtype=128,
                 tensor_core_dft=False, kernel_shapes=None, autotune=False):
        self.n_steps = n_steps
        self._device = cuda_device(device)
        self.device = device
        self.paths = spin.paths

        if time == 'imag':
            self.t_step = -1.0j * t_step
        elif time == 'real':
            self.t_step = t_step
        else:
            raise ValueError("time must be 'imag' or 'real'")
        self.time = time
        self.dt_out = self.t_step * MAGIC_GAMMA
        self.dt_in = self.t_step * (1 - 2 * MAGIC_GAMMA)

        self.rand_seed = spin.rand_seed
        if self.rand_seed is not None:
            torch.manual_seed(self.rand_seed)
        self.is_sampling = is_sampling

        self.atom_num = spin.atom_num
        self.is_coupling = spin.is_coupling
        self.g_sc = spin.g_sc
        self._bits = _bits(dtype)
        self._ctype = torch.complex64 if self._bits == 64 else torch.complex128
        self._rtype = torch.float32 if self._bits == 64 else torch.float64

        # FP64 fields; separable fields of a device-built spinor stay as
        # their 1-D parts (ops.SepField) and are never formed in 2-D here
        self._kin_np = [ops.as_field(k) for k in spin.kin_eng_spin]
        self._pot_np = [ops.as_field(v) for v in spin.pot_eng_spin]
        self._coupling_np = ops.as_field(spin.coupling)
        psik0 = [p if isinstance(p, torch.Tensor) else np.asarray(p)
                 for p in spin.psik]
        self._shape = tuple(psik0[0].shape)
        ny, nx = self._shape
        keys_space = ['dr', 'dk', 'x_mesh', 'y_mesh', 'dv_r', 'dv_k']
        self._space_np = {k: _space_value(spin.space[k]) for k in keys_space}
        self._kx_np = _space_value(spin.space['kx_mesh']) \
            if 'kx_mesh' in spin.space else None
        self._ky_np = _space_value(spin.space['ky_mesh']) \
            if 'ky_mesh' in spin.space else None
        self._space_dev = None

        # pylint: disable=invalid-name
        self.kL_recoil = spin.kL_recoil
        self.rot_coupling = spin.rot_coupling
        if spin.rot_coupling:                     # tensor_propagator.py:125-129
            self._expon_np = None
        else:
            self._expon_np = 2 * self.kL_recoil * self._space_np['x_mesh']

        if self.is_sampling:
            assert self.n_steps % n_samples == 0, (
                f"The number of samples requested {n_samples} does not evenly "
                f"divide the total number of steps {self.n_steps}.")
        self.sample_rate = self.n_steps / n_samples

        self._plan = _native.Plan(ny, nx, self._bits, self._device.index)
        self.tensor_core_dft = bool(tensor_core_dft)
        if self.tensor_core_dft:
            self._plan.set_dft_mode(1)
        elif kernel_shapes is not None:
            self._plan.set_shapes(*kernel_shapes)
        elif tuning.lookup(self._bits, ny, nx) is not None:
            self._plan.set_shapes(*tuning.lookup(self._bits, ny, nx))
        dv_r = float(self._space_np['dv_r'])
        dv_k = float(self._space_np['dv_k'])
        self._plan.set_physics(float(self.g_sc['uu']), float(self.g_sc['dd']),
                               float(self.g_sc['ud']), float(self.atom_num),
                               dv_r, dv_k, self.is_coupling)
        self._prepared = ops.Prepared(self._kin_np, self._pot_np,
                                      self._coupling_np, self._expon_np)
        spec_out = ops.build_substep(self.dt_out, self._kin_np, self._pot_np,
                                     self._coupling_np, self._expon_np, True,
                                     self._prepared)
        spec_in = ops.build_substep(self.dt_in, self._kin_np, self._pot_np,
                                    self._coupling_np, self._expon_np, False,
                                    self._prepared)
        self._plan.set_substep(0, spec_out)
        self._plan.set_substep(1, spec_in)
        self.eng_out = SubstepOperators(self, 0, spec_out)
        self.eng_in = SubstepOperators(self, 1, spec_in)
        self._set_energy_fields()
        self._psik_cache = None
        self.psik = [torch.as_tensor(p, dtype=self._ctype, device=self._device)
                     for p in psik0]
        self.tune_times = None
        if autotune and not self.tensor_core_dft:
            self.autotune()

    # ------------------------------------------------------------ attributes
    @property
    def space(self):
        """Grid quantities as device tensors (tensor_propagator.py:118-121),
        formed on first access."""
        if self._space_dev is None:
            self._space_dev = {k: torch.tensor(np.asarray(v), device=self._device)
                               for k, v in self._space_np.items()}
        return self._space_dev

    @property
    def expon(self):
        """The Raman phase 2 kL x as a device tensor (0 in the rotated frame)."""
        if self._expon_np is None:
            return torch.tensor(0.0)
        return torch.as_tensor(np.asarray(self._expon_np), device=self._device)

    @property
    def kin_eng_spin(self):
        """Kinetic energy grids as device tensors (tensor_propagator.py:114)."""
        return [torch.as_tensor(np.asarray(k), device=self._device)
                for k in self._kin_np]

    @property
    def pot_eng_spin(self):
        """Potential energy grids as device tensors (tensor_propagator.py:116)."""
        return [torch.as_tensor(np.asarray(v), device=self._device)
                for v in self._pot_np]

    @property
    def coupling(self):
        return torch.as_tensor(np.asarray(self._coupling_np), device=self._device)

    @property
    def psik(self):
        """The current k-space spinor: two device tensors, centred k order,
        renormalised to the atom number (tensor_propagator.py:271)."""
        if self._psik_cache is None:
            ny, nx = self._shape
            out = [torch.empty((ny, nx), dtype=self._ctype,
                               device=self._device) for _ in range(2)]
            self._plan.store_psik(torch, out)
            self._psik_cache = out
        return self._psik_cache

    @psik.setter
    def psik(self, value):
        psik = [torch.as_tensor(p, device=self._device).to(self._ctype)
                .contiguous() for p in value]
        if len(psik) != 2 or psik[0].shape != self._shape:
            raise ValueError(f'psik must be two {self._shape} arrays')
        self._plan.load_psik(torch, psik)
        self._psik_cache = [p.clone() for p in psik]

    # ------------------------------------------------------------- stepping
    def full_step(self):
        """Outer, inner, outer sub-steps (tensor_propagator.py:214-222)."""
        self._plan.full_steps(torch, 1, self._device)
        self._psik_cache = None

    def single_step(self, t_step, eng):
        """One Strang sub-step (tensor_propagator.py:224-271).  ``eng`` must
        be ``self.eng_out`` or ``self.eng_in`` (with their ``t_step``)."""
        if eng is self.eng_out:
            sub, expected = 0, self.dt_out
        elif eng is self.eng_in:
            sub, expected = 1, self.dt_in
        else:
            raise ValueError('single_step accepts only the eng_out / eng_in '
                             'operators of this propagator')
        if not np.isclose(complex(t_step), complex(expected), rtol=1e-12,
                          atol=0.0):
            raise ValueError('t_step does not match the operators passed')
        self._plan.single_step(torch, sub, self._device)
        self._psik_cache = None

    def check_device(self):
        """Raise ``SgpeError`` if a pass kernel gave up a bounded wait for
        its bulk copies since the plan was created (synchronous)."""
        self._plan.check_device_status()

    @property
    def kernel_shapes(self):
        """(row shape, column shape) of the plan's pass kernels."""
        return self._plan.shapes

    @kernel_shapes.setter
    def kernel_shapes(self, shapes):
        self._plan.set_shapes(*shapes)

    def autotune(self, n_steps=None):
        """Time ``n_steps`` full steps (default ``tuning.default_steps``) in
        every pair of kernel shapes, each from the current state, and keep
        the fastest; the state is unchanged.  The choice is remembered for
        this grid (``spinor_gpe.tuning``).  Returns {(row, col): microseconds
        per step}, also kept as ``tune_times``."""
        ny, nx = self._shape
        if n_steps is None:
            n_steps = tuning.default_steps(ny, nx)
        shapes, times = self._plan.autotune(torch, n_steps, self._device)
        tuning.remember(self._bits, ny, nx, shapes)
        self.tune_times = times
        return times

    def full_steps(self, n_steps, pops=None):
        """``n_steps`` full steps in one call; ``pops`` is an optional
        (n_steps, 2) float64 device tensor receiving the populations after
        each step (the last row is filled when the state is next read)."""
        if pops is not None:
            if (pops.dtype != torch.float64 or pops.device != self._device
                    or tuple(pops.shape) != (n_steps, 2)
                    or not pops.is_contiguous()):
                raise ValueError('pops must be a contiguous (n_steps, 2) '
                                 'float64 tensor on the propagator device')
        self._plan.full_steps(torch, n_steps, self._device, pops)
        self._psik_cache = None

    def prop_loop(self, n_steps):
        """Propagate ``n_steps`` full steps; record populations every step and
        optionally sample psik (tensor_propagator.py:151-212)."""
        pop_times = np.linspace(0, self.n_steps * np.abs(self.t_step),
                                n_steps)
        pops = {'times': pop_times, 'vals': np.empty((n_steps, 2))}
        pops_dev = torch.empty((max(n_steps, 1), 2), dtype=torch.float64,
                               device=self._device)
        if self.is_sampling:
            n_samples = int(n_steps / self.sample_rate)
            ny, nx = self._shape
            sampled_psik = np.empty((n_samples, 2, ny, nx),
                                    dtype=np.complex128)
            sampled_times = np.linspace(0, self.n_steps * np.abs(self.t_step),
                                        n_samples)
            rate = int(self.sample_rate)
            bounds = list(range(0, n_steps, rate)) + [n_steps]
        else:
            chunk = max(1, min(n_steps, 200))
            bounds = list(range(0, n_steps, chunk)) + [n_steps]
        bar = _tqdm(range(len(bounds) - 1), disable=len(bounds) < 3)
        for b in bar:
            i0, i1 = bounds[b], bounds[b + 1]
            if self.is_sampling:
                idx = i0 // rate
                sampled_psik[idx] = np.array(ttools.to_numpy(self.psik))
            if i1 > i0:
                self.full_steps(i1 - i0, pops_dev[i0:i1])
        psik_t = self.psik                  # also fills the last pops row
        pops['vals'][:] = pops_dev[:n_steps].cpu().numpy()
        energy = self.eng_expect(psik_t)

        if self.is_sampling:
            test_name = self.paths['trial'] + 'psik_sampled'
            file_name = next_available_path(test_name, self.paths['folder'],
                                            '.npz')
            np.savez(file_name, psiks=sampled_psik, times=sampled_times)
        else:
            file_name = None

        psi_t = ttools.ifft_2d(psik_t, self._space_np['dr'])
        derived = {k: (ttools.to_numpy(v) if isinstance(v, list) else v)
                   for k, v in self.analysis(psi_t, psik_t).items()}
        psik = ttools.to_numpy(psik_t)
        psi = ttools.to_numpy(psi_t)
        self.check_device()
        return prop_result.PropResult(psi, psik, energy, pops, file_name,
                                      derived=derived)

    def analysis(self, psi=None, psik=None):
        """Derived fields of a spinor computed on the device (the
        original's ``PropResult`` fields, prop_result.py:76-88): component
        densities ``dens``, k-space densities ``densk``, phases ``phase``
        (zero where the density is below 1e-6 of its maximum), and ``sums``
        = [sum n0 n1, sum n0^2, sum n1^2, max n0, max n1] in FP64 with
        ``separation`` = 1 - sums[0] / sqrt(sums[1] sums[2]).  Defaults:
        the current state."""
        if psik is None:
            psik = self.psik
        if psi is None:
            psi = ttools.ifft_2d(psik, self._space_np['dr'])
        psi = [torch.as_tensor(p, device=self._device).to(self._ctype).contiguous()
               for p in psi]
        psik = [torch.as_tensor(p, device=self._device).to(self._ctype).contiguous()
                for p in psik]
        def empty():
            return [torch.empty(self._shape, dtype=self._rtype, device=self._device)
                    for _ in range(2)]
        dens, densk, phase = empty(), empty(), empty()
        sums = torch.empty(5, dtype=torch.float64, device=self._device)
        self._plan.analysis(torch, psi, psik, dens, densk, phase, sums)
        s = sums.cpu().numpy()
        return {'dens': dens, 'densk': densk, 'phase': phase, 'sums': s,
                'separation': float(1 - s[0] / np.sqrt(s[1] * s[2]))}

    # --------------------------------------------------------------- energy
    ENERGY_KEYS = ('kin', 'pot', 'int', 'cpl', 'total', 'mu', 'atoms_k',
                   'atoms_r', 's1', 's2')

    def _set_energy_fields(self):
        """Slot 0: the energy of the propagated Hamiltonian (K_c as
        propagated, V_c, coupling h = (Omega/2) exp(-i theta)).  Slot 1: the
        original's reporting convention (tensor_propagator.py:308-324):
        free kinetic energy plus kL kx with coupling, h = Omega/2."""
        kin0 = [ops.energy_pair(d)
                for d in ops.Prepared.decompose(self._kin_np)]
        pot = [ops.energy_pair(d) for d in self._prepared.pot]
        nx = self._shape[1]
        cpl0 = ops.coupling_energy_spec(self._coupling_np, self._expon_np, nx)
        self._plan.set_energy_fields(0, kin0, pot, cpl0)
        if self._kx_np is not None and self._ky_np is not None:
            k_ref = (self._kx_np**2 + self._ky_np**2) / 2
            if self.is_coupling:
                k_ref = k_ref + self.kL_recoil * self._kx_np
            kin1 = [ops.energy_pair(ops.Decomposition(k_ref))] * 2
            cpl1 = ops.coupling_energy_spec(self._coupling_np, None, nx)
            self._plan.set_energy_fields(1, kin1, pot, cpl1)
            self._has_ref_energy = True
        else:
            self._has_ref_energy = False

    def _energy_values(self, slot, psik=None):
        if psik is None:
            psik = self.psik
        psik = [torch.as_tensor(p, device=self._device).to(self._ctype)
                .contiguous() for p in psik]
        out = torch.empty(10, dtype=torch.float64, device=self._device)
        self._plan.energy(torch, slot, psik, out)
        return out.cpu().numpy()

    def energy_to(self, out, psik=None, slot=0):
        """Queue the FP64 energy functional of ``psik`` (default: the current
        state) into ``out``, a float64 device tensor of 10 values ordered as
        ``ENERGY_KEYS``, on the current stream, without waiting for it."""
        if psik is None:
            psik = self.psik
        psik = [torch.as_tensor(p, device=self._device).to(self._ctype)
                .contiguous() for p in psik]
        if (out.dtype != torch.float64 or out.device != self._device
                or out.numel() != 10 or not out.is_contiguous()):
            raise ValueError('out must be 10 contiguous float64 values on the '
                             'propagator device')
        self._plan.energy(torch, slot, psik, out)
        return out

    def energy(self, psik=None):
        """FP64 energy functional of ``psik`` (default: the current state),
        computed on the device: kinetic (spectral, with the propagated K_c),
        potential, interaction (g_ij/2 n_i n_j), coupling, total, chemical
        potential mu and the atom numbers in k- and real space."""
        vals = self._energy_values(0, psik)
        return dict(zip(self.ENERGY_KEYS, (float(v) for v in vals)))

    def eng_expect(self, psik):
        """[E_tot, E_kin, E_pot, E_int] in the convention of
        ``tensor_propagator.py:273-324`` (grid sums without the area
        element, interaction without the 1/2, coupling without the Raman
        phase).  The kinetic term sum(|grad sqrt(n)|^2 + n |grad phi|^2
        + 2 kL n d_x phi)/2 is evaluated spectrally as
        sum_k ((kx^2+ky^2)/2 + kL kx) |psik|^2 dv_k / dv_r (the kL term only
        with coupling), which needs no phase unwrapping."""
        assert len(psik) == 2, ("Requires two spinor components to calculate "
                                "the energy expectation value.")
        if not self._has_ref_energy:
            raise ValueError('eng_expect needs the k-space meshes of the '
                             'PSpinor (space kx_mesh / ky_mesh)')
        v = self._energy_values(1, psik)
        dv_r = float(self._space_np['dv_r'])
        kin, pot = v[0] / dv_r, v[1] / dv_r
        int_e = (v[8] + v[9]) / dv_r
        cpl = v[3] / dv_r
        return [kin + pot + int_e + cpl, kin, pot, int_e]
