"""``DeviceSpinor``: the ``PSpinor`` set-up with its O(Nx Ny) work on the GPU.

Same constructor arguments, attributes and methods as ``PSpinor``
(``spinor_gpe/pspinor/pspinor.py:113-745``), for the separable problems the
set-up methods produce (harmonic traps, free and momentum-shifted kinetic
energies, uniform or gradient couplings and detunings):

* the meshes and energy grids are ``ops.SepField`` objects (value
  a[x] + b[y] from two 1-D FP64 parts; ``np.asarray`` forms the 2-D array on
  request), so the propagator builds its operators from the 1-D parts;
* ``psi`` / ``psik`` are CUDA tensors, written by native kernels
  (``sgpe_setup_spinor``, ``sgpe_imprint_vortices``, ``sgpe_fourier_split_x``)
  and the native transforms.

Differences from ``PSpinor``: grids are formed as sums of 1-D parts (for
example x^2/2 + y^2/2 instead of (x^2 + y^2)/2), so set-up values can differ
from the host path in the last bits; the Thomas-Fermi file ``tf_wf-*.npz`` is
not written (the state never leaves the device unless read).  The operator
set-up in ``TensorPropagator`` then costs O(Nx + Ny) on the host.
"""
import numpy as np
import torch

from . import _native
from . import operators as ops
from . import tensor_tools as ttools
from .pspinor import PSpinor


def _dev64(a, device):
    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device=device)


class DeviceSpinor(PSpinor):
    """``PSpinor`` with device-side state set-up (see the module docstring).

    Extra keyword arguments: ``device`` (CUDA device, default 'cuda') and
    ``dtype`` (64 or 128: complex64 or complex128 wavefunctions, default
    128)."""

    # pylint: disable=too-many-arguments,super-init-not-called
    def __init__(self, path, omeg=None, g_sc=None, mesh_points=(256, 256),
                 r_sizes=(16, 16), atom_num=1e4, pop_frac=(0.5, 0.5),
                 **kwargs):
        phase_factor = kwargs.get('phase_factor', 1)
        overwrite = kwargs.get('overwrite', False)
        self.device = torch.device(kwargs.get('device', 'cuda'))
        if self.device.type != 'cuda':
            raise ValueError('DeviceSpinor builds its state on a CUDA device')
        if self.device.index is None:
            self.device = torch.device('cuda', torch.cuda.current_device())
        self.bits = 64 if kwargs.get('dtype', 128) in (64, torch.complex64) else 128
        self.ctype = torch.complex64 if self.bits == 64 else torch.complex128
        self.setup_data_path(path, overwrite)
        self.atom_num = atom_num
        self.space = {}
        assert sum(pop_frac) == 1.0, "Total population must equal 1."
        self.pop_frac = pop_frac
        if omeg is None:
            omeg0 = 2 * np.pi * 50
            self.omeg = {'x': omeg0, 'y': omeg0, 'z': 40 * omeg0}
        else:
            names = {'x', 'y', 'z'}
            assert names == omeg.keys(), ("Keys for `omeg` must have "
                                          f"the form: {names}.")
            self.omeg = omeg
        if g_sc is None:
            self.g_sc = {'uu': 1.0, 'dd': 0.995, 'ud': 0.995}
        else:
            names = {'uu', 'dd', 'ud'}
            assert names == g_sc.keys(), ("Keys for `g_sc` must have "
                                          f"the form: {names}.")
            self.g_sc = g_sc
        self.compute_tf_params()
        self.compute_spatial_grids(mesh_points, r_sizes)
        self.compute_energy_grids()
        self.compute_tf_psi(phase_factor)
        self.no_coupling_setup()
        self.rand_seed = None
        self.prop = None
        nx, ny = self.space['mesh_points']
        self.coupling = ops.SepField(np.zeros(nx), np.zeros(ny))
        self.detuning = ops.SepField(np.zeros(nx), np.zeros(ny))
        self.rot_coupling = True

    # ---------------------------------------------------------------- grids
    def compute_spatial_grids(self, mesh_points=(256, 256), r_sizes=(16, 16)):
        """1-D grids and separable meshes (pspinor.py:315-364)."""
        assert all(point % 2 == 0 for point in mesh_points), (
            f"Number of mesh points {mesh_points} should be powers of 2.")
        mesh_points = np.array(mesh_points)
        r_sizes = np.array(r_sizes)
        self.space['dr'] = 2 * r_sizes / mesh_points
        k_sizes = np.pi / self.space['dr']
        self.space['dk'] = np.pi / r_sizes
        for name, sizes, axis in (('x', r_sizes, 0), ('y', r_sizes, 1),
                                  ('kx', k_sizes, 0), ('ky', k_sizes, 1)):
            self.space[name] = self._compute_lin(sizes, mesh_points, axis=axis)
        zx, zy = np.zeros(mesh_points[0]), np.zeros(mesh_points[1])
        self.space['x_mesh'] = ops.SepField(self.space['x'], zy)
        self.space['y_mesh'] = ops.SepField(zx, self.space['y'])
        self.space['kx_mesh'] = ops.SepField(self.space['kx'], zy)
        self.space['ky_mesh'] = ops.SepField(zx, self.space['ky'])
        self.space['dv_r'] = np.prod(self.space['dr'])
        self.space['dv_k'] = np.prod(self.space['dk'])
        self.space['mesh_points'] = mesh_points
        self.space['r_sizes'] = r_sizes
        self.space['k_sizes'] = k_sizes

    def compute_energy_grids(self):
        """Harmonic trap and free kinetic energy, separable (pspinor.py:413-430)."""
        y_trap = self.omeg['y'] / self.omeg['x']
        self.pot_eng = ops.SepField(self.space['x']**2 / 2,
                                    (y_trap * self.space['y'])**2 / 2)
        self.kin_eng = ops.SepField(self.space['kx']**2 / 2,
                                    self.space['ky']**2 / 2)

    # ---------------------------------------------------------------- state
    def set_tf_state(self, mu, amps, noise=0.0, seed=0, renorm=True):
        """psi_c = sqrt(max(mu - V, 0)) amps[c] exp(i phi_c) on the device,
        phi_c ~ U(-noise, noise) (seeded hash), renormalised to atom_num when
        ``renorm``; sets ``psi`` and ``psik``."""
        lib = _native.load()
        nx, ny = self.space['mesh_points']
        pot = self.pot_eng
        vx, vy = _dev64(pot.a, self.device), _dev64(pot.b, self.device)
        amp = np.array([complex(a) for a in amps], dtype=np.complex128).view(np.float64)
        amp_t = np.ascontiguousarray(amp)
        scratch = torch.empty(304, dtype=torch.float64, device=self.device)
        psi = [torch.empty((ny, nx), dtype=self.ctype, device=self.device) for _ in range(2)]
        stream = torch.cuda.current_stream(self.device).cuda_stream
        _native.check(lib.sgpe_setup_spinor(
            self.bits, int(ny), int(nx), _native.c_ptr(vx), _native.c_ptr(vy),
            float(mu), amp_t.ctypes.data_as(_native.c_void_p),
            float(noise), int(seed) & 0xFFFFFFFFFFFFFFFF,
            float(self.atom_num) if renorm else 0.0, float(self.space['dv_r']),
            _native.c_ptr(scratch), _native.c_ptr(psi[0]), _native.c_ptr(psi[1]),
            _native.c_void_p(stream)))
        self.psi = psi
        self.psik = ttools.fft_2d(self.psi, self.space['dr'])
        return scratch

    def compute_tf_psi(self, phase_factor=1.0):
        """Thomas-Fermi spinor on the device (pspinor.py:248-281)."""
        assert abs(phase_factor) == 1.0, ("Relative phase factor must have "
                                          "unit magnitude.")
        g_bare = [self.g_sc['uu'], self.g_sc['dd']]
        amps = [np.sqrt(pop / abs(g)) for pop, g in zip(self.pop_frac, g_bare)]
        amps[1] = amps[1] * phase_factor
        scratch = self.set_tf_state(self.chem_pot, amps)
        # healing lengths from the peak density of the renormalised state
        total = float(np.sum(scratch.cpu().numpy()))
        scale2 = self.atom_num / (float(self.space['dv_r']) * total)
        peak = max(self.chem_pot - self.pot_eng.min(), 0.0)
        self.heal = [(8 * np.pi * peak * abs(a)**2 * scale2 * self.a_sc)**(-1 / 2)
                     for a in amps]

    def coupling_setup(self, wavel=790.1e-9, scale=1.0, kin_shift=False):
        """Raman recoil and spin-dependent kinetic shift, min-shifted
        (pspinor.py:476-501)."""
        self.is_coupling = True
        # pylint: disable=invalid-name
        self.kL_recoil = scale * (np.sqrt(2) * np.pi / wavel * self.a_x)
        self.EL_recoil = self.kL_recoil**2 / 2
        shift = self.space['kx_mesh'] * self.kL_recoil if kin_shift else 0.0
        kin = [self.kin_eng + shift, self.kin_eng - shift]
        self.kin_eng_spin = [k - k.min() for k in kin]

    def coupling_grad(self, slope, offset, axis=1):
        """Linear coupling gradient (pspinor.py:577-606)."""
        self.coupling = self._axis_mesh(axis) * slope + offset

    def coupling_uniform(self, value):
        """Uniform coupling (pspinor.py:608-625)."""
        assert value >= 0, f"Cannot have a negative coupling value: {value}."
        nx, ny = self.space['mesh_points']
        self.coupling = ops.SepField(np.full(nx, float(value)), np.zeros(ny))

    def detuning_uniform(self, value):
        """Uniform detuning (pspinor.py:662-678)."""
        nx, ny = self.space['mesh_points']
        self.detuning = ops.SepField(np.full(nx, float(value)), np.zeros(ny))

    def seed_vortices(self, positions, windings):
        """Imprint vortices on the device (pspinor.py:680-745)."""
        positions = np.array(positions, dtype=np.float64)
        assert positions.shape[-1] == 2, ("Positions should be ordered "
                                          "pairs, e.g. (x, y).")
        ident_pos = False
        if len(positions.shape) == 2:
            n_pos = len(positions)
            positions = np.array([positions, positions])
            ident_pos = True
        else:
            assert len(positions.shape) == 3, ("`positions` must be at most "
                                               "a three-dimensional array.")
        windings = np.array(windings)
        if windings.shape == (1,):
            windings = windings * np.ones(positions.shape[:-1], dtype=int)
        elif len(windings.shape) == 1:
            assert ident_pos and len(windings) == n_pos, \
                ("The number of supplied windings must match the number of "
                 "supplied positions")
            windings = np.array([windings, windings])
        elif len(windings.shape) == 2:
            assert windings.shape == positions.shape[:-1], \
                ("The number of supplied windings must match the number of "
                 "supplied positions")
        rows = [(c, x, y, float(windings[c, j]))
                for c in range(2) for j, (x, y) in enumerate(positions[c])]
        vort = _dev64(np.array(rows, dtype=np.float64).reshape(-1, 4), self.device)
        x, y = _dev64(self.space['x'], self.device), _dev64(self.space['y'], self.device)
        heal = np.ascontiguousarray(self.heal, dtype=np.float64)
        nx, ny = self.space['mesh_points']
        stream = torch.cuda.current_stream(self.device).cuda_stream
        _native.check(_native.load().sgpe_imprint_vortices(
            self.bits, int(ny), int(nx), _native.c_ptr(x), _native.c_ptr(y),
            _native.c_ptr(vort), len(rows), heal.ctypes.data_as(_native.c_void_p),
            _native.c_ptr(self.psi[0]), _native.c_ptr(self.psi[1]),
            _native.c_void_p(stream)))
        self.psik = ttools.fft_2d(self.psi, delta_r=self.space['dr'])

    def shift_momentum(self, psik=None, scale=1.0, frac=(0.5, 0.5)):
        """Momentum split by +/- scale * kL_recoil on the device
        (pspinor.py:503-545)."""
        assert self.is_coupling, ("The `is_coupling` option is "
                                  f"{self.is_coupling}. Initialize coupling "
                                  "with `coupling_setup()`.")
        if psik is None:
            psik = self.psik
        shift = scale * self.kL_recoil / self.space['dk'][0]
        input_ = ttools.fft_2d(psik, self.space['dr'])
        nx, ny = self.space['mesh_points']
        stream = torch.cuda.current_stream(self.device).cuda_stream
        result = [torch.empty_like(p) for p in input_]
        for i in range(2):
            _native.check(_native.load().sgpe_fourier_split_x(
                self.bits, int(ny), int(nx), float(shift), float(frac[0]),
                float(frac[1]), _native.c_ptr(input_[i]), _native.c_ptr(result[i]),
                _native.c_void_p(stream)))
            frac = np.flip(frac)
        self.psik = ttools.ifft_2d(result, self.space['dr'])
        self.psi = ttools.ifft_2d(self.psik, self.space['dr'])
