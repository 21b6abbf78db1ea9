"""Drop-in ``PSpinor``: problem set-up and the ``imaginary()`` / ``real()``
entry points of spinor-gpe (``spinor_gpe/pspinor/pspinor.py``).

The set-up (grids, Thomas-Fermi state, interaction scaling, Raman coupling
and detuning fields, vortex seeding, momentum shift) runs once per problem on
the host in NumPy, with the same formulas and the same order of floating
point operations as the original, so the fields it produces are identical.
``imaginary()`` and ``real()`` hand the problem to the GPU propagator
(``tensor_propagator.TensorPropagator``).

Differences: ``device`` defaults to ``'cuda'`` and a ``dtype`` keyword (64 or
128) selects complex64 or complex128 propagation; a relative ``path`` is
created under ``./data/`` of the working directory; matplotlib plotting
methods raise ``NotImplementedError``.
"""
import os
import shutil

import numpy as np
from scipy.ndimage import fourier_shift

from .. import constants as const
from . import tensor_tools as ttools
from . import tensor_propagator as tprop


# pylint: disable=too-many-public-methods,too-many-instance-attributes
class PSpinor:
    """Pseudospin-1/2 GPE problem (see the module docstring).

    Lengths are in units of the x-trap oscillator length a_x, energies in
    hbar * omeg['x'] (``pspinor.py:20-111``).
    """

    # pylint: disable=too-many-arguments
    def __init__(self, path, omeg=None, g_sc=None, mesh_points=(256, 256),
                 r_sizes=(16, 16), atom_num=1e4, pop_frac=(0.5, 0.5),
                 **kwargs):
        phase_factor = kwargs.get('phase_factor', 1)
        overwrite = kwargs.get('overwrite', False)
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
        self.coupling = np.zeros(np.flip(mesh_points))
        self.detuning = np.zeros(np.flip(mesh_points))
        self.rot_coupling = True

    # ---------------------------------------------------------------- set-up
    def setup_data_path(self, path, overwrite):
        """Create the data directory tree {data, trial_data, code}
        (pspinor.py:198-246)."""
        if not os.path.isabs(path):
            data_path = os.path.join(os.getcwd(), 'data', path) + '/'
        else:
            data_path = path
        trial_data_path = data_path + 'trial_data/'
        code_data_path = data_path + 'code/'
        if os.path.isdir(data_path):
            if not overwrite:
                raise FileExistsError(
                    f"The directory {data_path} already exists. "
                    "To overwrite this directory, supply the parameter "
                    "`overwrite=True`.")
            shutil.rmtree(data_path)
        data_path = f'{os.path.normpath(data_path)}{os.sep}'
        code_data_path = f'{os.path.normpath(code_data_path)}{os.sep}'
        trial_data_path = f'{os.path.normpath(trial_data_path)}{os.sep}'
        for p in (data_path, code_data_path, trial_data_path):
            os.makedirs(p, exist_ok=True)
        folder_name = os.path.basename(os.path.normpath(data_path))
        self.paths = {'data': data_path, 'trial': trial_data_path,
                      'code': code_data_path, 'folder': folder_name}

    def compute_tf_psi(self, phase_factor=1.0):
        """Thomas-Fermi spinor ``psi`` and its transform ``psik``
        (pspinor.py:248-281)."""
        assert abs(phase_factor) == 1.0, ("Relative phase factor must have "
                                          "unit magnitude.")
        g_bare = [self.g_sc['uu'], self.g_sc['dd']]
        profile = np.real(np.sqrt((self.chem_pot - self.pot_eng + 0.j)))
        self.psi = [profile * np.sqrt(pop / abs(g))
                    for pop, g in zip(self.pop_frac, g_bare)]
        self.psi[1] = self.psi[1] * phase_factor
        self.psi, _ = ttools.norm(self.psi, self.space['dv_r'], self.atom_num)
        self.psik = ttools.fft_2d(self.psi, self.space['dr'])
        self.heal = [(8 * np.pi * np.max(np.abs(p)**2) * self.a_sc)**(-1 / 2)
                     for p in self.psi]
        np.savez(self.paths['trial'] + 'tf_wf-' + self.paths['folder'],
                 psi=self.psi, psik=self.psik)

    def compute_tf_params(self, species='Rb87'):
        """Length, interaction and chemical-potential scales
        (pspinor.py:283-313)."""
        y_trap = self.omeg['y'] / self.omeg['x']
        z_trap = self.omeg['z'] / self.omeg['x']
        self.a_x = np.sqrt(const.hbar / (const.Rb87['m'] * self.omeg['x']))
        if species == 'Rb87':
            self.a_sc = const.Rb87['a_sc'] / self.a_x
        else:
            self.a_sc = 1
        self.chem_pot = ((4 * self.atom_num * self.a_sc * y_trap
                          * np.sqrt(z_trap / (2 * np.pi)))**(1 / 2))
        g_scale = np.sqrt(8 * z_trap * np.pi) * self.a_sc
        self.g_sc.update({k: g_scale * self.g_sc[k] for k in self.g_sc})
        self.rad_tf = np.sqrt(2 * self.chem_pot)
        self.time_scale = 1 / self.omeg['x']

    def compute_spatial_grids(self, mesh_points=(256, 256), r_sizes=(16, 16)):
        """Real- and k-space grids, spacings and volume elements
        (pspinor.py:315-364).  Arrays are (Ny, Nx) with x contiguous."""
        assert all(point % 2 == 0 for point in mesh_points), (
            f"Number of mesh points {mesh_points} should be powers of 2.")
        mesh_points = np.array(mesh_points)
        r_sizes = np.array(r_sizes)
        self.space['dr'] = 2 * r_sizes / mesh_points
        k_sizes = np.pi / self.space['dr']
        self.space['dk'] = np.pi / r_sizes
        self.space['x'] = self._compute_lin(r_sizes, mesh_points, axis=0)
        self.space['y'] = self._compute_lin(r_sizes, mesh_points, axis=1)
        self.space['kx'] = self._compute_lin(k_sizes, mesh_points, axis=0)
        self.space['ky'] = self._compute_lin(k_sizes, mesh_points, axis=1)
        x_mesh, y_mesh = np.meshgrid(self.space['x'], self.space['y'])
        kx_mesh, ky_mesh = np.meshgrid(self.space['kx'], self.space['ky'])
        self.space.update({'x_mesh': x_mesh, 'y_mesh': y_mesh,
                           'kx_mesh': kx_mesh, 'ky_mesh': ky_mesh})
        self.space['dv_r'] = np.prod(self.space['dr'])
        self.space['dv_k'] = np.prod(self.space['dk'])
        self.space['mesh_points'] = mesh_points
        self.space['r_sizes'] = r_sizes
        self.space['k_sizes'] = k_sizes

    @classmethod
    def _compute_lin(cls, sizes, points, axis=0):
        """linspace(-size, size, points, endpoint=False) (pspinor.py:366-380)."""
        return np.linspace(-sizes[axis], sizes[axis], num=points[axis],
                           endpoint=False)

    @property
    def pot_eng(self):
        """2-D potential energy grid; setting it resets ``pot_eng_spin``
        (pspinor.py:382-396)."""
        return self._pot_eng

    @pot_eng.setter
    def pot_eng(self, array):
        self._pot_eng = array
        self.pot_eng_spin = [self._pot_eng] * 2

    @property
    def kin_eng(self):
        """2-D kinetic energy grid; setting it resets ``kin_eng_spin``
        (pspinor.py:398-411)."""
        return self._kin_eng

    @kin_eng.setter
    def kin_eng(self, array):
        self._kin_eng = array
        self.kin_eng_spin = [self._kin_eng] * 2

    def compute_energy_grids(self):
        """Harmonic trap and free-particle kinetic energy (pspinor.py:413-430)."""
        y_trap = self.omeg['y'] / self.omeg['x']
        self.pot_eng = (self.space['x_mesh']**2
                        + (y_trap * self.space['y_mesh'])**2) / 2
        self.kin_eng = (self.space['kx_mesh']**2
                        + self.space['ky_mesh']**2) / 2

    def _calc_atoms(self, psi=None, space='r'):
        """Total atom number of a real- or k-space spinor (pspinor.py:432-467)."""
        if space == 'r':
            psi = self.psi if psi is None else psi
            vol_elem = self.space['dv_r']
        elif space == 'k':
            psi = self.psik if psi is None else psi
            vol_elem = self.space['dv_k']
        return ttools.calc_atoms(psi, vol_elem)

    def no_coupling_setup(self):
        """Defaults without coupling (pspinor.py:469-474)."""
        self.is_coupling = False
        self.kL_recoil = 1.0  # pylint: disable=invalid-name
        self.EL_recoil = 1.0  # pylint: disable=invalid-name

    def coupling_setup(self, wavel=790.1e-9, scale=1.0, kin_shift=False):
        """Raman recoil scales and (optionally) the spin-dependent kinetic
        momentum shift, min-shifted to zero (pspinor.py:476-501)."""
        self.is_coupling = True
        # pylint: disable=invalid-name
        self.kL_recoil = scale * (np.sqrt(2) * np.pi / wavel * self.a_x)
        self.EL_recoil = self.kL_recoil**2 / 2
        if kin_shift:
            shift = self.space['kx_mesh'] * self.kL_recoil
        else:
            shift = 0
        self.kin_eng_spin = [self.kin_eng + shift, self.kin_eng - shift]
        self.kin_eng_spin = [k - np.min(k) for k in self.kin_eng_spin]

    def shift_momentum(self, psik=None, scale=1.0, frac=(0.5, 0.5)):
        """Split each component's momentum peak by +/- scale * kL_recoil
        (pspinor.py:503-545)."""
        assert self.is_coupling, ("The `is_coupling` option is "
                                  f"{self.is_coupling}. Initialize coupling "
                                  "with `coupling_setup()`.")
        if psik is None:
            psik = self.psik
        shift = scale * self.kL_recoil / self.space['dk'][0]
        input_ = ttools.fft_2d(psik, self.space['dr'])
        result = [np.zeros_like(pk) for pk in psik]
        for i in range(len(psik)):
            positive = fourier_shift(input_[i], shift=[0, shift], axis=1)
            negative = fourier_shift(input_[i], shift=[0, -shift], axis=1)
            result[i] = frac[0] * positive + frac[1] * negative
            frac = np.flip(frac)
        self.psik = ttools.ifft_2d(result, self.space['dr'])
        self.psi = ttools.ifft_2d(self.psik, self.space['dr'])

    @property
    def coupling(self):
        """2-D coupling (Raman Rabi frequency) field (pspinor.py:547-560)."""
        return self._coupling

    @coupling.setter
    def coupling(self, array):
        self._coupling = array

    @property
    def detuning(self):
        """2-D detuning field; setting it splits ``pot_eng_spin`` into
        V +/- detuning/2 (pspinor.py:562-575)."""
        return self._detuning

    @detuning.setter
    def detuning(self, array):
        self._detuning = array
        self.pot_eng_spin = [self.pot_eng + self._detuning / 2,
                             self.pot_eng - self._detuning / 2]

    def _axis_mesh(self, axis):
        if axis == 0:
            return self.space['x_mesh']
        if axis == 1:
            return self.space['y_mesh']
        raise ValueError('axis must be 0 (x) or 1 (y)')

    def coupling_grad(self, slope, offset, axis=1):
        """Linear coupling gradient along x (axis=0) or y (axis=1)
        (pspinor.py:577-606)."""
        self.coupling = self._axis_mesh(axis) * slope + offset

    def coupling_uniform(self, value):
        """Uniform coupling (pspinor.py:608-625)."""
        assert value >= 0, f"Cannot have a negative coupling value: {value}."
        self.coupling = np.ones_like(self.space['x_mesh']) * value

    def detuning_grad(self, slope, offset=0.0, axis=1):
        """Linear detuning gradient (pspinor.py:627-660)."""
        self.detuning = self._axis_mesh(axis) * slope + offset

    def detuning_uniform(self, value):
        """Uniform detuning (pspinor.py:662-678)."""
        self.detuning = np.ones_like(self.space['x_mesh']) * value

    def seed_vortices(self, positions, windings):
        """Imprint vortices (profile r/sqrt(r^2 + xi^2) and phase
        exp(i w atan2)) at ``positions``; ``windings`` is a list (one per
        position) or a nested list per component (pspinor.py:680-745)."""
        positions = np.array(positions)
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
        for i in range(len(self.psi)):
            for j, (x, y) in enumerate(positions[i]):
                xdiff = self.space['x_mesh'] - x
                ydiff = self.space['y_mesh'] - y
                v_grid = (np.sqrt(xdiff**2 + ydiff**2) / self.heal[i])
                v_profile = (v_grid / np.sqrt(v_grid**2 + 1))
                v_phase = np.exp(windings[i, j] * 1j * np.arctan2(ydiff,
                                                                  xdiff))
                self.psi[i] = (self.psi[i] * v_profile * v_phase)
        self.psik = ttools.fft_2d(self.psi, delta_r=self.space['dr'])

    def seed_regular_vortices(self):
        """Not implemented in the original either (pspinor.py:747-752)."""
        raise NotImplementedError()

    def seed_random_vortices(self, N):  # pylint: disable=invalid-name
        """Not implemented in the original either (pspinor.py:754-756)."""
        raise NotImplementedError()

    def _no_plotting(self, *_, **__):
        raise NotImplementedError('plotting is not part of this package')

    plot_rdens = plot_kdens = plot_rphase = plot_spins = _no_plotting

    # ----------------------------------------------------------- propagation
    def _propagate(self, time, t_step, n_steps, device, is_sampling,
                   n_samples, dtype):
        prop = tprop.TensorPropagator(self, t_step, n_steps, device,
                                      time=time, is_sampling=is_sampling,
                                      n_samples=n_samples, dtype=dtype)
        result = prop.prop_loop(prop.n_steps)
        result.paths = self.paths
        result.time_scale = self.time_scale
        result.space = self.space
        self.psik = result.psik
        self.psi = result.psi
        return result, prop

    # pylint: disable=too-many-arguments
    def imaginary(self, t_step, n_steps=1000, device='cuda',
                  is_sampling=False, n_samples=1, dtype=128):
        """Imaginary-time propagation; returns (PropResult, propagator) and
        writes the final psi/psik back (pspinor.py:890-925)."""
        return self._propagate('imag', t_step, n_steps, device, is_sampling,
                               n_samples, dtype)

    def real(self, t_step, n_steps=1000, device='cuda', is_sampling=False,
             n_samples=1, dtype=128):
        """Real-time propagation; returns (PropResult, propagator) and
        writes the final psi/psik back (pspinor.py:927-962)."""
        return self._propagate('real', t_step, n_steps, device, is_sampling,
                               n_samples, dtype)
