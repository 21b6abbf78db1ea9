"""Generate the golden fixtures in this folder by running the original
spinor-gpe package on the CPU.

Run from the repository root with the path of a checkout of the original
package (read-only is enough), as the first argument or in the environment
variable ``SPINOR_GPE_REFERENCE``::

    python tests/golden/make_golden.py /path/to/spinor-gpe

matplotlib and scikit-image are imported at module level by the original
package (``spinor_gpe/pspinor/tensor_tools.py:7``,
``spinor_gpe/pspinor/plotting_tools.py:7-8``,
``spinor_gpe/pspinor/prop_result.py:8-10``) but are not installed here, so
empty stand-in modules are registered first.  Nothing on the propagation path
uses them.  ``unwrap_phase`` is reached only through ``eng_expect``, which is
recorded once, on a phase-smooth ground state, with the identity as
``unwrap_phase`` (exact when no phase wraps).

Each propagation case builds its problem with the shared recipe in
``spinor-gpe_gb300/spinor_gpe/workloads.py`` through the original ``PSpinor``
class, constructs the original ``TensorPropagator`` exactly as
``PSpinor.imaginary``/``real`` do (``spinor_gpe/pspinor/pspinor.py:890-962``)
and drives ``full_step()`` in a loop, recording ``calc_pops`` after every step
as ``prop_loop`` does (``spinor_gpe/pspinor/tensor_propagator.py:185-194``).
The complex64 cases cast the propagator's tensors after construction.

Outputs: ``cases.npz`` (propagation inputs/outputs), ``setup.npz`` (the
``PSpinor`` set-up fields of a default physical-unit problem).
"""
import importlib.util
import os
import sys
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get('SPINOR_GPE_REFERENCE')
if not REF:
    sys.exit('usage: python tests/golden/make_golden.py /path/to/spinor-gpe '
             '(or set SPINOR_GPE_REFERENCE)')


def _install_stubs():
    """Register empty stand-ins for matplotlib and scikit-image."""
    class _Anything(types.ModuleType):
        def __getattr__(self, name):
            if name.startswith('__'):
                raise AttributeError(name)
            return lambda *a, **k: None

    for name in ['matplotlib', 'matplotlib.pyplot', 'matplotlib.gridspec',
                 'matplotlib.animation', 'skimage', 'skimage.restoration']:
        sys.modules[name] = _Anything(name)
    sys.modules['matplotlib'].pyplot = sys.modules['matplotlib.pyplot']
    sys.modules['matplotlib'].gridspec = sys.modules['matplotlib.gridspec']
    sys.modules['matplotlib'].animation = sys.modules['matplotlib.animation']
    sys.modules['skimage'].restoration = sys.modules['skimage.restoration']


def _load_workloads():
    path = os.path.join(REPO, 'spinor-gpe_gb300', 'spinor_gpe', 'workloads.py')
    spec = importlib.util.spec_from_file_location('_sgpe_workloads', path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


# name: (build kwargs, time, dt, n_steps, dtype, chained-from)
CASES = {
    # plain imaginary-time ground state, no coupling (C1 in miniature)
    'imag_plain_32': (dict(nx=32, ny=32, half_x=4.0, half_y=4.0,
                           g=(100.0, 99.5, 99.0), seed=11),
                      'imag', 0.02, 12, 128),
    # non-square grid, Raman coupling in the non-rotated frame, kinetic shift
    'imag_raman_64x32': (dict(nx=64, ny=32, half_x=8.0, half_y=4.0,
                              g=(200.0, 199.0, 198.0), omega=1.5, k_l=2.0,
                              delta=0.2, rot_coupling=False, kin_shift=True,
                              seed=12),
                         'imag', 0.02, 8, 128),
    # real-time Raman quench (C2 in miniature), anisotropic trap
    'real_raman_32': (dict(nx=32, ny=32, half_x=4.0, half_y=4.0,
                           g=(100.0, 100.0, 99.0), lam=1.3, omega=1.0,
                           k_l=3.0, delta=0.5, rot_coupling=False, seed=13),
                      'real', 1e-3, 20, 128),
    # real time, rotated-frame coupling (theta = 0)
    'real_rot_32x64': (dict(nx=32, ny=64, half_x=4.0, half_y=8.0,
                            g=(150.0, 140.0, 145.0), omega=2.0, k_l=1.0,
                            delta=-0.3, rot_coupling=True, seed=14),
                       'real', 2e-3, 10, 128),
    # 64^2 imaginary time with coupling: the largest fixture
    'imag_raman_64': (dict(nx=64, ny=64, half_x=8.0, half_y=8.0,
                           g=(300.0, 298.0, 296.0), omega=0.7, k_l=3.0,
                           delta=0.0, rot_coupling=False, seed=15),
                      'imag', 0.01, 10, 128),
    # the same problems run in complex64 (tensors cast after construction)
    'imag_plain_32_c64': (dict(nx=32, ny=32, half_x=4.0, half_y=4.0,
                               g=(100.0, 99.5, 99.0), seed=11),
                          'imag', 0.02, 12, 64),
    'real_raman_32_c64': (dict(nx=32, ny=32, half_x=4.0, half_y=4.0,
                               g=(100.0, 100.0, 99.0), lam=1.3, omega=1.0,
                               k_l=3.0, delta=0.5, rot_coupling=False,
                               seed=13),
                          'real', 1e-3, 20, 64),
}

# Non-uniform operator fields, set after the recipe: (case, setter)
FIELD_CASES = {
    # y-gradient coupling and x-gradient detuning: fields that vary along one
    # axis (coupling_grad/detuning_grad, pspinor.py:577-660)
    'imag_gradients_32': (dict(nx=32, ny=32, half_x=4.0, half_y=4.0,
                               g=(120.0, 118.0, 119.0), omega=1.0, k_l=2.0,
                               rot_coupling=False, seed=16),
                          'imag', 0.02, 6, 128, 'gradients'),
    # non-separable potential bump (arbitrary pot_eng array)
    'real_bump_32': (dict(nx=32, ny=32, half_x=4.0, half_y=4.0,
                          g=(100.0, 100.0, 99.0), omega=0.5, k_l=1.5,
                          rot_coupling=False, seed=17),
                     'real', 1e-3, 10, 128, 'bump'),
}


def _apply_fields(ps, kind):
    if kind == 'gradients':
        ps.coupling_grad(0.3, 1.0, axis=1)
        ps.detuning_grad(0.05, 0.1, axis=0)
    elif kind == 'bump':
        x, y = ps.space['x_mesh'], ps.space['y_mesh']
        ps.pot_eng = 0.5 * (x**2 + y**2) + 3.0 * np.exp(-((x - 0.7)**2
                                                         + (y + 0.4)**2 * 2))
        ps.detuning_uniform(0.25)


def _cast_c64(prop, torch):
    """Cast a propagator's tensors to complex64/float32 after construction."""
    prop.psik = [p.to(torch.complex64) for p in prop.psik]
    for eng in (prop.eng_out, prop.eng_in):
        eng['kin'] = [e.to(torch.complex64) for e in eng['kin']]
        eng['pot'] = [e.to(torch.complex64) for e in eng['pot']]
        eng['coupl'] = [[e.to(torch.complex64) for e in row]
                        for row in eng['coupl']]
    prop.space = {k: (v.to(torch.float32) if v.is_floating_point() else v)
                  for k, v in prop.space.items()}


def main():
    _install_stubs()
    sys.path.insert(0, REF)
    import torch
    from spinor_gpe.pspinor import pspinor as rspin
    from spinor_gpe.pspinor import tensor_tools as rtt
    from spinor_gpe.pspinor import tensor_propagator as rtp
    wl = _load_workloads()

    tmp = tempfile.mkdtemp(prefix='sgpe_golden_')
    out = {}
    all_cases = {k: v + (None,) for k, v in CASES.items()}
    all_cases.update(FIELD_CASES)
    for name, (kw, time, dt, n_steps, dtype, fields) in all_cases.items():
        ps = wl.build(rspin.PSpinor, rtt.fft_2d, os.path.join(tmp, name) + '/',
                      **kw)
        if fields:
            _apply_fields(ps, fields)
        pre = f'{name}/'
        out[pre + 'psik0'] = np.array(ps.psik)
        out[pre + 'kin_eng_spin'] = np.array(ps.kin_eng_spin)
        out[pre + 'pot_eng_spin'] = np.array(ps.pot_eng_spin)
        out[pre + 'coupling'] = np.asarray(ps.coupling, dtype=np.float64)
        out[pre + 'x_mesh'] = ps.space['x_mesh']
        out[pre + 'y_mesh'] = ps.space['y_mesh']
        out[pre + 'dr'] = ps.space['dr']
        out[pre + 'dk'] = ps.space['dk']
        out[pre + 'dv'] = np.array([ps.space['dv_r'], ps.space['dv_k']])
        out[pre + 'g'] = np.array([ps.g_sc['uu'], ps.g_sc['dd'],
                                   ps.g_sc['ud']])
        out[pre + 'scalars'] = np.array([ps.atom_num, ps.kL_recoil,
                                         float(ps.rot_coupling),
                                         float(ps.is_coupling), dt,
                                         float(n_steps), float(dtype),
                                         1.0 if time == 'imag' else 0.0])
        prop = rtp.TensorPropagator(ps, dt, n_steps, 'cpu', time=time)
        if dtype == 64:
            _cast_c64(prop, torch)
        # one outer sub-step alone (tensor_propagator.py:224-271)
        saved = [p.clone() for p in prop.psik]
        prop.single_step(prop.dt_out, prop.eng_out)
        out[pre + 'psik_single_out'] = np.array([p.numpy() for p in prop.psik])
        prop.psik = saved
        pops = np.empty((n_steps, 2))
        for i in range(n_steps):
            prop.full_step()
            pops[i] = rtt.calc_pops(prop.psik, prop.space['dv_k'])
            if i == 0:
                out[pre + 'psik_step1'] = np.array([p.numpy()
                                                    for p in prop.psik])
        out[pre + 'psik_final'] = np.array([p.numpy() for p in prop.psik])
        out[pre + 'pops'] = pops
        print(f'{name}: {n_steps} steps, final pops {pops[-1]}')

    # The original energy convention on a phase-smooth ground state: with no
    # phase wraps, an identity stand-in for scikit-image's unwrap_phase gives
    # the original's eng_expect exactly (tensor_propagator.py:273-324).
    import skimage.restoration as _rest
    _rest.unwrap_phase = lambda a: a
    kw, time, dt, n_steps, _, _ = all_cases['imag_plain_32']
    ps = wl.build(rspin.PSpinor, rtt.fft_2d, os.path.join(tmp, 'energy') + '/', **kw)
    prop = rtp.TensorPropagator(ps, dt, n_steps, 'cpu', time=time)
    for _ in range(n_steps):
        prop.full_step()
    out['energy/psik'] = np.array([p.numpy() for p in prop.psik])
    out['energy/kx_mesh'] = ps.space['kx_mesh']
    out['energy/ky_mesh'] = ps.space['ky_mesh']
    out['energy/eng_expect'] = np.array(prop.eng_expect(prop.psik))

    # FFT helpers on a random non-square pair (tensor_tools.py:201-258)
    rng = np.random.default_rng(5)
    f_in = [rng.standard_normal((16, 32)) + 1j * rng.standard_normal((16, 32))
            for _ in range(2)]
    dr = np.array([0.25, 0.125])
    out['fft/in'] = np.array(f_in)
    out['fft/dr'] = dr
    out['fft/fft_2d'] = np.array(rtt.fft_2d(f_in, dr))
    out['fft/ifft_2d'] = np.array(rtt.ifft_2d(f_in, dr))
    out['fft/fft_1d_x'] = np.array(rtt.fft_1d(f_in, dr, axis=0))
    out['fft/fft_1d_y'] = np.array(rtt.fft_1d(f_in, dr, axis=1))
    out['fft/ifft_1d_x'] = np.array(rtt.ifft_1d(f_in, dr, axis=0))
    out['fft/ifft_1d_y'] = np.array(rtt.ifft_1d(f_in, dr, axis=1))
    np.savez_compressed(os.path.join(HERE, 'cases.npz'), **out)

    # PSpinor set-up in physical units (pspinor.py:113-501, 680-745)
    setup = {}
    ps = rspin.PSpinor(os.path.join(tmp, 'setup') + '/', overwrite=True,
                       atom_num=1e4, mesh_points=(64, 32), r_sizes=(16, 8),
                       omeg={'x': 2 * np.pi * 50, 'y': 2 * np.pi * 60,
                             'z': 2 * np.pi * 2000},
                       g_sc={'uu': 1.0, 'dd': 0.98, 'ud': 1.02},
                       pop_frac=(0.7, 0.3), phase_factor=1j)
    for k in ['x', 'y', 'kx', 'ky', 'x_mesh', 'y_mesh', 'kx_mesh', 'ky_mesh',
              'dr', 'dk', 'dv_r', 'dv_k', 'mesh_points', 'r_sizes', 'k_sizes']:
        setup['space_' + k] = np.asarray(ps.space[k])
    setup['pot_eng'] = ps.pot_eng
    setup['kin_eng'] = ps.kin_eng
    setup['psi'] = np.array(ps.psi)
    setup['psik'] = np.array(ps.psik)
    setup['g_sc'] = np.array([ps.g_sc['uu'], ps.g_sc['dd'], ps.g_sc['ud']])
    setup['scalars'] = np.array([ps.a_x, ps.a_sc, ps.chem_pot, ps.rad_tf,
                                 ps.time_scale, ps.heal[0], ps.heal[1]])
    ps.coupling_setup(wavel=790.1e-9, scale=1.3, kin_shift=True)
    setup['coupled_kin_eng_spin'] = np.array(ps.kin_eng_spin)
    setup['coupled_scalars'] = np.array([ps.kL_recoil, ps.EL_recoil])
    ps.detuning_grad(0.1, 0.05, axis=0)
    setup['detuned_pot_eng_spin'] = np.array(ps.pot_eng_spin)
    ps.coupling_grad(0.2, 1.0, axis=1)
    setup['coupling_grad'] = ps.coupling
    ps.seed_vortices([(1.0, -0.5), (-2.0, 1.5)], [1, -1])
    setup['vortex_psi'] = np.array(ps.psi)
    setup['vortex_psik'] = np.array(ps.psik)
    ps.shift_momentum(scale=0.8, frac=(0.3, 0.7))
    setup['shifted_psik'] = np.array(ps.psik)
    setup['shifted_psi'] = np.array(ps.psi)
    np.savez_compressed(os.path.join(HERE, 'setup.npz'), **setup)
    print('wrote', os.path.join(HERE, 'cases.npz'), 'and setup.npz')


if __name__ == '__main__':
    main()
