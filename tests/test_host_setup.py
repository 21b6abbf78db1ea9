"""Host-side set-up and operator construction (CPU only).

``PSpinor`` must reproduce the original's set-up fields exactly
(``tests/golden/setup.npz`` from the original package), and the compact
operator descriptions uploaded to the library must reproduce the dense
operators of the original propagator (here: the pinned oracle).
"""
import os

import numpy as np
import pytest

from conftest import prop_case_names, GOLDEN, case_params, load_cases
from oracle import OraclePropagator, inputs_from_arrays
from spinor_gpe import workloads
from spinor_gpe.pspinor import operators as ops
from spinor_gpe.pspinor import pspinor as spin
from spinor_gpe.pspinor import tensor_tools as ttools

SETUP = np.load(os.path.join(GOLDEN, 'setup.npz'))
CASES = load_cases()


def _setup_problem(tmp_path):
    return spin.PSpinor(str(tmp_path / 'setup') + '/', overwrite=True,
                        atom_num=1e4, mesh_points=(64, 32), r_sizes=(16, 8),
                        omeg={'x': 2 * np.pi * 50, 'y': 2 * np.pi * 60,
                              'z': 2 * np.pi * 2000},
                        g_sc={'uu': 1.0, 'dd': 0.98, 'ud': 1.02},
                        pop_frac=(0.7, 0.3), phase_factor=1j)


def test_pspinor_setup_is_bit_identical(tmp_path):
    ps = _setup_problem(tmp_path)
    for k in ['x', 'y', 'kx', 'ky', 'x_mesh', 'y_mesh', 'kx_mesh', 'ky_mesh',
              'dr', 'dk', 'dv_r', 'dv_k', 'mesh_points', 'r_sizes',
              'k_sizes']:
        np.testing.assert_array_equal(ps.space[k], SETUP['space_' + k])
    np.testing.assert_array_equal(ps.pot_eng, SETUP['pot_eng'])
    np.testing.assert_array_equal(ps.kin_eng, SETUP['kin_eng'])
    np.testing.assert_array_equal(np.array(ps.psi), SETUP['psi'])
    np.testing.assert_array_equal(np.array(ps.psik), SETUP['psik'])
    np.testing.assert_array_equal(
        [ps.g_sc['uu'], ps.g_sc['dd'], ps.g_sc['ud']], SETUP['g_sc'])
    np.testing.assert_array_equal(
        [ps.a_x, ps.a_sc, ps.chem_pot, ps.rad_tf, ps.time_scale, ps.heal[0],
         ps.heal[1]], SETUP['scalars'])


def test_pspinor_coupling_detuning_vortices_shift(tmp_path):
    ps = _setup_problem(tmp_path)
    ps.coupling_setup(wavel=790.1e-9, scale=1.3, kin_shift=True)
    np.testing.assert_array_equal(np.array(ps.kin_eng_spin),
                                  SETUP['coupled_kin_eng_spin'])
    np.testing.assert_array_equal([ps.kL_recoil, ps.EL_recoil],
                                  SETUP['coupled_scalars'])
    ps.detuning_grad(0.1, 0.05, axis=0)
    np.testing.assert_array_equal(np.array(ps.pot_eng_spin),
                                  SETUP['detuned_pot_eng_spin'])
    ps.coupling_grad(0.2, 1.0, axis=1)
    np.testing.assert_array_equal(ps.coupling, SETUP['coupling_grad'])
    ps.seed_vortices([(1.0, -0.5), (-2.0, 1.5)], [1, -1])
    np.testing.assert_array_equal(np.array(ps.psi), SETUP['vortex_psi'])
    np.testing.assert_array_equal(np.array(ps.psik), SETUP['vortex_psik'])
    ps.shift_momentum(scale=0.8, frac=(0.3, 0.7))
    np.testing.assert_array_equal(np.array(ps.psik), SETUP['shifted_psik'])
    np.testing.assert_array_equal(np.array(ps.psi), SETUP['shifted_psi'])


def test_pspinor_errors(tmp_path):
    path = str(tmp_path / 'p') + '/'
    spin.PSpinor(path, mesh_points=(32, 32))
    with pytest.raises(FileExistsError):
        spin.PSpinor(path, mesh_points=(32, 32))
    with pytest.raises(AssertionError):
        spin.PSpinor(str(tmp_path / 'q') + '/', mesh_points=(33, 32))
    with pytest.raises(AssertionError):
        spin.PSpinor(str(tmp_path / 'r') + '/', pop_frac=(0.5, 0.6))
    ps = spin.PSpinor(str(tmp_path / 's') + '/', mesh_points=(32, 32))
    with pytest.raises(AssertionError):
        ps.coupling_uniform(-1.0)
    with pytest.raises(AssertionError):
        ps.shift_momentum()


@pytest.mark.parametrize('name', prop_case_names(CASES))
def test_operator_specs_reproduce_dense_operators(name):
    case = CASES[name]
    p = case_params(case)
    inp = inputs_from_arrays(case)
    orc = OraclePropagator(inp, p['dt'], p['time'], 128)
    expon = None if inp.rot_coupling else 2 * inp.kL_recoil * inp.x_mesh
    ny, nx = inp.psik[0].shape
    for dt, eng, outer in [(orc.dt_out, orc.eng_out, True),
                           (orc.dt_in, orc.eng_in, False)]:
        s = ops.build_substep(dt, inp.kin_eng_spin, inp.pot_eng_spin,
                              inp.coupling, expon, outer)
        for c in range(2):
            kin = np.fft.fftshift(s.kin_a[c].dense(ny, nx)
                                  * s.kin_b[c].dense(ny, nx))
            np.testing.assert_allclose(kin, eng['kin'][c].numpy(),
                                       rtol=0, atol=1e-15)
            pot = s.pot_a[c].dense(ny, nx) * s.pot_b[c].dense(ny, nx)
            np.testing.assert_allclose(pot, eng['pot'][c].numpy(),
                                       rtol=0, atol=1e-15)
        cc, cs, ce = (s.cpl_c.dense(ny, nx), s.cpl_s.dense(ny, nx),
                      s.cpl_e.dense(ny, nx))
        mat = eng['coupl']
        for got, ref in [(cc, mat[0][0]), (cs * np.conj(ce), mat[0][1]),
                         (cs * ce, mat[1][0]), (cc, mat[1][1])]:
            np.testing.assert_allclose(got, ref.numpy(), rtol=0, atol=1e-15)
        assert s.int_z == -1.0j * dt / 2


def test_field_classification():
    nx, ny = 16, 8
    y, x = np.mgrid[0:ny, 0:nx].astype(float)
    a, b = ops.phase_op(np.full((ny, nx), 2.0), 0.1)
    assert (a.kind, b.kind) == ('uniform', 'uniform')
    a, b = ops.phase_op(x**2, 0.1)
    assert (a.kind, b.kind) == ('x', 'uniform')
    a, b = ops.phase_op(y * 3, 0.1)
    assert (a.kind, b.kind) == ('y', 'uniform')
    a, b = ops.phase_op(x**2 / 2 + (1.3 * y)**2 / 2, 0.1)
    assert (a.kind, b.kind) == ('x', 'y')
    a, b = ops.phase_op(x * y, 0.1)
    assert (a.kind, b.kind) == ('full', 'uniform')
    np.testing.assert_allclose(a.dense(ny, nx), np.exp(-0.1j * x * y))
    assert ops.value_op(np.ones((ny, nx)), nx).kind == 'uniform'


def test_numpy_transforms_match_reference():
    f = CASES['fft']
    psi = list(f['in'])
    np.testing.assert_allclose(np.array(ttools.fft_2d(psi, f['dr'])),
                               f['fft_2d'], rtol=0, atol=1e-13)
    np.testing.assert_allclose(np.array(ttools.ifft_2d(psi, f['dr'])),
                               f['ifft_2d'], rtol=0, atol=1e-13)
    np.testing.assert_allclose(np.array(ttools.fft_1d(psi, f['dr'], 0)),
                               f['fft_1d_x'], rtol=0, atol=1e-13)
    np.testing.assert_allclose(np.array(ttools.ifft_1d(psi, f['dr'], 1)),
                               f['ifft_1d_y'], rtol=0, atol=1e-13)


def test_workload_recipes_build(tmp_path):
    ps = workloads.ground_state_256(spin.PSpinor, ttools.fft_2d,
                                    str(tmp_path / 'c1') + '/', n=64)
    assert ps.psik[0].shape == (64, 64)
    assert ps.g_sc == {'uu': 1000.0, 'dd': 995.0, 'ud': 990.0}
    ps = workloads.raman_quench_1024(spin.PSpinor, ttools.fft_2d,
                                     str(tmp_path / 'c2') + '/', n=64,
                                     delta=0.5)
    assert ps.is_coupling and not ps.rot_coupling and ps.kL_recoil == 3.0
    np.testing.assert_allclose(ps.pot_eng_spin[0] - ps.pot_eng_spin[1], 0.5)
    ps = workloads.vortex_2048(spin.PSpinor, ttools.fft_2d,
                               str(tmp_path / 'c3') + '/', n=64)
    assert ps.psik[0].shape == (64, 64)
