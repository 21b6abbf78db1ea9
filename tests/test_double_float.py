"""The double-float precision (``dtype='double-float'``) and the long-horizon
error of every precision.

Double-float plans keep the state, the operator tables and the transforms
in FP32 head + tail pairs (about 48 significant bits).  They are checked
with the complex128 tolerance (relative L2 1e-10 against the complex128
reference): on the golden vectors of the original package, against the
oracle at the problem sizes, through the PSpinor / prop_loop API and for the
energy functional.

The long-horizon test runs the 1024^2 Raman-dressed problem in real time for
400 full steps in every precision against the complex128 oracle (run on the
same GPU).  Its bounds come from the measured error-vs-step curves of the
full 3000 + 10000-step problem: complex64 arithmetic reaches ~1e-4 within a
few hundred real-time steps (6.4e-4 after 13000), while double-float and
complex128 stay near 1e-12 over the whole run.
"""
import numpy as np
import pytest
import torch

from conftest import case_params, load_cases, prop_case_names, rel_l2, spin_from_case
from oracle import OracleInputs, OraclePropagator
from oracle.energy import energy_functional

pytestmark = pytest.mark.gpu

DF = 'double-float'
TOL = 1e-10                          # the complex128 tolerance
CASES = load_cases()
C128_CASES = [n for n in prop_case_names(CASES) if not n.endswith('_c64')]


@pytest.fixture(scope='module')
def tp():
    assert torch.cuda.is_available(), 'these tests need a CUDA device'
    from spinor_gpe.pspinor import tensor_propagator
    return tensor_propagator


def _inputs(ps):
    return OracleInputs(
        psik=[np.asarray(p) for p in ps.psik],
        kin_eng_spin=[np.asarray(k) for k in ps.kin_eng_spin],
        pot_eng_spin=[np.asarray(v) for v in ps.pot_eng_spin],
        coupling=np.asarray(ps.coupling, dtype=np.float64),
        x_mesh=ps.space['x_mesh'], dr=ps.space['dr'],
        dv_r=float(ps.space['dv_r']), dv_k=float(ps.space['dv_k']),
        g_sc=dict(ps.g_sc), atom_num=float(ps.atom_num),
        kL_recoil=float(ps.kL_recoil), rot_coupling=bool(ps.rot_coupling),
        is_coupling=bool(ps.is_coupling))


def _state(prop):
    return np.array([t.cpu().numpy() for t in prop.psik])


@pytest.mark.parametrize('name', C128_CASES)
def test_double_float_matches_golden_vectors(tp, tmp_path, name):
    case = CASES[name]
    p = case_params(case)
    spin = spin_from_case(case, tmp_path)
    prop = tp.TensorPropagator(spin, p['dt'], p['n_steps'], 'cuda', time=p['time'], dtype=DF)
    assert prop.psik[0].dtype == torch.complex128
    prop.single_step(prop.dt_out, prop.eng_out)
    assert rel_l2(_state(prop), case['psik_single_out']) <= TOL
    prop = tp.TensorPropagator(spin, p['dt'], p['n_steps'], 'cuda', time=p['time'], dtype=DF)
    prop.full_step()
    assert rel_l2(_state(prop), case['psik_step1']) <= TOL
    n = p['n_steps'] - 1
    pops = torch.empty((n, 2), dtype=torch.float64, device='cuda')
    prop.full_steps(n, pops)
    assert rel_l2(_state(prop), case['psik_final']) <= TOL
    np.testing.assert_allclose(pops.cpu().numpy(), case['pops'][1:], rtol=0, atol=1e-12)


def test_double_float_load_store_round_trip(tp, tmp_path):
    """psik read back before any step: the complex128 values as head + tail
    (2^-48 relative)."""
    case = CASES['imag_raman_64']
    prop = tp.TensorPropagator(spin_from_case(case, tmp_path), 0.01, 1, 'cuda', dtype=DF)
    assert rel_l2(_state(prop), case['psik0']) <= 1e-14


def test_double_float_ground_state_256_and_energy(tp, tmp_path):
    from spinor_gpe import workloads
    from spinor_gpe.pspinor import pspinor as spin
    from spinor_gpe.pspinor import tensor_tools as ttools
    ps = workloads.ground_state_256(spin.PSpinor, ttools.fft_2d, str(tmp_path / 'c1') + '/')
    n = 20
    orc = OraclePropagator(_inputs(ps), 0.02, 'imag', 128)
    ref_pops = orc.run(n)
    ref = orc.psik_numpy()
    prop = tp.TensorPropagator(ps, 0.02, n, 'cuda', time='imag', dtype=DF)
    pops = torch.empty((n, 2), dtype=torch.float64, device='cuda')
    prop.full_steps(n, pops)
    got = _state(prop)
    assert rel_l2(got, ref) <= TOL
    np.testing.assert_allclose(pops.cpu().numpy(), ref_pops, rtol=0, atol=1e-12)
    # FP64 energy functional of the double-float state (complex128 transforms)
    e = prop.energy()
    theta = 0.0 if ps.rot_coupling else 2 * ps.kL_recoil * ps.space['x_mesh']
    want = energy_functional(ref, ps.kin_eng_spin, ps.pot_eng_spin,
                             np.asarray(ps.coupling, dtype=np.float64), theta,
                             (ps.g_sc['uu'], ps.g_sc['dd'], ps.g_sc['ud']),
                             ps.space['dr'], float(ps.space['dv_r']), float(ps.space['dv_k']))
    assert abs(e['total'] - want[4]) <= 1e-10 * abs(want[4])
    assert abs(e['mu'] - want[5]) <= 1e-10 * abs(want[5])


def test_double_float_through_pspinor_api(tmp_path):
    """imaginary() then real() with dtype='double-float' (PropResult
    contract as for the other precisions)."""
    from spinor_gpe import workloads
    from spinor_gpe.pspinor import pspinor as spin
    from spinor_gpe.pspinor import tensor_tools as ttools
    ps = workloads.build(spin.PSpinor, ttools.fft_2d, str(tmp_path / 'loop') + '/',
                         nx=64, ny=128, half_x=4.0, half_y=8.0,
                         g=(300.0, 298.0, 296.0), omega=0.7, k_l=3.0,
                         rot_coupling=False, seed=5)
    orc = OraclePropagator(_inputs(ps), 0.01, 'imag', 128)
    ref_pops = orc.run(10)
    res, _ = ps.imaginary(0.01, 10, 'cuda', dtype=DF)
    assert rel_l2(res.psik, orc.psik_numpy()) <= TOL
    np.testing.assert_allclose(res.pops['vals'], ref_pops, rtol=0, atol=1e-12)
    ps.detuning_uniform(0.3)
    orc2 = OraclePropagator(_inputs(ps), 1e-3, 'real', 128)
    orc2.run(6, record_pops=False)
    res2, _ = ps.real(1e-3, 6, 'cuda', dtype=DF)
    assert rel_l2(res2.psik, orc2.psik_numpy()) <= TOL


@pytest.mark.parametrize('shape', [(192, 384), (768, 256), (32, 4096)])
def test_double_float_radix3_and_extreme_shapes(tp, tmp_path, shape):
    from spinor_gpe import workloads
    from spinor_gpe.pspinor import pspinor as spin
    from spinor_gpe.pspinor import tensor_tools as ttools
    ny, nx = shape
    ps = workloads.build(spin.PSpinor, ttools.fft_2d, str(tmp_path / 'x') + '/',
                         nx=nx, ny=ny, half_x=nx * 0.0625 / 2, half_y=ny * 0.0625 / 2,
                         g=(100.0, 100.0, 99.0), omega=1.0, k_l=3.0, delta=0.2, seed=3)
    orc = OraclePropagator(_inputs(ps), 1e-3, 'real', 128)
    orc.run(3, record_pops=False)
    prop = tp.TensorPropagator(ps, 1e-3, 3, 'cuda', time='real', dtype=DF)
    prop.full_steps(3)
    assert rel_l2(_state(prop), orc.psik_numpy()) <= TOL


# bounds of the 400-step real-time run (relative L2 against complex128);
# measured on GB300: complex64 8.5e-5, complex128 2.5e-13, double-float 1.5e-12
LONG_BOUND = {64: 2e-4, 128: 1e-10, DF: 1e-10}


def test_long_horizon_real_time_1024_every_precision(tp, tmp_path):
    """400 real-time full steps of the 1024^2 Raman-dressed problem
    (delta = 0.5) in complex64, complex128 and double-float against the
    complex128 oracle."""
    from spinor_gpe import workloads
    from spinor_gpe.pspinor import pspinor as spin
    from spinor_gpe.pspinor import tensor_tools as ttools
    ps = workloads.raman_quench_1024(spin.PSpinor, ttools.fft_2d, str(tmp_path / 'c2') + '/', delta=0.5)
    n = 400
    orc = OraclePropagator(_inputs(ps), 1e-3, 'real', 128, device='cuda')
    for _ in range(n):
        orc.full_step()
    ref = orc.psik_numpy()
    del orc
    errs = {}
    for dtype in (64, 128, DF):
        prop = tp.TensorPropagator(ps, 1e-3, n, 'cuda', time='real', dtype=dtype)
        prop.full_steps(n)
        errs[dtype] = rel_l2(_state(prop).astype(np.complex128), ref)
        del prop
    print('long-horizon errors', errs)
    for dtype, e in errs.items():
        assert e <= LONG_BOUND[dtype], (dtype, e)


def test_double_float_in_a_batch_matches_alone(tp, tmp_path):
    """A batch mixing a double-float plan with complex64 and complex128
    plans (the double-float plan runs as its own graph branch) gives every
    solve exactly what it gives alone; double-float plans have one kernel
    shape, so autotuning leaves them as they are."""
    from spinor_gpe.batch import PropagatorBatch
    names = ['imag_raman_64', 'real_raman_32', 'imag_plain_32']
    dtypes = [DF, 64, 128]

    def make(i):
        case = CASES[names[i]]
        p = case_params(case)
        return tp.TensorPropagator(spin_from_case(case, tmp_path / f'b{i}'), p['dt'], 8,
                                   'cuda', time=p['time'], dtype=dtypes[i])
    alone = []
    for i in range(3):
        prop = make(i)
        prop.full_steps(12)
        alone.append(_state(prop))
    props = [make(i) for i in range(3)]
    assert props[0].kernel_shapes == (0, 0)
    props[0].autotune()
    assert props[0].kernel_shapes == (0, 0)
    batch = PropagatorBatch(props)
    batch.full_steps(12)
    for i, prop in enumerate(props):
        np.testing.assert_array_equal(_state(prop), alone[i])
    batch.close()
