"""Parity of the native GPU path with the original propagator.

Every check runs the drop-in ``TensorPropagator`` / ``tensor_tools`` (which
call the C ABI of ``libspinor_gb300.so``) and compares with the golden
vectors of the original package or with the pinned CPU oracle on the same
inputs.

Tolerances (relative L2 over both components, against the complex128
reference): 1e-10 for complex128 runs, 1e-5 for complex64 runs.
"""
import os

import numpy as np
import pytest
import torch

from conftest import prop_case_names, case_params, load_cases, rel_l2, spin_from_case
from oracle import OraclePropagator, OracleInputs, calc_pops

pytestmark = pytest.mark.gpu

TOL = {128: 1e-10, 64: 1e-5}
CASES = load_cases()
PROP_CASES = prop_case_names(CASES)


@pytest.fixture(scope='module')
def tp():
    assert torch.cuda.is_available(), 'these tests need a CUDA device'
    from spinor_gpe.pspinor import tensor_propagator
    return tensor_propagator


def _c128_twin(name):
    """Golden complex128 case with the same inputs as a complex64 case."""
    return CASES[name[:-4]] if name.endswith('_c64') else CASES[name]


@pytest.mark.parametrize('name', PROP_CASES)
def test_single_step_matches_reference(tp, tmp_path, name):
    case = CASES[name]
    p = case_params(case)
    prop = tp.TensorPropagator(spin_from_case(case, tmp_path), p['dt'],
                               p['n_steps'], 'cuda', time=p['time'],
                               dtype=p['dtype'])
    prop.single_step(prop.dt_out, prop.eng_out)
    got = np.array([t.cpu().numpy() for t in prop.psik])
    ref = _c128_twin(name)['psik_single_out']
    assert rel_l2(got, ref) <= TOL[p['dtype']]


@pytest.mark.parametrize('name', PROP_CASES)
def test_full_steps_and_pops_match_reference(tp, tmp_path, name):
    case = CASES[name]
    p = case_params(case)
    prop = tp.TensorPropagator(spin_from_case(case, tmp_path), p['dt'],
                               p['n_steps'], 'cuda', time=p['time'],
                               dtype=p['dtype'])
    prop.full_step()
    got1 = np.array([t.cpu().numpy() for t in prop.psik])
    twin = _c128_twin(name)
    assert rel_l2(got1, twin['psik_step1']) <= TOL[p['dtype']]
    n = p['n_steps'] - 1
    pops = torch.empty((n, 2), dtype=torch.float64, device='cuda')
    prop.full_steps(n, pops)
    got = np.array([t.cpu().numpy() for t in prop.psik])
    assert rel_l2(got, twin['psik_final']) <= TOL[p['dtype']]
    ptol = 1e-12 if p['dtype'] == 128 else 1e-6
    np.testing.assert_allclose(pops.cpu().numpy(), twin['pops'][1:],
                               rtol=0, atol=ptol)


def test_complex64_tracks_reference_complex64(tp, tmp_path):
    """The complex64 run is as close to the original's own complex64 run as
    both are to complex128."""
    for name in ['imag_plain_32_c64', 'real_raman_32_c64']:
        case = CASES[name]
        p = case_params(case)
        prop = tp.TensorPropagator(spin_from_case(case, tmp_path), p['dt'],
                                   p['n_steps'], 'cuda', time=p['time'],
                                   dtype=64)
        prop.full_steps(p['n_steps'])
        got = np.array([t.cpu().numpy() for t in prop.psik])
        assert rel_l2(got, case['psik_final']) <= 1e-5


def _oracle_run(inputs, dt, time, n_steps, dtype=128):
    orc = OraclePropagator(inputs, dt, time, dtype)
    pops = orc.run(n_steps)
    return orc.psik_numpy(), pops


def _inputs_from_spin(ps):
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


@pytest.mark.parametrize('dtype', [128, 64])
def test_ground_state_256_against_oracle(tp, tmp_path, dtype):
    """256^2 plain ground state (complex128 in its problem statement)."""
    from spinor_gpe import workloads
    from spinor_gpe.pspinor import pspinor as spin
    from spinor_gpe.pspinor import tensor_tools as ttools
    ps = workloads.ground_state_256(spin.PSpinor, ttools.fft_2d,
                                    str(tmp_path / 'c1') + '/')
    n = 20
    ref_psik, ref_pops = _oracle_run(_inputs_from_spin(ps), 0.02, 'imag', n)
    prop = tp.TensorPropagator(ps, 0.02, n, 'cuda', time='imag', dtype=dtype)
    pops = torch.empty((n, 2), dtype=torch.float64, device='cuda')
    prop.full_steps(n, pops)
    got = np.array([t.cpu().numpy() for t in prop.psik])
    assert rel_l2(got, ref_psik) <= TOL[dtype]
    np.testing.assert_allclose(pops.cpu().numpy(), ref_pops, rtol=0,
                               atol=1e-12 if dtype == 128 else 1e-6)


def test_raman_quench_1024_complex64_against_oracle(tp, tmp_path):
    """1024^2 complex64 real-time Raman-coupled steps against complex128."""
    from spinor_gpe import workloads
    from spinor_gpe.pspinor import pspinor as spin
    from spinor_gpe.pspinor import tensor_tools as ttools
    ps = workloads.raman_quench_1024(spin.PSpinor, ttools.fft_2d,
                                     str(tmp_path / 'c2') + '/', delta=0.5)
    n = 4
    ref_psik, ref_pops = _oracle_run(_inputs_from_spin(ps), 1e-3, 'real', n)
    prop = tp.TensorPropagator(ps, 1e-3, n, 'cuda', time='real', dtype=64)
    pops = torch.empty((n, 2), dtype=torch.float64, device='cuda')
    prop.full_steps(n, pops)
    got = np.array([t.cpu().numpy() for t in prop.psik])
    assert rel_l2(got, ref_psik) <= 1e-5
    np.testing.assert_allclose(pops.cpu().numpy(), ref_pops, rtol=0,
                               atol=1e-6)


@pytest.mark.parametrize('shape', [(32, 32), (64, 128), (256, 32),
                                   (512, 512), (128, 2048), (4096, 64)])
@pytest.mark.parametrize('dtype', [torch.complex64, torch.complex128])
def test_fft_2d_matches_numpy(shape, dtype):
    from spinor_gpe.pspinor import tensor_tools as ttools
    rng = np.random.default_rng(7)
    a = [rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
         for _ in range(2)]
    dr = (0.125, 0.25)
    ref_k = ttools.fft_2d(a, dr)           # NumPy on the host
    ref_r = ttools.ifft_2d(a, dr)
    t = [torch.as_tensor(x, dtype=dtype, device='cuda') for x in a]
    got_k = [x.cpu().numpy() for x in ttools.fft_2d(t, dr)]
    got_r = [x.cpu().numpy() for x in ttools.ifft_2d(t, dr)]
    tol = 1e-14 if dtype == torch.complex128 else 2e-6
    assert rel_l2(got_k, ref_k) <= tol
    assert rel_l2(got_r, ref_r) <= tol


@pytest.mark.parametrize('n', [128, 256, 512, 1024])
def test_fft_invariants_on_gpu(n):
    """The original's FFT test invariants on all-ones grids
    (spinor_gpe/tests/fft_func_tests.py: round trip, atom number, Parseval;
    10 eps)."""
    from spinor_gpe.pspinor import tensor_tools as ttools
    eps = torch.finfo(torch.complex128).eps * 10
    for shape in [(n, n), (n, 128), (128, n)]:
        grid = [torch.ones(shape, dtype=torch.complex128, device='cuda')] * 2
        grid_k = ttools.fft_2d(grid, (1, 1))
        grid_r = ttools.ifft_2d(grid_k, (1, 1))
        for g, r in zip(grid, grid_r):
            assert float(torch.max(torch.abs(r - g))) <= eps
        npts = shape[0] * shape[1]
        atoms = ttools.calc_atoms(grid)
        assert abs(atoms - ttools.calc_atoms(grid_r)) <= eps * npts
        vol = 4 * np.pi**2 / npts
        assert abs(atoms - ttools.calc_atoms(grid_k, vol)) <= eps * npts


def test_prop_loop_api(tmp_path):
    """imaginary() then real() through PSpinor, with sampling: the
    PropResult contract (prop_result.py:50-82) and the sampled npz format
    (tensor_propagator.py:198-204)."""
    from spinor_gpe import workloads
    from spinor_gpe.pspinor import pspinor as spin
    from spinor_gpe.pspinor import tensor_tools as ttools
    ps = workloads.build(spin.PSpinor, ttools.fft_2d, str(tmp_path / 'loop') + '/',
                         nx=64, ny=64, half_x=8.0, half_y=8.0,
                         g=(300.0, 298.0, 296.0), omega=0.7, k_l=3.0,
                         rot_coupling=False, seed=5)
    inp = _inputs_from_spin(ps)
    res, prop = ps.imaginary(0.01, 10, 'cuda', is_sampling=True, n_samples=5)
    ref_psik, ref_pops = _oracle_run(inp, 0.01, 'imag', 10)
    assert rel_l2(res.psik, ref_psik) <= 1e-10
    np.testing.assert_allclose(res.pops['vals'], ref_pops, rtol=0, atol=1e-12)
    assert res.pops['times'].shape == (10,)
    assert np.allclose(res.pops['vals'].sum(axis=1), 1.0)
    assert len(res.eng_final) == 4 and np.isfinite(res.eng_final).all()
    assert res.psi[0].shape == (64, 64) and len(res.dens) == 2
    np.testing.assert_allclose(ps.psik[0], res.psik[0])
    data = np.load(res.sampled_path)
    assert data['psiks'].shape == (5, 2, 64, 64)
    assert data['times'].shape == (5,)
    # chained real-time run after a detuning change (examples/3_raman_rabi.py)
    ps.detuning_uniform(0.3)
    inp2 = _inputs_from_spin(ps)
    res2, _ = ps.real(1e-3, 6, 'cuda')
    ref2, _ = _oracle_run(inp2, 1e-3, 'real', 6)
    assert rel_l2(res2.psik, ref2) <= 1e-10


def test_psik_setter_and_cpu_rejection(tp, tmp_path):
    case = CASES['imag_plain_32']
    spin = spin_from_case(case, tmp_path)
    with pytest.raises(ValueError):
        tp.TensorPropagator(spin, 0.02, 1, 'cpu')
    prop = tp.TensorPropagator(spin, 0.02, 1, 'cuda')
    before = [t.clone() for t in prop.psik]
    np.testing.assert_array_equal(before[0].cpu().numpy(), case['psik0'][0])
    prop.full_step()
    prop.psik = before
    prop.full_step()
    got = np.array([t.cpu().numpy() for t in prop.psik])
    assert rel_l2(got, case['psik_step1']) <= 1e-10
    with pytest.raises(ValueError):
        prop.single_step(prop.dt_in, prop.eng_out)


@pytest.mark.parametrize('shape', [(2048, 2048), (32, 4096), (4096, 32)])
def test_large_and_extreme_shapes_conserve_norm(tp, tmp_path, shape):
    """Real-time steps at the size limits: atom number before renormalisation
    stays 1 to complex64 rounding, and the state stays finite."""
    from spinor_gpe import workloads
    from spinor_gpe.pspinor import pspinor as spin
    from spinor_gpe.pspinor import tensor_tools as ttools
    ny, nx = shape
    ps = workloads.build(spin.PSpinor, ttools.fft_2d, str(tmp_path / 'x') + '/',
                         nx=nx, ny=ny, half_x=nx * 0.0625 / 2,
                         half_y=ny * 0.0625 / 2, g=(100.0, 100.0, 99.0),
                         omega=1.0, k_l=3.0, delta=0.2, seed=3)
    prop = tp.TensorPropagator(ps, 1e-3, 3, 'cuda', time='real', dtype=64)
    pops = torch.empty((3, 2), dtype=torch.float64, device='cuda')
    prop.full_steps(3, pops)
    psik = prop.psik
    assert all(torch.isfinite(p).all() for p in psik)
    np.testing.assert_allclose(pops.cpu().numpy().sum(axis=1), 1.0,
                               atol=1e-9)
    assert abs(sum(calc_pops(psik, float(ps.space['dv_k']))) - 1.0) < 1e-5


@pytest.mark.parametrize('dtype', [64, 128])
def test_graph_replay_matches_eager_steps(tp, tmp_path, dtype, monkeypatch):
    """Steady-state steps replayed from the plan's CUDA graphs give exactly
    the state that eager launches of the same kernels give, and both match
    the oracle."""
    case = CASES['imag_raman_64']
    p = case_params(case)
    spin = spin_from_case(case, tmp_path)
    a = tp.TensorPropagator(spin, p['dt'], 20, 'cuda', time=p['time'],
                            dtype=dtype)
    monkeypatch.setenv('SGPE_DISABLE_GRAPHS', '1')
    b = tp.TensorPropagator(spin, p['dt'], 20, 'cuda', time=p['time'],
                            dtype=dtype)
    monkeypatch.delenv('SGPE_DISABLE_GRAPHS')
    a.full_steps(20)                 # eager first step, then graphs (8, 8, 1, 1, 1)
    b.full_steps(20)                 # eager throughout
    for _ in range(3):
        a.full_step()                # 1-step graph
        b.full_step()
    ga = np.array([t.cpu().numpy() for t in a.psik])
    gb = np.array([t.cpu().numpy() for t in b.psik])
    np.testing.assert_array_equal(ga, gb)
    ref, _ = _oracle_run(inputs_from_arrays_case(case), p['dt'], p['time'], 23)
    assert rel_l2(ga, ref) <= TOL[dtype]


def inputs_from_arrays_case(case):
    from oracle import inputs_from_arrays
    return inputs_from_arrays(case)


@pytest.mark.parametrize('name', ['imag_raman_64x32', 'imag_raman_64',
                                  'real_raman_32', 'real_rot_32x64',
                                  'imag_gradients_32', 'real_bump_32'])
def test_complex64_error_not_worse_than_reference_complex64(tp, tmp_path, name):
    """Over 40 steps, the complex64 drop-in stays as close to the complex128
    reference as the original's own complex64 arithmetic does (up to 1.5x,
    or 1e-5, whichever is larger)."""
    case = CASES[name]
    p = case_params(case)
    n = 40
    from oracle import inputs_from_arrays
    ref128, _ = _oracle_run(inputs_from_arrays(case), p['dt'], p['time'], n, 128)
    ref64, _ = _oracle_run(inputs_from_arrays(case), p['dt'], p['time'], n, 64)
    bar = max(1e-5, 1.5 * rel_l2(ref64, ref128))
    prop = tp.TensorPropagator(spin_from_case(case, tmp_path), p['dt'], n,
                               'cuda', time=p['time'], dtype=64)
    prop.full_steps(n)
    got = np.array([t.cpu().numpy() for t in prop.psik])
    assert rel_l2(got, ref128) <= bar


@pytest.mark.parametrize('name', ['imag_plain_32', 'imag_raman_64x32',
                                  'real_raman_32', 'imag_gradients_32',
                                  'real_bump_32', 'real_rot_32x64'])
@pytest.mark.parametrize('dtype', [128, 64])
def test_device_energy_matches_oracle(tp, tmp_path, name, dtype):
    """FP64 energy functional on the device vs the oracle's NumPy FP64
    evaluation of the same functional on the same state."""
    from oracle.energy import energy_functional
    case = CASES[name]
    p = case_params(case)
    prop = tp.TensorPropagator(spin_from_case(case, tmp_path), p['dt'],
                               p['n_steps'], 'cuda', time=p['time'],
                               dtype=dtype)
    prop.full_steps(3)
    psik = [t.cpu().numpy().astype(np.complex128) for t in prop.psik]
    sc = case['scalars']
    theta = 0.0 if bool(sc[2]) else 2 * sc[1] * case['x_mesh']
    ref = energy_functional(psik, case['kin_eng_spin'], case['pot_eng_spin'],
                            case['coupling'], theta, case['g'], case['dr'],
                            case['dv'][0], case['dv'][1])
    got = prop.energy()
    vals = np.array([got[k] for k in prop.ENERGY_KEYS])
    tol = 1e-11 if dtype == 128 else 2e-6
    scale = np.maximum(np.abs(ref), abs(ref[4]))
    assert np.all(np.abs(vals - ref) <= tol * scale), (vals, ref)


def test_eng_expect_matches_reference_convention(tp, tmp_path):
    """The drop-in eng_expect reproduces the original's potential and
    interaction terms exactly on the golden ground state, and its total to
    the finite-difference truncation of the original's kinetic term."""
    e = CASES['energy']
    case = CASES['imag_plain_32']
    spin = spin_from_case(case, tmp_path)
    prop = tp.TensorPropagator(spin, 0.02, 1, 'cuda', time='imag', dtype=128)
    got = prop.eng_expect([torch.as_tensor(p, device='cuda') for p in e['psik']])
    ref = e['eng_expect']
    np.testing.assert_allclose(got[2:], ref[2:], rtol=1e-11)
    assert abs(got[1] - ref[1]) / ref[1] < 0.03
    assert abs(got[0] - ref[0]) / ref[0] < 1e-3


@pytest.mark.parametrize('shape', [(192, 192), (384, 192), (192, 768), (768, 768)])
@pytest.mark.parametrize('dtype', [torch.complex64, torch.complex128])
def test_fft_2d_radix3_sizes_match_numpy(shape, dtype):
    """Grid sides 3 * 2^k (radix-3 stage) against NumPy."""
    from spinor_gpe.pspinor import tensor_tools as ttools
    rng = np.random.default_rng(8)
    a = [rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
         for _ in range(2)]
    dr = (0.125, 0.125)
    t = [torch.as_tensor(x, dtype=dtype, device='cuda') for x in a]
    tol = 1e-14 if dtype == torch.complex128 else 2e-6
    assert rel_l2([x.cpu().numpy() for x in ttools.fft_2d(t, dr)],
                  ttools.fft_2d(a, dr)) <= tol
    assert rel_l2([x.cpu().numpy() for x in ttools.ifft_2d(t, dr)],
                  ttools.ifft_2d(a, dr)) <= tol


@pytest.mark.parametrize('n,dtype', [(192, 128), (384, 64), (768, 64)])
def test_radix3_grid_propagation_against_oracle(tp, tmp_path, n, dtype):
    from spinor_gpe import workloads
    from spinor_gpe.pspinor import pspinor as spin
    from spinor_gpe.pspinor import tensor_tools as ttools
    ps = workloads.build(spin.PSpinor, ttools.fft_2d, str(tmp_path / 'r3') + '/',
                         nx=n, ny=n, half_x=n * 0.0625, half_y=n * 0.0625,
                         g=(400.0, 398.0, 396.0), lam=1.2, omega=0.8, k_l=3.0,
                         delta=0.1, seed=21)
    steps = 6
    ref, ref_pops = _oracle_run(_inputs_from_spin(ps), 0.02, 'imag', steps)
    prop = tp.TensorPropagator(ps, 0.02, steps, 'cuda', time='imag', dtype=dtype)
    pops = torch.empty((steps, 2), dtype=torch.float64, device='cuda')
    prop.full_steps(steps, pops)
    got = np.array([t.cpu().numpy() for t in prop.psik])
    assert rel_l2(got, ref) <= TOL[dtype]


def test_batch_matches_solves_alone(tp, tmp_path):
    """A batch of uneven solves (sizes, parameters, precision, time) advanced
    together gives exactly what each gives when stepped alone."""
    from spinor_gpe import workloads
    from spinor_gpe.batch import PropagatorBatch
    from spinor_gpe.pspinor import pspinor as spin
    from spinor_gpe.pspinor import tensor_tools as ttools
    spins = workloads.batched_uneven(spin.PSpinor, ttools.fft_2d,
                                     str(tmp_path) + '/b/', n_solves=5,
                                     sizes=(64, 128, 192))
    kinds = [('imag', 64), ('imag', 128), ('real', 64), ('imag', 64), ('real', 128)]

    def make():
        return [tp.TensorPropagator(s, 0.02 if t == 'imag' else 1e-3, 20, 'cuda',
                                    time=t, dtype=d)
                for s, (t, d) in zip(spins, kinds)]
    alone, together = make(), make()
    for p in alone:
        p.full_steps(19)
    batch = PropagatorBatch(together)
    batch.full_steps(19)            # eager first step, then 8-, 8-, 1-, 1-step graphs

    def same():
        for a, b in zip(alone, together):
            np.testing.assert_array_equal(
                np.array([t.cpu().numpy() for t in a.psik]),
                np.array([t.cpu().numpy() for t in b.psik]))
    same()
    # new physics for one solve: the batch re-captures its graphs
    for p in (alone[1], together[1]):
        g = p.g_sc
        p._plan.set_physics(1.1 * g['uu'], 1.1 * g['dd'], 1.1 * g['ud'],
                            float(p.atom_num), float(p._space_np['dv_r']),
                            float(p._space_np['dv_k']), p.is_coupling)
    for p in alone:
        p.full_steps(9)
    batch.full_steps(9)
    same()
    batch.close()


@pytest.mark.parametrize('grouping', ['1', '0'])
def test_grouped_batch_matches_solves_alone(tp, tmp_path, monkeypatch, grouping):
    """Solves of one size and precision run as grouped launches (one kernel
    per pass for all of them); with grouping on or off every solve equals
    the same solve stepped alone, bit for bit."""
    from spinor_gpe import workloads
    from spinor_gpe.batch import PropagatorBatch
    from spinor_gpe.pspinor import pspinor as spin
    from spinor_gpe.pspinor import tensor_tools as ttools
    monkeypatch.setenv('SGPE_BATCH_GROUPING', grouping)
    spins = workloads.batched_uneven(spin.PSpinor, ttools.fft_2d,
                                     str(tmp_path) + '/g/', n_solves=6,
                                     sizes=(128,), seed=11)
    spins += workloads.batched_uneven(spin.PSpinor, ttools.fft_2d,
                                      str(tmp_path) + '/h/', n_solves=1,
                                      sizes=(256,), seed=12)
    kinds = [('imag', 64)] * 4 + [('real', 64)] * 2 + [('imag', 64)]

    def make():
        return [tp.TensorPropagator(s, 0.02 if t == 'imag' else 1e-3, 20, 'cuda',
                                    time=t, dtype=d)
                for s, (t, d) in zip(spins, kinds)]
    alone, together = make(), make()
    for p in alone:
        p.full_steps(21)
    batch = PropagatorBatch(together)
    batch.full_steps(21)
    for a, b in zip(alone, together):
        np.testing.assert_array_equal(np.array([t.cpu().numpy() for t in a.psik]),
                                      np.array([t.cpu().numpy() for t in b.psik]))
    batch.close()


@pytest.mark.parametrize('shape', [(64, 256), (1024, 1024), (2048, 256)])
def test_tensor_core_dft_fft_accuracy(shape):
    """The split-BF16 tensor-core DFT16 transforms agree with NumPy to the
    accuracy of the BF16 head/tail split (about 2^-16 per radix-16 stage),
    and more loosely than the FP32 path."""
    from spinor_gpe.pspinor import _native
    rng = np.random.default_rng(3)
    ny, nx = shape
    a = [rng.standard_normal(shape) + 1j * rng.standard_normal(shape) for _ in range(2)]
    t = [torch.as_tensor(x, dtype=torch.complex64, device='cuda') for x in a]
    ref = [np.fft.fft2(x) for x in a]
    errs = {}
    for mode in (0, 1):
        plan = _native.Plan(ny, nx, 64, 0)
        plan.set_dft_mode(mode)
        out = [torch.empty_like(x) for x in t]
        plan.fft2(torch, t, out, 0, 1.0)
        got = [np.fft.ifftshift(o.cpu().numpy()) for o in out]   # fft2 output is centred
        errs[mode] = rel_l2(got, ref)
    assert errs[0] <= 2e-6
    assert 1e-7 < errs[1] <= 2e-4


def test_tensor_core_dft_propagation_against_oracle(tp, tmp_path):
    """A 256^2 complex64 imaginary-time run with tensor-core DFT16 stages
    tracks the complex128 oracle within the BF16-split accuracy."""
    from spinor_gpe import workloads
    from spinor_gpe.pspinor import pspinor as spin
    from spinor_gpe.pspinor import tensor_tools as ttools
    ps = workloads.ground_state_256(spin.PSpinor, ttools.fft_2d, str(tmp_path / 'tc') + '/')
    steps = 20
    ref, _ = _oracle_run(_inputs_from_spin(ps), 0.02, 'imag', steps)
    res = {}
    for tc in (False, True):
        prop = tp.TensorPropagator(ps, 0.02, steps, 'cuda', time='imag', dtype=64,
                                   tensor_core_dft=tc)
        prop.full_steps(steps)
        res[tc] = rel_l2(np.array([x.cpu().numpy() for x in prop.psik]), ref)
    assert res[False] <= 1e-5
    assert res[True] <= 2e-3
    with pytest.raises(_native_error()):
        tp.TensorPropagator(ps, 0.02, steps, 'cuda', time='imag', dtype=128,
                            tensor_core_dft=True)


def _native_error():
    from spinor_gpe.pspinor import _native
    return _native.SgpeError


@pytest.mark.parametrize('dtype', [64, 128])
def test_device_analysis_matches_numpy(tp, tmp_path, dtype):
    """Densities, masked phases and the separation measure of PropResult
    computed on the device agree with the NumPy formulas of the original."""
    from spinor_gpe import workloads
    from spinor_gpe.pspinor import pspinor as spin
    from spinor_gpe.pspinor import prop_result
    from spinor_gpe.pspinor import tensor_tools as ttools
    ps = workloads.build(spin.PSpinor, ttools.fft_2d, str(tmp_path / 'an') + '/',
                         nx=128, ny=64, half_x=8.0, half_y=4.0, g=(500.0, 490.0, 480.0),
                         omega=0.9, k_l=2.0, delta=0.2, seed=31)
    prop = tp.TensorPropagator(ps, 0.02, 10, 'cuda', time='imag', dtype=dtype)
    prop.full_steps(10)
    d = prop.analysis()
    psik = ttools.to_numpy(prop.psik)
    psi = ttools.to_numpy(ttools.ifft_2d(prop.psik, ps.space['dr']))
    ref = prop_result.PropResult(psi, psik, 0.0, {})
    tol = 1e-6 if dtype == 64 else 1e-13
    for c in range(2):
        assert rel_l2(d['dens'][c].cpu().numpy(), ref.dens[c]) <= tol
        assert rel_l2(d['densk'][c].cpu().numpy(), ref.densk[c]) <= tol
        got_ph = d['phase'][c].cpu().numpy()
        # equal away from the mask edge and the +-pi branch cut
        ok = np.isclose(got_ph, ref.phase[c], rtol=0, atol=1e-5) | \
            np.isclose(np.abs(got_ph - ref.phase[c]), 2 * np.pi, atol=1e-5)
        assert ok.mean() > 0.999
    assert abs(d['separation'] - ref.calc_separation()) <= 1e-6
    res = prop.prop_loop(5)
    assert abs(res.calc_separation() - prop.analysis()['separation']) <= 1e-12


def test_stream_handle_follows_the_current_stream(tp):
    """The stream handle given to every C call is the caller's current
    stream (default, or one selected with ``torch.cuda.stream``), for a
    device given as torch.device, string or index."""
    import ctypes
    from spinor_gpe.pspinor import _native

    def handle(d):
        h = _native._stream(torch, d)
        return h.value if isinstance(h, ctypes.c_void_p) else h

    dev = torch.device('cuda', torch.cuda.current_device())
    torch.empty(1, device=dev)
    assert handle(dev) == torch.cuda.current_stream(dev).cuda_stream
    side = torch.cuda.Stream(dev)
    with torch.cuda.stream(side):
        for d in (dev, 'cuda', f'cuda:{dev.index}', dev.index):
            assert handle(d) == side.cuda_stream
    assert handle(dev) == torch.cuda.current_stream(dev).cuda_stream


@pytest.mark.parametrize('shape', [(4096, 4096), (2048, 4096)])
@pytest.mark.parametrize('dtype', [64, 128, 'double-float'])
def test_largest_grids_match_oracle(tp, tmp_path, shape, dtype):
    """Real-time Raman-dressed steps at the largest supported grids against
    the complex128 oracle (run on the same GPU): 1e-5 for complex64, 1e-10
    for complex128 and double-float."""
    from spinor_gpe import workloads
    from spinor_gpe.pspinor import pspinor as spin
    from spinor_gpe.pspinor import tensor_tools as ttools
    ny, nx = shape
    ps = workloads.build(spin.PSpinor, ttools.fft_2d, str(tmp_path / 'x') + '/',
                         nx=nx, ny=ny, half_x=nx * 0.0625 / 2,
                         half_y=ny * 0.0625 / 2, g=(1000.0, 995.0, 990.0),
                         omega=1.0, k_l=3.0, delta=0.3, seed=6)
    n = 3
    orc = OraclePropagator(_inputs_from_spin(ps), 1e-3, 'real', 128, device='cuda')
    for _ in range(n):
        orc.full_step()
    ref = orc.psik_numpy()
    del orc
    prop = tp.TensorPropagator(ps, 1e-3, n, 'cuda', time='real', dtype=dtype)
    prop.full_steps(n)
    got = np.array([t.cpu().numpy() for t in prop.psik]).astype(np.complex128)
    assert rel_l2(got, ref) <= (1e-5 if dtype == 64 else 1e-10)


@pytest.mark.parametrize('dtype', [64, 128, 'double-float'])
def test_zero_and_negative_step_counts(tp, tmp_path, dtype):
    """Zero steps (with or without an empty populations buffer) leave the
    state bit-for-bit as it was; a negative count is an argument error."""
    case = CASES['imag_raman_64']
    p = case_params(case)
    prop = tp.TensorPropagator(spin_from_case(case, tmp_path), p['dt'], 1, 'cuda',
                               time=p['time'], dtype=dtype)
    prop.full_steps(2)
    before = np.array([t.cpu().numpy() for t in prop.psik])
    prop.full_steps(0)
    prop.full_steps(0, torch.empty((0, 2), dtype=torch.float64, device='cuda'))
    after = np.array([t.cpu().numpy() for t in prop.psik])
    np.testing.assert_array_equal(before, after)
    with pytest.raises(_native_error()):
        prop.full_steps(-1)
    prop.full_steps(1)
    assert rel_l2(np.array([t.cpu().numpy() for t in prop.psik]), before) > 0
