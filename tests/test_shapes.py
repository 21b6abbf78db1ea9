"""Kernel shapes and the autotuner.

Every pass can run in several kernel shapes (points per thread and radix
plan; ``sgpe_shape_count``).  Each shape must meet the parity tolerances
against the oracle on its own (1e-10 relative L2 for complex128, 1e-5 for
complex64, against the complex128 reference); switching shapes keeps the
state; the autotuner leaves the state bit-identical and remembers its
choice; batches stay bit-identical to solves alone in any shapes.
"""
import ctypes
import itertools
import json

import numpy as np
import pytest

from conftest import case_params, load_cases, rel_l2, spin_from_case
from spinor_gpe import tuning
from spinor_gpe.pspinor import _native

TOL = {128: 1e-10, 64: 1e-5}
CASES = load_cases()


def _pairs(bits, ny, nx):
    lib = _native.load()
    nr = lib.sgpe_shape_count(bits, 0, nx)
    nc = lib.sgpe_shape_count(bits, 1, ny)
    return list(itertools.product(range(nr), range(nc)))


# ------------------------------------------------------------------ CPU only
def test_shape_counts(native_lib):
    lib = _native.load()
    assert lib.sgpe_shape_count(64, 0, 512) == 3
    assert lib.sgpe_shape_count(64, 1, 32) == 3
    assert lib.sgpe_shape_count(64, 0, 1024) == 2
    assert lib.sgpe_shape_count(64, 1, 1024) == 1
    assert lib.sgpe_shape_count(48, 0, 1024) == 1          # double-float: shape 0
    assert lib.sgpe_shape_count(48, 1, 192) == 1
    assert lib.sgpe_shape_count(64, 0, 2048) == 1
    assert lib.sgpe_shape_count(64, 0, 768) == 2
    assert lib.sgpe_shape_count(64, 1, 192) == 2
    assert lib.sgpe_shape_count(128, 0, 768) == 1
    assert lib.sgpe_shape_count(128, 0, 256) == 3
    assert lib.sgpe_shape_count(128, 1, 2048) == 1
    assert lib.sgpe_shape_count(64, 0, 48) == 0
    assert lib.sgpe_shape_count(32, 0, 256) == 0
    assert lib.sgpe_shape_count(64, 2, 256) == 0
    assert lib.sgpe_set_shapes(None, 0, 0) == _native.SGPE_ERR_ARG
    r, c = ctypes.c_int(), ctypes.c_int()
    assert lib.sgpe_get_shapes(None, ctypes.byref(r), ctypes.byref(c)) == _native.SGPE_ERR_ARG
    assert lib.sgpe_autotune(None, 8, ctypes.byref(r), ctypes.byref(c), None, None) == _native.SGPE_ERR_ARG


def test_wisdom_round_trip(tmp_path):
    tuning.forget()
    tuning.remember(64, 512, 256, (1, 2))
    tuning.remember(128, 256, 256, (1, 0))
    path = tmp_path / 'wisdom.json'
    tuning.save(path)
    data = json.loads(path.read_text())
    assert len(data['kernel_shapes']) == 2
    tuning.forget()
    assert tuning.lookup(64, 512, 256) is None
    tuning.load(path)
    assert tuning.lookup(64, 512, 256) == (1, 2)
    assert tuning.lookup(128, 256, 256) == (1, 0)
    tuning.forget()
    assert tuning.default_steps(1024, 1024) == 19
    assert tuning.default_steps(32, 32) == 256
    assert tuning.default_steps(4096, 4096) == 16


# ------------------------------------------------------------------ GPU
@pytest.fixture(scope='module')
def tp():
    import torch
    assert torch.cuda.is_available(), 'these tests need a CUDA device'
    from spinor_gpe.pspinor import tensor_propagator
    tuning.forget()
    yield tensor_propagator
    tuning.forget()


def _psik(prop):
    return np.array([t.cpu().numpy() for t in prop.psik])


def _c128_twin(name):
    return CASES[name[:-4]] if name.endswith('_c64') else CASES[name]


@pytest.mark.gpu
@pytest.mark.parametrize('name', ['imag_raman_64x32', 'real_rot_32x64', 'real_raman_32_c64',
                                  'imag_plain_32_c64', 'imag_gradients_32', 'real_bump_32',
                                  'imag_raman_64'])
def test_every_shape_matches_reference(tp, tmp_path, name):
    case = CASES[name]
    p = case_params(case)
    ny, nx = case['x_mesh'].shape
    ref = _c128_twin(name)['psik_final']
    pairs = _pairs(p['dtype'], ny, nx)
    assert len(pairs) > 1
    for shapes in pairs:
        prop = tp.TensorPropagator(spin_from_case(case, tmp_path), p['dt'], p['n_steps'], 'cuda',
                                   time=p['time'], dtype=p['dtype'], kernel_shapes=shapes)
        assert prop.kernel_shapes == shapes
        prop.full_steps(p['n_steps'])
        assert rel_l2(_psik(prop), ref) <= TOL[p['dtype']], shapes


def _oracle(ps, dt, time, n):
    from oracle import OraclePropagator, OracleInputs
    inp = OracleInputs(
        psik=[np.asarray(x) for x in ps.psik],
        kin_eng_spin=[np.asarray(k) for k in ps.kin_eng_spin],
        pot_eng_spin=[np.asarray(v) for v in ps.pot_eng_spin],
        coupling=np.asarray(ps.coupling, dtype=np.float64),
        x_mesh=ps.space['x_mesh'], dr=ps.space['dr'],
        dv_r=float(ps.space['dv_r']), dv_k=float(ps.space['dv_k']),
        g_sc=dict(ps.g_sc), atom_num=float(ps.atom_num),
        kL_recoil=float(ps.kL_recoil), rot_coupling=bool(ps.rot_coupling),
        is_coupling=bool(ps.is_coupling))
    orc = OraclePropagator(inp, dt, time, 128)
    orc.run(n)
    return orc.psik_numpy()


@pytest.mark.gpu
@pytest.mark.parametrize('dtype', [128, 64])
def test_ground_state_256_every_shape(tp, tmp_path, dtype):
    """The 256^2 plain ground state in every pair of shapes."""
    from spinor_gpe import workloads
    from spinor_gpe.pspinor import pspinor as spin
    from spinor_gpe.pspinor import tensor_tools as ttools
    ps = workloads.ground_state_256(spin.PSpinor, ttools.fft_2d, str(tmp_path / 'c1') + '/')
    n = 10
    ref = _oracle(ps, 0.02, 'imag', n)
    for shapes in _pairs(dtype, 256, 256):
        prop = tp.TensorPropagator(ps, 0.02, n, 'cuda', time='imag', dtype=dtype, kernel_shapes=shapes)
        prop.full_steps(n)
        assert rel_l2(_psik(prop), ref) <= TOL[dtype], shapes


@pytest.mark.gpu
def test_raman_512_complex64_every_shape(tp, tmp_path):
    """Real-time Raman-coupled 512^2 complex64 steps in every pair of shapes."""
    from spinor_gpe import workloads
    from spinor_gpe.pspinor import pspinor as spin
    from spinor_gpe.pspinor import tensor_tools as ttools
    ps = workloads.raman_quench_1024(spin.PSpinor, ttools.fft_2d, str(tmp_path / 'q') + '/',
                                     n=512, delta=0.5)
    n = 3
    ref = _oracle(ps, 1e-3, 'real', n)
    for shapes in _pairs(64, 512, 512):
        prop = tp.TensorPropagator(ps, 1e-3, n, 'cuda', time='real', dtype=64, kernel_shapes=shapes)
        prop.full_steps(n)
        assert rel_l2(_psik(prop), ref) <= 1e-5, shapes


@pytest.mark.gpu
@pytest.mark.parametrize('n', [192, 384, 768])
def test_radix3_sides_every_shape(tp, tmp_path, n):
    """Sides 3 * 2^k: both radix plans (12 or 24 points per thread) against
    the oracle, complex64 real time."""
    from spinor_gpe import workloads
    from spinor_gpe.pspinor import pspinor as spin
    from spinor_gpe.pspinor import tensor_tools as ttools
    ps = workloads.raman_quench_1024(spin.PSpinor, ttools.fft_2d, str(tmp_path / 'q') + '/',
                                     n=n, delta=0.5)
    steps = 3
    ref = _oracle(ps, 1e-3, 'real', steps)
    pairs = _pairs(64, n, n)
    assert len(pairs) == 4
    for shapes in pairs:
        prop = tp.TensorPropagator(ps, 1e-3, steps, 'cuda', time='real', dtype=64, kernel_shapes=shapes)
        prop.full_steps(steps)
        assert rel_l2(_psik(prop), ref) <= 1e-5, shapes


@pytest.mark.gpu
def test_raman_1024_complex64_every_shape(tp, tmp_path):
    """1024^2 complex64: both row shapes (16 and 32 points per thread)
    against the oracle."""
    from spinor_gpe import workloads
    from spinor_gpe.pspinor import pspinor as spin
    from spinor_gpe.pspinor import tensor_tools as ttools
    ps = workloads.raman_quench_1024(spin.PSpinor, ttools.fft_2d, str(tmp_path / 'q') + '/',
                                     n=1024, delta=0.5)
    n = 3
    ref = _oracle(ps, 1e-3, 'real', n)
    pairs = _pairs(64, 1024, 1024)
    assert len(pairs) == 2
    for shapes in pairs:
        prop = tp.TensorPropagator(ps, 1e-3, n, 'cuda', time='real', dtype=64, kernel_shapes=shapes)
        prop.full_steps(n)
        assert rel_l2(_psik(prop), ref) <= 1e-5, shapes


@pytest.mark.gpu
def test_shape_switch_keeps_the_state(tp, tmp_path):
    """Switching shapes between steps continues the same solve (within the
    complex64 tolerance of the run in one shape)."""
    case = CASES['real_raman_32_c64']
    p = case_params(case)
    one = tp.TensorPropagator(spin_from_case(case, tmp_path), p['dt'], 20, 'cuda', time='real',
                              dtype=64, kernel_shapes=(0, 0))
    one.full_steps(20)
    two = tp.TensorPropagator(spin_from_case(case, tmp_path), p['dt'], 20, 'cuda', time='real',
                              dtype=64, kernel_shapes=(0, 0))
    two.full_steps(7)
    two.kernel_shapes = (2, 1)
    two.full_steps(6)
    two.kernel_shapes = (1, 2)
    two.full_steps(7)
    ref = _c128_twin('real_raman_32_c64')['psik_final']
    assert rel_l2(_psik(two), _psik(one)) <= 1e-5
    assert rel_l2(_psik(two), ref) <= 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize('time,dtype', [('imag', 128), ('real', 64)])
def test_autotune_keeps_state_and_remembers(tp, tmp_path, time, dtype):
    from spinor_gpe import workloads
    from spinor_gpe.pspinor import pspinor as spin
    from spinor_gpe.pspinor import tensor_tools as ttools
    tuning.forget()
    ps = workloads.raman_quench_1024(spin.PSpinor, ttools.fft_2d, str(tmp_path / 'a') + '/',
                                     n=256, delta=0.5)
    dt = 0.02 if time == 'imag' else 1e-3
    prop = tp.TensorPropagator(ps, dt, 10, 'cuda', time=time, dtype=dtype)
    prop.full_steps(3)
    before = _psik(prop)
    initial = prop.kernel_shapes
    times = prop.autotune(n_steps=8)
    assert np.array_equal(_psik(prop), before)
    pairs = _pairs(dtype, 256, 256)
    assert sorted(times) == sorted(pairs)
    assert all(t > 0 for t in times.values())
    chosen = prop.kernel_shapes
    assert chosen in pairs
    assert tuning.lookup(dtype, 256, 256) == chosen
    # the tuned plan continues the same solve as an untuned one
    ref = tp.TensorPropagator(ps, dt, 10, 'cuda', time=time, dtype=dtype, kernel_shapes=initial)
    ref.full_steps(3)
    assert np.array_equal(_psik(ref), before)
    prop.full_steps(5)
    ref.full_steps(5)
    assert rel_l2(_psik(prop), _psik(ref)) <= (1e-12 if dtype == 128 else 1e-5)
    # a new propagator of the same grid starts in the remembered shapes
    again = tp.TensorPropagator(ps, dt, 10, 'cuda', time=time, dtype=dtype)
    assert again.kernel_shapes == chosen
    tuning.forget()


@pytest.mark.gpu
def test_tensor_core_mode_runs_shape_zero(tp, tmp_path):
    from spinor_gpe import workloads
    from spinor_gpe.pspinor import pspinor as spin
    from spinor_gpe.pspinor import tensor_tools as ttools
    ps = workloads.raman_quench_1024(spin.PSpinor, ttools.fft_2d, str(tmp_path / 't') + '/',
                                     n=256, delta=0.5)
    prop = tp.TensorPropagator(ps, 1e-3, 10, 'cuda', time='real', dtype=64,
                               kernel_shapes=(1, 1))
    assert prop.kernel_shapes == (1, 1)
    prop._plan.set_dft_mode(1)
    assert prop.kernel_shapes == (0, 0)
    with pytest.raises(_native.SgpeError):
        prop.kernel_shapes = (1, 0)
    with pytest.raises(_native.SgpeError):
        prop.kernel_shapes = (5, 0)


@pytest.mark.gpu
def test_batch_in_other_shapes_matches_solves_alone(tp, tmp_path):
    """Grouped launches run the members' shapes; plans of one size in
    different shapes form separate groups; every solve equals itself
    stepped alone, bit for bit."""
    from spinor_gpe import workloads
    from spinor_gpe.batch import PropagatorBatch
    from spinor_gpe.pspinor import pspinor as spin
    from spinor_gpe.pspinor import tensor_tools as ttools
    spins = workloads.batched_uneven(spin.PSpinor, ttools.fft_2d, str(tmp_path) + '/g/',
                                     n_solves=6, sizes=(128,), seed=21)
    shapes = [(1, 2), (1, 2), (1, 2), (2, 0), (2, 0), (0, 1)]

    def make():
        return [tp.TensorPropagator(s, 0.02, 20, 'cuda', time='imag', dtype=64, kernel_shapes=sh)
                for s, sh in zip(spins, shapes)]
    alone, together = make(), make()
    for p in alone:
        p.full_steps(19)
    batch = PropagatorBatch(together)
    batch.full_steps(19)
    for a, b in zip(alone, together):
        np.testing.assert_array_equal(_psik(a), _psik(b))
    batch.close()


@pytest.mark.gpu
@pytest.mark.parametrize('bits,ny,nx', [(64, 256, 128), (128, 256, 128), (64, 1024, 1024)])
def test_fft_every_shape_matches_numpy(tp, bits, ny, nx):
    """The plan's centred 2-D transforms in every pair of shapes (both
    directions) against NumPy."""
    import torch
    from spinor_gpe.pspinor import tensor_tools as ttools
    rng = np.random.default_rng(3)
    a = [rng.standard_normal((ny, nx)) + 1j * rng.standard_normal((ny, nx)) for _ in range(2)]
    dr = (0.125, 0.25)
    ref_k = ttools.fft_2d(a, dr)
    ref_r = ttools.ifft_2d(a, dr)
    norm = dr[0] * dr[1] / (2 * np.pi)
    dt = torch.complex64 if bits == 64 else torch.complex128
    t = [torch.as_tensor(x, dtype=dt, device='cuda') for x in a]
    plan = _native.Plan(ny, nx, bits, torch.cuda.current_device())
    tol = 2e-6 if bits == 64 else 1e-14
    try:
        for shapes in _pairs(bits, ny, nx):
            plan.set_shapes(*shapes)
            assert plan.shapes == shapes
            out = [torch.empty_like(x) for x in t]
            plan.fft2(torch, t, out, False, norm)
            assert rel_l2([o.cpu().numpy() for o in out], ref_k) <= tol, shapes
            plan.fft2(torch, t, out, True, 1.0 / (ny * nx * norm))
            assert rel_l2([o.cpu().numpy() for o in out], ref_r) <= tol, shapes
    finally:
        plan.close()


@pytest.mark.gpu
def test_batch_autotune_keeps_states_and_matches_solves_alone(tp, tmp_path):
    """PropagatorBatch.autotune picks shapes per grid class, restores every
    state, and the tuned batch equals its solves stepped alone in the same
    shapes, bit for bit."""
    from spinor_gpe import workloads
    from spinor_gpe.batch import PropagatorBatch
    from spinor_gpe.pspinor import pspinor as spin
    from spinor_gpe.pspinor import tensor_tools as ttools
    spins = workloads.batched_uneven(spin.PSpinor, ttools.fft_2d, str(tmp_path) + '/t/',
                                     n_solves=5, sizes=(128, 192), seed=31)
    props = [tp.TensorPropagator(s, 0.02, 20, 'cuda', time='imag', dtype=64) for s in spins]
    before = [_psik(p) for p in props]
    batch = PropagatorBatch(props)
    tuned = batch.autotune(n_steps=8, warmup=9)
    assert tuned
    for p, b in zip(props, before):
        assert np.array_equal(_psik(p), b)
    for (bits, ny, nx), times in tuned.items():
        assert sorted(times) == sorted(_pairs(bits, ny, nx))
        shapes = {p.kernel_shapes for p in props if p._shape == (ny, nx)}
        assert len(shapes) == 1 and shapes.pop() in times
    batch.full_steps(13)
    alone = [tp.TensorPropagator(s, 0.02, 20, 'cuda', time='imag', dtype=64,
                                 kernel_shapes=p.kernel_shapes) for s, p in zip(spins, props)]
    for a, p in zip(alone, props):
        a.full_steps(13)
        np.testing.assert_array_equal(_psik(a), _psik(p))
    batch.close()
