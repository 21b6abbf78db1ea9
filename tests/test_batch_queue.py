"""The batch work queue: ``PropagatorBatch(..., queue=True)`` (C ABI
``sgpe_batch_set_queue``) steps many complex64 solves of different sizes in
one persistent launch whose blocks claim pass items from a device counter.

Checked against the complex128 oracle at the complex64 tolerance (1e-5) and
against the same solves stepped alone (its item shapes differ from the
single-solve kernels', so to complex64 rounding, not bit for bit); its
results do not depend on which block claims which item (bit-identical from
run to run); the error word stays clear; plans it cannot run are refused;
its bounded wait gives up instead of hanging.
"""
import numpy as np
import pytest
import torch

from conftest import rel_l2
from oracle import OracleInputs, OraclePropagator

pytestmark = pytest.mark.gpu

# (ny, nx, time, dt, seed): every size class of the queue, one grid that is
# not square, imaginary and real time
PROBLEMS = [(128, 128, 'imag', 0.02, 1), (192, 192, 'real', 1e-3, 2),
            (256, 512, 'imag', 0.02, 3), (384, 384, 'real', 1e-3, 4),
            (512, 512, 'imag', 0.02, 5), (768, 768, 'real', 1e-3, 6),
            (1024, 1024, 'imag', 0.02, 7), (128, 128, 'real', 1e-3, 8)]
STEPS = 17      # two 8-step launches and one 1-step launch


def _spin(tmp_path, ny, nx, seed):
    from spinor_gpe import workloads
    from spinor_gpe.pspinor import pspinor as spin
    from spinor_gpe.pspinor import tensor_tools as ttools
    return workloads.build(spin.PSpinor, ttools.fft_2d, str(tmp_path / f'q{seed}') + '/',
                           nx=nx, ny=ny, half_x=nx * 0.0625, half_y=ny * 0.0625,
                           g=(800.0 + 50 * seed, 795.0, 790.0), omega=0.8, k_l=3.0,
                           delta=0.1 * seed, lam=1.1, rot_coupling=False, seed=seed)


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


@pytest.fixture(scope='module')
def problems(tmp_path_factory):
    assert torch.cuda.is_available(), 'these tests need a CUDA device'
    tmp = tmp_path_factory.mktemp('queue')
    return [(_spin(tmp, ny, nx, seed), t, dt) for ny, nx, t, dt, seed in PROBLEMS]


def _props(problems, dtype=64):
    from spinor_gpe.pspinor import tensor_propagator as tprop
    return [tprop.TensorPropagator(ps, dt, STEPS, 'cuda', time=t, dtype=dtype)
            for ps, t, dt in problems]


def test_queue_matches_oracle_and_solves_alone(problems):
    from spinor_gpe.batch import PropagatorBatch
    props = _props(problems)
    batch = PropagatorBatch(props, queue=True)
    batch.full_steps(STEPS)
    batch.check_device()
    got = [_state(p) for p in props]
    batch.close()
    alone = _props(problems)
    for (ps, t, dt), prop, g in zip(problems, alone, got):
        prop.full_steps(STEPS)
        # other radix plans (768: 12 points per thread against 24) and
        # column tiles round differently: complex64 agreement, not bits
        assert rel_l2(g, _state(prop)) <= 1e-5
        orc = OraclePropagator(_inputs(ps), dt, t, 128, device='cuda')
        for _ in range(STEPS):
            orc.full_step()
        assert rel_l2(g.astype(np.complex128), orc.psik_numpy()) <= 1e-5


def test_queue_results_do_not_depend_on_the_claim_order(problems):
    """Blocks claim items dynamically; each item's arithmetic is fixed, so
    two runs give the same bits, and splitting the steps differently
    (8 + 1 launches against one 9-step call) does too."""
    from spinor_gpe.batch import PropagatorBatch
    runs = []
    for split in ([9], [4, 5]):
        props = _props(problems)
        batch = PropagatorBatch(props, queue=True)
        for n in split:
            batch.full_steps(n)
        batch.check_device()
        runs.append([_state(p) for p in props])
        batch.close()
    for a, b in zip(*runs):
        np.testing.assert_array_equal(a, b)


def test_queue_mode_can_be_switched_off_and_on(problems):
    """A batch leaves the queue for grouped launches and comes back (its
    graphs are re-captured each time); the states follow the oracle."""
    from spinor_gpe.batch import PropagatorBatch
    sub = problems[:3]
    props = _props(sub)
    batch = PropagatorBatch(props, queue=True)
    batch.full_steps(3)
    batch._batch.set_queue(False)
    batch.full_steps(9)
    batch._batch.set_queue(True)
    batch.full_steps(2)
    batch.check_device()
    got = [_state(p) for p in props]
    batch.close()
    for (ps, t, dt), g in zip(sub, got):
        orc = OraclePropagator(_inputs(ps), dt, t, 128, device='cuda')
        for _ in range(14):
            orc.full_step()
        assert rel_l2(g.astype(np.complex128), orc.psik_numpy()) <= 1e-5


def test_queue_refuses_plans_it_cannot_run(problems):
    from spinor_gpe.batch import PropagatorBatch
    from spinor_gpe.pspinor import _native
    ps, t, dt = problems[0]
    from spinor_gpe.pspinor import tensor_propagator as tprop
    c128 = tprop.TensorPropagator(ps, dt, 4, 'cuda', time=t, dtype=128)
    with pytest.raises(_native.SgpeError):
        PropagatorBatch([c128], queue=True)


def test_queue_wait_is_bounded():
    """One block waits for a counter that nothing increments: the wait ends
    by its limit (about 1 s) and says so."""
    import ctypes
    from spinor_gpe.pspinor import _native
    lib = _native.load()
    gave_up = ctypes.c_int(-1)
    ms = ctypes.c_double(0.0)
    _native.check(lib.sgpe_check_queue_wait(ctypes.byref(gave_up), ctypes.byref(ms)))
    assert gave_up.value == 1
    assert 900.0 <= ms.value <= 5000.0
