"""Set-up on the device (DeviceSpinor, native set-up kernels) against the
host PSpinor set-up of the original's formulas."""
import numpy as np
import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _pair(tmp_path, dtype=128, **kw):
    from spinor_gpe.pspinor import pspinor as spin
    from spinor_gpe.pspinor.device_spinor import DeviceSpinor
    args = dict(mesh_points=(128, 64), r_sizes=(8.0, 4.0), atom_num=1e4,
                omeg={'x': 2 * np.pi * 50, 'y': 2 * np.pi * 60, 'z': 2 * np.pi * 2000},
                g_sc={'uu': 1.0, 'dd': 0.995, 'ud': 0.99})
    args.update(kw)
    host = spin.PSpinor(str(tmp_path / 'h') + '/', overwrite=True, **args)
    dev = DeviceSpinor(str(tmp_path / 'd') + '/', overwrite=True, dtype=dtype, **args)
    return host, dev


def _np(x):
    return np.array([t.cpu().numpy() if isinstance(t, torch.Tensor) else np.asarray(t) for t in x])


def test_device_spinor_set_up_matches_host(tmp_path):
    host, dev = _pair(tmp_path)
    assert rel_l2(np.asarray(dev.pot_eng), host.pot_eng) <= 1e-15
    assert rel_l2(np.asarray(dev.kin_eng), host.kin_eng) <= 1e-15
    assert rel_l2(_np(dev.psi), _np(host.psi)) <= 1e-13
    assert rel_l2(_np(dev.psik), _np(host.psik)) <= 1e-13
    np.testing.assert_allclose(dev.heal, host.heal, rtol=1e-12)
    for ps in (host, dev):
        ps.coupling_setup(kin_shift=True)
        ps.coupling_uniform(1.5)
        ps.detuning_grad(0.3, 0.1, axis=0)
    for a, b in zip(dev.kin_eng_spin, host.kin_eng_spin):
        assert np.abs(np.asarray(a) - b).max() <= 1e-12 * np.abs(b).max()
    for a, b in zip(dev.pot_eng_spin, host.pot_eng_spin):
        assert np.abs(np.asarray(a) - b).max() <= 1e-12 * np.abs(b).max()
    np.testing.assert_array_equal(np.asarray(dev.coupling), host.coupling)
    for ps in (host, dev):
        ps.seed_vortices([(1.0, -0.5), (-2.0, 1.0)], [1, -1])
    assert rel_l2(_np(dev.psi), _np(host.psi)) <= 1e-12
    for ps in (host, dev):
        ps.shift_momentum(scale=0.8, frac=(0.3, 0.7))
    assert rel_l2(_np(dev.psik), _np(host.psik)) <= 1e-12
    assert rel_l2(_np(dev.psi), _np(host.psi)) <= 1e-12


@pytest.mark.parametrize('dtype,tol', [(128, 1e-10), (64, 1e-5)])
def test_device_built_propagation_matches_host_built(tmp_path, dtype, tol):
    from spinor_gpe import workloads
    from spinor_gpe.pspinor import pspinor as spin
    from spinor_gpe.pspinor import tensor_propagator as tprop
    from spinor_gpe.pspinor import tensor_tools as ttools
    kw = dict(nx=128, ny=128, half_x=8.0, half_y=8.0, g=(600.0, 597.0, 594.0),
              lam=1.3, omega=0.8, k_l=3.0, delta=0.2, phase_noise=0.0)
    host = workloads.build(spin.PSpinor, ttools.fft_2d, str(tmp_path / 'h') + '/', **kw)
    dev = workloads.build_device(str(tmp_path / 'd') + '/', dtype=dtype, **kw)
    out = {}
    for name, ps in (('host', host), ('dev', dev)):
        p = tprop.TensorPropagator(ps, 0.02, 20, 'cuda', time='imag', dtype=dtype)
        p.full_steps(20)
        out[name] = (_np(p.psik), p.energy())
    assert rel_l2(out['dev'][0], out['host'][0]) <= tol
    assert abs(out['dev'][1]['total'] - out['host'][1]['total']) <= tol * abs(out['host'][1]['total'])


def test_device_noise_is_seeded_and_bounded(tmp_path):
    from spinor_gpe import workloads
    kw = dict(nx=64, ny=64, half_x=4.0, half_y=4.0, g=(600.0, 597.0, 594.0))
    a = workloads.build_device(str(tmp_path / 'a') + '/', seed=5, dtype=128, **kw)
    b = workloads.build_device(str(tmp_path / 'b') + '/', seed=5, dtype=128, **kw)
    c = workloads.build_device(str(tmp_path / 'c') + '/', seed=6, dtype=128, **kw)
    z = workloads.build_device(str(tmp_path / 'z') + '/', seed=5, phase_noise=0.0, dtype=128, **kw)
    pa, pc, pz = _np(a.psi), _np(c.psi), _np(z.psi)
    np.testing.assert_array_equal(pa, _np(b.psi))
    assert not np.array_equal(pa, pc)
    mask = np.abs(pz) > 0
    ph = np.angle(pa[mask] / pz[mask])
    assert np.abs(ph).max() <= 0.01 and np.abs(ph).max() > 0.005
    assert np.allclose(np.abs(pa), np.abs(pz), rtol=1e-12, atol=0)
