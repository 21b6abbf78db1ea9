"""Test configuration: the ``gpu`` marker, import paths and shared helpers.

Tests marked ``gpu`` need a CUDA device and the native library; everything
else runs on the CPU.
"""
import os
import sys
import types

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, 'spinor-gpe_gb300')
for p in (PKG, REPO):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(REPO, 'tests', 'golden')


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA GPU and the native library')


@pytest.fixture(scope='session')
def native_lib():
    """Path of libspinor_gb300.so, building it first if needed."""
    import build_native
    return build_native.build()


def load_cases():
    """Golden propagation cases: {name: {key: array}}."""
    z = np.load(os.path.join(GOLDEN, 'cases.npz'))
    out = {}
    for k in z.files:
        name, key = k.split('/', 1)
        out.setdefault(name, {})[key] = z[k]
    return out


def prop_case_names(cases):
    """Names of the propagation cases (entries with run parameters)."""
    return sorted(k for k, v in cases.items() if 'scalars' in v)


def case_params(case):
    sc = case['scalars']
    return dict(dt=float(sc[4]), n_steps=int(sc[5]), dtype=int(sc[6]),
                time='imag' if sc[7] == 1 else 'real')


def spin_from_case(case, tmpdir):
    """An object with the attributes the propagator reads from a PSpinor
    (spinor_gpe/pspinor/tensor_propagator.py:93-129)."""
    g = case['g']
    sc = case['scalars']
    space = {'dr': case['dr'], 'dk': case['dk'], 'x_mesh': case['x_mesh'],
             'y_mesh': case['y_mesh'], 'dv_r': case['dv'][0],
             'dv_k': case['dv'][1]}
    ny, nx = case['x_mesh'].shape
    dk = case['dk']
    kx = np.linspace(-np.pi / case['dr'][0], np.pi / case['dr'][0], nx,
                     endpoint=False)
    ky = np.linspace(-np.pi / case['dr'][1], np.pi / case['dr'][1], ny,
                     endpoint=False)
    space['kx_mesh'], space['ky_mesh'] = np.meshgrid(kx, ky)
    del dk
    trial = os.path.join(str(tmpdir), 'trial_data') + os.sep
    os.makedirs(trial, exist_ok=True)
    return types.SimpleNamespace(
        paths={'data': str(tmpdir) + os.sep, 'trial': trial,
               'code': str(tmpdir) + os.sep, 'folder': 'golden'},
        rand_seed=None, atom_num=float(sc[0]), is_coupling=bool(sc[3]),
        g_sc={'uu': float(g[0]), 'dd': float(g[1]), 'ud': float(g[2])},
        kin_eng_spin=list(case['kin_eng_spin']),
        pot_eng_spin=list(case['pot_eng_spin']),
        psik=list(case['psik0']), space=space, coupling=case['coupling'],
        kL_recoil=float(sc[1]), rot_coupling=bool(sc[2]))


def rel_l2(a, b):
    """||a - b|| / ||b|| over all components."""
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))
