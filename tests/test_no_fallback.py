"""The native library is the only compute path: without it, or on a CPU
device, the drop-in raises instead of falling back to another
implementation."""
import os
import subprocess
import sys

import pytest

from conftest import PKG, load_cases, spin_from_case

CASES = load_cases()


def test_missing_library_raises_import_error(tmp_path):
    code = ('import sys; sys.path.insert(0, %r)\n'
            'from spinor_gpe.pspinor import _native\n'
            'try:\n'
            '    _native.load()\n'
            'except ImportError as e:\n'
            '    print("raised", "no fallback" in str(e))\n' % PKG)
    env = dict(os.environ, SGPE_LIB_PATH=str(tmp_path / 'absent.so'))
    out = subprocess.run([sys.executable, '-c', code], env=env, capture_output=True, text=True,
                         timeout=300)
    assert out.stdout.strip() == 'raised True', out.stderr[-2000:]


@pytest.mark.parametrize('device', ['cpu', 'meta'])
def test_non_cuda_device_is_rejected(tmp_path, device):
    from spinor_gpe.pspinor import tensor_propagator as tprop
    case = CASES['imag_plain_32']
    with pytest.raises(ValueError, match='no CPU fallback'):
        tprop.TensorPropagator(spin_from_case(case, tmp_path), 0.02, 4, device, time='imag')
