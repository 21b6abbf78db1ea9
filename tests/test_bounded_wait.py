"""Bounded device waits.

The pass kernels wait for their own bulk (TMA) copies on an mbarrier with a
limit; a wait that runs out records the plan's device error word and the
kernel continues instead of hanging.  This checks the limit on the GPU with
a phase that no copy completes, and that a healthy plan reports status 0.
"""
import ctypes

import pytest

from spinor_gpe.pspinor import _native


@pytest.mark.gpu
def test_wait_gives_up_by_its_limit():
    import torch
    assert torch.cuda.is_available()
    lib = _native.load()
    gave_up, ms = ctypes.c_int(), ctypes.c_double()
    _native.check(lib.sgpe_check_bounded_wait(ctypes.byref(gave_up), ctypes.byref(ms)))
    assert gave_up.value == 1
    assert 400.0 <= ms.value <= 5000.0


@pytest.mark.gpu
def test_healthy_plan_reports_no_device_error(tmp_path):
    import torch
    from spinor_gpe import workloads
    from spinor_gpe.pspinor import pspinor as spin
    from spinor_gpe.pspinor import tensor_propagator as tprop
    from spinor_gpe.pspinor import tensor_tools as ttools
    ps = workloads.raman_quench_1024(spin.PSpinor, ttools.fft_2d, str(tmp_path / 'q') + '/',
                                     n=1024, delta=0.5)
    prop = tprop.TensorPropagator(ps, 1e-3, 4, 'cuda', time='real', dtype=64)
    prop.full_steps(4)
    torch.cuda.synchronize()
    prop.check_device()


def test_wait_check_rejects_null_outputs(native_lib):
    lib = _native.load()
    assert lib.sgpe_check_bounded_wait(None, None) == _native.SGPE_ERR_ARG
