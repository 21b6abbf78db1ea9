"""The C ABI library: it loads, exports every function declared in
``include/spinor_gb300.h``, and its ctypes mirror of the structs matches the
C layout.  Only argument checks that return before any CUDA call are
exercised here (no GPU in this suite)."""
import ctypes
import os
import re

import pytest

from conftest import REPO
from spinor_gpe.pspinor import _native

HEADER = os.path.join(REPO, 'include', 'spinor_gb300.h')


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r'^\s*(?:const\s+)?\w+\*?\s+\**(sgpe_\w+)\s*\(',
                                 text, flags=re.M)))


def test_header_declares_the_binding(native_lib):
    assert declared_functions() == sorted(_native.EXPORTED)


def test_library_exports_every_declared_symbol(native_lib):
    lib = ctypes.CDLL(native_lib)
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_struct_layout():
    assert ctypes.sizeof(_native.Field) == 24
    assert ctypes.sizeof(_native.SubstepOps) == 11 * 24 + 16
    assert _native.SubstepOps.int_z_re.offset == 11 * 24


def test_argument_errors_without_gpu(native_lib):
    lib = _native.load()
    h = ctypes.c_void_p()
    # unsupported sizes and dtypes are rejected before any device work
    assert lib.sgpe_plan_create(ctypes.byref(h), 48, 64, 64, 0) == _native.SGPE_ERR_ARG
    assert b'powers of two' in lib.sgpe_last_error()
    assert lib.sgpe_plan_create(ctypes.byref(h), 64, 8192, 64, 0) == _native.SGPE_ERR_ARG
    assert lib.sgpe_plan_create(ctypes.byref(h), 64, 64, 32, 0) == _native.SGPE_ERR_ARG
    assert lib.sgpe_plan_create(None, 64, 64, 64, 0) == _native.SGPE_ERR_ARG
    assert lib.sgpe_set_physics(None, 1, 1, 1, 1, 1, 1, 0) == _native.SGPE_ERR_ARG
    assert lib.sgpe_full_steps(None, 1, None, None) == _native.SGPE_ERR_ARG
    assert lib.sgpe_plan_destroy(None) == _native.SGPE_OK
    assert lib.sgpe_set_dft_mode(None, 1) == _native.SGPE_ERR_ARG
    with pytest.raises(_native.SgpeError):
        _native.check(lib.sgpe_single_step(None, 0, None))
    # batch and work-queue entry points
    st = ctypes.c_int(-1)
    assert lib.sgpe_batch_steps(None, 1, None) == _native.SGPE_ERR_ARG
    assert lib.sgpe_batch_set_queue(None, 1) == _native.SGPE_ERR_ARG
    assert lib.sgpe_batch_device_status(None, ctypes.byref(st)) == _native.SGPE_ERR_ARG
    assert lib.sgpe_check_queue_wait(None, None) == _native.SGPE_ERR_ARG
    assert lib.sgpe_batch_destroy(None) == _native.SGPE_OK
    assert lib.sgpe_version() >= 100


def test_double_float_dtype_constant_and_parsing():
    """The header's double-float dtype code is the one the binding passes;
    the propagator accepts it by name and rejects other names before any
    device work."""
    m = re.search(r'#define\s+SGPE_DTYPE_DF\s+(\d+)', open(HEADER).read())
    assert m and int(m.group(1)) == _native.SGPE_DTYPE_DF
    from spinor_gpe.pspinor import tensor_propagator as tprop
    for name in ('double-float', 'df', _native.SGPE_DTYPE_DF):
        assert tprop._bits(name) == _native.SGPE_DTYPE_DF
    assert tprop._bits('complex64') == 64 and tprop._bits(128) == 128
    with pytest.raises(ValueError):
        tprop._bits('bfloat16')
