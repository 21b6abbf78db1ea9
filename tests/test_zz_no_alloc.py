"""The allocation-free transform entry point, sgpe_fft2_static.

It serves callers that cannot allocate device memory where they need a
transform (a host-owned pool allocator that holds the device's free memory,
latency-critical loops, foreign-language hosts holding raw pointers): it
uses a static device scratch array instead of a plan.  Here it is called
through the C ABI and compared with the plan-based sgpe_fft2 and with
NumPy's centred transform on two consecutive calls with different data,
forward and inverse, in both precisions, at the tolerances of the other
transform tests; after a warm-up call, repeat calls leave the device's free
memory unchanged.  The file is named so that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu

# the transform tests' tolerances, against the plan path and against NumPy
TOL = {torch.complex64: 2e-6, torch.complex128: 1e-14}


@pytest.fixture(scope='module')
def native():
    assert torch.cuda.is_available(), 'this test needs a CUDA device'
    from spinor_gpe.pspinor import _native
    _native.load()
    return _native


def _static(native, inp, out, inverse, scale):
    ny, nx = inp[0].shape
    bits = 64 if inp[0].dtype == torch.complex64 else 128
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    return native.load().sgpe_fft2_static(
        ny, nx, bits, inp[0].data_ptr(), inp[1].data_ptr(), out[0].data_ptr(),
        out[1].data_ptr(), int(inverse), float(scale), stream)


@pytest.mark.parametrize('dtype', [torch.complex64, torch.complex128])
@pytest.mark.parametrize('shape', [(64, 128), (256, 256), (32, 2048)])
def test_static_transform_matches_plan_transform(native, dtype, shape):
    ny, nx = shape
    bits = 64 if dtype == torch.complex64 else 128
    plan = native.Plan(ny, nx, bits, torch.cuda.current_device())
    rng = np.random.default_rng(11)
    for call in range(2):                      # two calls in a row, fresh data
        for inverse, scale in [(0, 0.0625 / (2 * np.pi)), (1, 1.0 / (nx * ny))]:
            inp = [torch.as_tensor(rng.standard_normal(shape)
                                   + 1j * rng.standard_normal(shape),
                                   dtype=dtype, device='cuda')
                   for _ in range(2)]
            ref = [torch.empty_like(inp[0]) for _ in range(2)]
            got = [torch.full_like(inp[0], float('nan')) for _ in range(2)]
            plan.fft2(torch, inp, ref, inverse, scale)
            rc = _static(native, inp, got, inverse, scale)
            assert rc == native.SGPE_OK, native.load().sgpe_last_error()
            torch.cuda.synchronize()
            r = np.array([t.cpu().numpy() for t in ref])
            g = np.array([t.cpu().numpy() for t in got])
            assert np.isfinite(g).all(), (call, inverse)
            assert rel_l2(g, r) <= TOL[dtype], (call, inverse)
            # directly against NumPy: forward = scale * fftshift(fft2(x)),
            # inverse = scale * (unnormalised inverse of ifftshift(x))
            x = np.array([t.cpu().numpy() for t in inp]).astype(np.complex128)
            if inverse:
                want = np.fft.ifft2(np.fft.ifftshift(x, axes=(1, 2)), axes=(1, 2)) * (nx * ny) * scale
            else:
                want = np.fft.fftshift(np.fft.fft2(x, axes=(1, 2)), axes=(1, 2)) * scale
            assert rel_l2(g, want) <= TOL[dtype], (call, inverse)
    plan.close()


def test_static_transform_allocates_nothing_on_repeat_calls(native):
    shape = (128, 256)
    inp = [torch.randn(shape, dtype=torch.complex64, device='cuda') for _ in range(2)]
    out = [torch.empty_like(inp[0]) for _ in range(2)]
    for inverse in (0, 1):                     # warm-up: loads the kernels' modules
        assert _static(native, inp, out, inverse, 1.0) == native.SGPE_OK
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    stats0 = torch.cuda.memory_stats().get('allocation.all.allocated', 0)
    for _ in range(3):
        for inverse in (0, 1):
            assert _static(native, inp, out, inverse, 1.0) == native.SGPE_OK
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert torch.cuda.memory_stats().get('allocation.all.allocated', 0) == stats0


def test_static_transform_rejects_grids_beyond_its_scratch(native):
    # 512 x 256 complex128 needs 4 MiB of scratch, more than the array holds
    a = [torch.zeros((512, 256), dtype=torch.complex128, device='cuda')
         for _ in range(2)]
    b = [torch.empty_like(a[0]) for _ in range(2)]
    rc = _static(native, a, b, 0, 1.0)
    assert rc == native.SGPE_ERR_ARG
    assert b'static scratch holds' in native.load().sgpe_last_error()
