"""Array helpers with the interface of spinor-gpe's ``tensor_tools``
(``spinor_gpe/pspinor/tensor_tools.py``).

* NumPy arrays are handled on the host with NumPy, as in the original; the
  problem set-up (``PSpinor``) runs there once per problem.
* CUDA tensors go through the native library: ``fft_2d`` / ``ifft_2d`` run
  the same row/column FFT kernels as the propagator.  Torch tensors on the
  CPU are rejected for the transforms: this package has no CPU compute path.
* Phase unwrapping (``phase(..., uwrap=True)``) needs scikit-image in the
  original (``tensor_tools.py:7, 531``); it is not provided here.
"""
import operator
from functools import reduce

import numpy as np
import torch

from . import _native

_PLANS = {}


def prod(factors):
    """Product of the elements of a 1-D sequence (tensor_tools.py:594-600)."""
    return reduce(operator.mul, factors, 1)


def to_numpy(input_tens):
    """Tensor (or list of tensors) -> NumPy array(s) (tensor_tools.py:14-38)."""
    if isinstance(input_tens, list):
        return [inp.cpu().numpy() for inp in input_tens]
    return input_tens.cpu().numpy()


def to_tensor(input_arr, dev='cpu', dtype=64):
    """NumPy array(s) -> tensor(s) of dtype 32/64/128 (tensor_tools.py:41-77)."""
    all_dtypes = {32: torch.float32, 64: torch.float64, 128: torch.complex128}
    if isinstance(input_arr, list):
        return [torch.as_tensor(inp, dtype=all_dtypes[dtype], device=dev)
                for inp in input_arr]
    return torch.as_tensor(input_arr, dtype=all_dtypes[dtype], device=dev)


def to_cpu(input_tens):
    """Move tensor(s) to host memory (tensor_tools.py:80-100)."""
    if isinstance(input_tens, list):
        return [inp.cpu() for inp in input_tens]
    return input_tens.cpu()


def to_gpu(input_tens, dev='cuda'):
    """Move tensor(s) to a CUDA device (tensor_tools.py:103-127)."""
    if isinstance(input_tens, list):
        return [inp.to(dev) for inp in input_tens]
    return input_tens.to(dev)


def _scalar_list(delta_r):
    if isinstance(delta_r, torch.Tensor):
        return [float(v) for v in delta_r.detach().cpu().reshape(-1)]
    return [float(v) for v in np.asarray(delta_r).reshape(-1)]


def _plan_for(t):
    ny, nx = t.shape
    bits = 64 if t.dtype == torch.complex64 else 128
    key = (ny, nx, bits, t.device.index)
    plan = _PLANS.get(key)
    if plan is None:
        plan = _native.Plan(ny, nx, bits, t.device.index)
        _PLANS[key] = plan
    return plan


def _prepare_cuda(psi):
    if len(psi) != 2:
        raise ValueError('the native transforms take two-component spinors')
    out = []
    for p in psi:
        if not p.is_complex():
            p = p.to(torch.complex128 if p.dtype == torch.float64
                     else torch.complex64)
        out.append(p.contiguous())
    if out[0].shape != out[1].shape or out[0].dtype != out[1].dtype:
        raise ValueError('both components must have the same shape and dtype')
    return out


def _native_fft2(psi, scale, inverse):
    psi = _prepare_cuda(psi)
    res = [torch.empty_like(psi[0]), torch.empty_like(psi[1])]
    _plan_for(psi[0]).fft2(torch, psi, res, inverse, scale)
    return res


def _reject_cpu_tensor(name):
    raise NotImplementedError(
        f'{name}: torch tensors on the CPU are not supported; this package '
        'computes on CUDA devices (NumPy arrays are handled on the host).')


def fft_2d(psi, delta_r=(1, 1)) -> list:
    """fftshift(fftn(psi_c)) * dx dy / (2 pi) (tensor_tools.py:201-228)."""
    normalization = prod(_scalar_list(delta_r)) / (2 * np.pi)
    if isinstance(psi[0], np.ndarray):
        return [np.fft.fftshift(np.fft.fftn(p) * normalization) for p in psi]
    if psi[0].is_cuda:
        return _native_fft2(psi, normalization, inverse=False)
    return _reject_cpu_tensor('fft_2d')


def ifft_2d(psik, delta_r=(1, 1)) -> list:
    """ifftn(ifftshift(psik_c)) / (dx dy / (2 pi)) (tensor_tools.py:231-258)."""
    normalization = prod(_scalar_list(delta_r)) / (2 * np.pi)
    if isinstance(psik[0], np.ndarray):
        return [np.fft.ifftn(np.fft.ifftshift(p)) / normalization
                for p in psik]
    if psik[0].is_cuda:
        n = psik[0].shape[0] * psik[0].shape[1]
        return _native_fft2(psik, 1.0 / (n * normalization), inverse=True)
    return _reject_cpu_tensor('ifft_2d')


def fft_1d(psi, delta_r=(1, 1), axis=0) -> list:
    """One-axis forward transform, NumPy only (tensor_tools.py:130-164):
    axis 0 is x (array dim 1), 1 is y."""
    true_ax = [1, 0]
    normalization = _scalar_list(delta_r)[axis] / np.sqrt(2 * np.pi)
    if not isinstance(psi[0], np.ndarray):
        raise NotImplementedError('fft_1d is provided for NumPy arrays only')
    return [np.fft.fftshift(np.fft.fftn(p, axes=[true_ax[axis]])
                            * normalization, axes=true_ax[axis]) for p in psi]


def ifft_1d(psik, delta_r=(1, 1), axis=0) -> list:
    """One-axis inverse transform, NumPy only (tensor_tools.py:167-198)."""
    true_ax = [1, 0]
    normalization = _scalar_list(delta_r)[axis] / np.sqrt(2 * np.pi)
    if not isinstance(psik[0], np.ndarray):
        raise NotImplementedError('ifft_1d is provided for NumPy arrays only')
    return [np.fft.ifftn(np.fft.ifftshift(p, axes=true_ax[axis]),
                         axes=[true_ax[axis]]) / normalization for p in psik]


def norm_sq(psi_comp):
    """|psi|^2 of one component (tensor_tools.py:414-441)."""
    if isinstance(psi_comp, np.ndarray):
        return np.abs(psi_comp)**2
    if isinstance(psi_comp, torch.Tensor):
        return torch.abs(psi_comp)**2
    raise TypeError(f'`psi_comp` is of type {type(psi_comp)}')


def density(psi):
    """Component densities (tensor_tools.py:392-411)."""
    if isinstance(psi, list):
        return [norm_sq(p) for p in psi]
    return norm_sq(psi)


def norm(psi, vol_elem, atom_num, pop_frac=None):
    """Renormalise a spinor to ``atom_num``; returns (psi, densities)
    (tensor_tools.py:261-311)."""
    if pop_frac is not None:
        raise NotImplementedError('Normalizing to the expected population '
                                  'fractions is not implemented.')
    dens = density(psi)
    if isinstance(dens[0], np.ndarray):
        factor = np.sum(dens[0] + dens[1]) * vol_elem / atom_num
        return [p / np.sqrt(factor) for p in psi], [d / factor for d in dens]
    factor = float((torch.sum(dens[0] + dens[1]) * vol_elem / atom_num).item())
    return [p / np.sqrt(factor) for p in psi], [d / factor for d in dens]


def calc_pops(psi, vol_elem=1.0):
    """Per-component populations (tensor_tools.py:466-484)."""
    return [float(d.sum() * vol_elem) for d in density(psi)]


def calc_atoms(psi, vol_elem=1.0):
    """Total atom number (tensor_tools.py:444-463)."""
    return sum(calc_pops(psi, vol_elem=vol_elem))


def conj(psi):
    """Complex conjugate of a spinor or component (tensor_tools.py:364-389)."""
    if isinstance(psi, list):
        return [conj(p) for p in psi]
    if isinstance(psi, np.ndarray):
        return np.conj(psi)
    return torch.conj(psi)


def grad_comp(psi_comp, delta_r):
    """Spatial gradient of one NumPy component (tensor_tools.py:331-348)."""
    if isinstance(psi_comp, np.ndarray):
        return np.gradient(psi_comp, *np.array(delta_r))
    raise NotImplementedError('Spatial gradients for tensors are not yet '
                              'implemented.')


def grad(psi, delta_r):
    """Gradient of a spinor or component (tensor_tools.py:314-328)."""
    if isinstance(psi, list):
        return [grad_comp(p, delta_r) for p in psi]
    return grad_comp(psi, delta_r)


def grad_sq_comp(psi_comp, delta_r):
    gx, gy = grad_comp(psi_comp, delta_r)
    return gx**2 + gy**2


def grad_sq(psi, delta_r):
    """|grad|^2 of a spinor or component (tensor_tools.py:351-361)."""
    if isinstance(psi, list):
        return [grad_sq_comp(p, delta_r) for p in psi]
    return grad_sq_comp(psi, delta_r)


def phase_comp(psi_comp, uwrap=False, dens=None):
    """Phase of one component, zeroed where the density is below 1e-6 of its
    maximum (tensor_tools.py:514-539)."""
    if uwrap:
        raise NotImplementedError('phase unwrapping (scikit-image in the '
                                  'original) is not provided')
    if isinstance(psi_comp, np.ndarray):
        ang = np.angle(psi_comp)
    else:
        ang = torch.angle(psi_comp)
    if dens is not None:
        ang[dens < (dens.max() * 1e-6)] = 0
    return ang


def phase(psi, uwrap=False, dens=None):
    """Phases of a spinor or component (tensor_tools.py:487-511)."""
    if isinstance(psi, list):
        dens = dens if dens is not None else [None] * len(psi)
        return [phase_comp(p, uwrap, d) for p, d in zip(psi, dens)]
    return phase_comp(psi, uwrap, dens)


def evolution_op(t_step, energy):
    """exp(-i E t) (tensor_tools.py:546-560)."""
    if isinstance(energy, list):
        return [torch.exp(-1.0j * eng * t_step) for eng in energy]
    return torch.exp(-1.0j * energy * t_step)


def coupling_op(t_step, coupling=None, expon=torch.tensor(0)):
    """2x2 coupling propagator (tensor_tools.py:563-591)."""
    if coupling is None:
        coupling = torch.tensor(0)
    arg = coupling * t_step / 2
    cosine = torch.cos(arg)
    sine = -1.0j * torch.sin(arg)
    return [[cosine, sine * torch.exp(-1.0j * expon)],
            [sine * torch.exp(1.0j * expon), cosine]]
