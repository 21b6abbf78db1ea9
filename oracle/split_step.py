"""Restatement of the original spinor-gpe split-step propagation on the CPU.

TEST INFRASTRUCTURE ONLY (see the package docstring): the checker and the
timed CPU baseline, never part of the solver.

Every function cites the file:line of the original it follows (paths are
relative to the spinor-gpe repository).  The arithmetic is carried out with
the same torch operations in the same order as the original, in complex128 by
default, so that the result is pinned to the original's own output on the
same inputs (golden fixtures in ``tests/golden``).

Parity-relevant details of the original reproduced here:

* the Strang composition uses gamma = 1/(2 + 2**(1/3)) for the two outer
  sub-steps and 1 - 2 gamma for the inner one
  (``spinor_gpe/pspinor/tensor_propagator.py:101-103``);
* the second interaction half-step reuses the operator built from the density
  after the first renormalisation (``tensor_propagator.py:262-267``);
* the atom number is renormalised in real space and in k-space in every
  sub-step, in real time as well (``tensor_propagator.py:244, 271``);
* the coupling operator is built with Omega/2 and the outer step for the outer
  sub-steps, and with Omega and half the inner step for the inner sub-step, so
  each application rotates by Omega t / 4 (``tensor_propagator.py:138-149``).
"""
from dataclasses import dataclass
from functools import reduce
import operator

import numpy as np
import torch


# --------------------------------------------------------------- tensor tools

def _prod(factors):
    """Product of a 1-D sequence (``spinor_gpe/pspinor/tensor_tools.py:594-600``)."""
    return reduce(operator.mul, factors, 1)


def fft_2d(psi, delta_r):
    """fftshift(fftn(psi_c)) * dx*dy/(2 pi) per component
    (``tensor_tools.py:201-228``)."""
    scale = _prod(delta_r) / (2 * np.pi)
    return [torch.fft.fftshift(torch.fft.fftn(p) * scale) for p in psi]


def ifft_2d(psik, delta_r):
    """ifftn(ifftshift(psik_c)) / (dx*dy/(2 pi)) per component
    (``tensor_tools.py:231-258``)."""
    scale = _prod(delta_r) / (2 * np.pi)
    return [torch.fft.ifftn(torch.fft.ifftshift(p)) / scale for p in psik]


def fft_1d(psi, delta_r, axis=0):
    """One-axis forward transform; ``axis`` 0 is x (array dim 1), 1 is y
    (``tensor_tools.py:130-164``)."""
    dim = (1, 0)[axis]
    scale = delta_r[axis] / np.sqrt(2 * np.pi)
    return [torch.fft.fftshift(torch.fft.fftn(p, dim=[dim]) * scale, dim=dim)
            for p in psi]


def ifft_1d(psik, delta_r, axis=0):
    """One-axis inverse transform (``tensor_tools.py:167-198``)."""
    dim = (1, 0)[axis]
    scale = delta_r[axis] / np.sqrt(2 * np.pi)
    return [torch.fft.ifftn(torch.fft.ifftshift(p, dim=dim), dim=dim) / scale
            for p in psik]


def density(psi):
    """|psi_c|^2 per component (``tensor_tools.py:392-441``)."""
    return [torch.abs(p)**2 for p in psi]


def norm(psi, vol_elem, atom_num):
    """Renormalise to the total atom number; also return the renormalised
    densities (``tensor_tools.py:261-311``, torch branch ``:301-305``)."""
    dens = density(psi)
    factor = (torch.sum(dens[0] + dens[1]) * vol_elem / atom_num).item()
    return ([p / np.sqrt(factor) for p in psi],
            [d / factor for d in dens])


def calc_pops(psi, vol_elem):
    """Per-component populations (``tensor_tools.py:466-484``)."""
    return [float(d.sum() * vol_elem) for d in density(psi)]


def evolution_op(t_step, energy):
    """exp(-i E t) per component (``tensor_tools.py:546-560``)."""
    return [torch.exp(-1.0j * e * t_step) for e in energy]


def coupling_op(t_step, coupling, expon):
    """2x2 coupling propagator [[cos a, -i sin a e^{-i th}],
    [-i sin a e^{+i th}, cos a]], a = coupling * t / 2
    (``tensor_tools.py:563-591``)."""
    arg = coupling * t_step / 2
    cos_a = torch.cos(arg)
    msin_a = -1.0j * torch.sin(arg)
    return [[cos_a, msin_a * torch.exp(-1.0j * expon)],
            [msin_a * torch.exp(1.0j * expon), cos_a]]


# ----------------------------------------------------------------- propagator

@dataclass
class OracleInputs:
    """Everything the original propagator reads from its ``PSpinor``
    (``tensor_propagator.py:93-129``)."""
    psik: list            # 2 x (Ny, Nx) complex128, centred k order
    kin_eng_spin: list    # 2 x (Ny, Nx) float64, centred k order
    pot_eng_spin: list    # 2 x (Ny, Nx) float64
    coupling: np.ndarray  # (Ny, Nx) float64
    x_mesh: np.ndarray    # (Ny, Nx) float64
    dr: np.ndarray        # (dx, dy)
    dv_r: float
    dv_k: float
    g_sc: dict            # {'uu', 'dd', 'ud'}
    atom_num: float
    kL_recoil: float
    rot_coupling: bool
    is_coupling: bool


def inputs_from_arrays(case):
    """Build ``OracleInputs`` from a dict of arrays as stored in the golden
    fixtures (keys without the case prefix)."""
    sc = case['scalars']
    g = case['g']
    return OracleInputs(
        psik=[np.asarray(p) for p in case['psik0']],
        kin_eng_spin=[np.asarray(k) for k in case['kin_eng_spin']],
        pot_eng_spin=[np.asarray(v) for v in case['pot_eng_spin']],
        coupling=np.asarray(case['coupling']),
        x_mesh=np.asarray(case['x_mesh']),
        dr=np.asarray(case['dr']),
        dv_r=float(case['dv'][0]), dv_k=float(case['dv'][1]),
        g_sc={'uu': float(g[0]), 'dd': float(g[1]), 'ud': float(g[2])},
        atom_num=float(sc[0]), kL_recoil=float(sc[1]),
        rot_coupling=bool(sc[2]), is_coupling=bool(sc[3]))


class OraclePropagator:
    """The original ``TensorPropagator`` time stepping, on plain inputs.

    ``time`` is 'imag' or 'real' (``tensor_propagator.py:95-99``);
    ``dtype`` 128 keeps the original complex128 arithmetic, 64 casts all
    tensors to complex64/float32 after the operators are built, the way a
    complex64 run of the original is obtained.
    """

    MAGIC_GAMMA = 1 / (2 + 2**(1 / 3))   # tensor_propagator.py:101

    def __init__(self, inp: OracleInputs, t_step, time='imag', dtype=128,
                 device='cpu'):
        self.time = time
        self.t_step = -1.0j * t_step if time == 'imag' else t_step
        self.dt_out = self.t_step * self.MAGIC_GAMMA
        self.dt_in = self.t_step * (1 - 2 * self.MAGIC_GAMMA)
        dev = device
        self.atom_num = inp.atom_num
        self.is_coupling = inp.is_coupling
        self.g_sc = dict(inp.g_sc)
        f64 = torch.float64
        kin = [torch.as_tensor(k, dtype=f64, device=dev)
               for k in inp.kin_eng_spin]
        pot = [torch.as_tensor(v, dtype=f64, device=dev)
               for v in inp.pot_eng_spin]
        self.psik = [torch.as_tensor(p, dtype=torch.complex128, device=dev)
                     for p in inp.psik]
        # float64 0-d tensors, as torch.tensor(numpy float64) gives in the
        # original (tensor_propagator.py:119-121)
        self.dr = torch.tensor(np.asarray(inp.dr, dtype=np.float64),
                               device=dev)
        self.dv_r = torch.tensor(inp.dv_r, dtype=f64, device=dev)
        self.dv_k = torch.tensor(inp.dv_k, dtype=f64, device=dev)
        coupling = torch.as_tensor(inp.coupling, dtype=f64, device=dev)
        if inp.rot_coupling:                       # tensor_propagator.py:125-129
            expon = torch.tensor(0.0)
        else:
            expon = 2 * inp.kL_recoil * torch.as_tensor(inp.x_mesh,
                                                        device=dev)
        # Pre-computed operators (tensor_propagator.py:138-149)
        self.eng_out = {'kin': evolution_op(self.dt_out / 2, kin),
                        'pot': evolution_op(self.dt_out, pot),
                        'coupl': coupling_op(self.dt_out, coupling / 2,
                                             expon)}
        self.eng_in = {'kin': evolution_op(self.dt_in / 2, kin),
                       'pot': evolution_op(self.dt_in, pot),
                       'coupl': coupling_op(self.dt_in / 2, coupling, expon)}
        if dtype == 64:
            self._cast_c64()

    def _cast_c64(self):
        c64 = torch.complex64
        self.psik = [p.to(c64) for p in self.psik]
        for eng in (self.eng_out, self.eng_in):
            eng['kin'] = [e.to(c64) for e in eng['kin']]
            eng['pot'] = [e.to(c64) for e in eng['pot']]
            eng['coupl'] = [[e.to(c64) for e in row] for row in eng['coupl']]
        self.dr = self.dr.to(torch.float32)
        self.dv_r = self.dv_r.to(torch.float32)
        self.dv_k = self.dv_k.to(torch.float32)

    @staticmethod
    def _apply_coupling(mat, psi):
        """psi <- C psi, summing row terms in order
        (``tensor_propagator.py:252-254``)."""
        return [sum([m * p for m, p in zip(row, psi)]) for row in mat]

    def single_step(self, t_step, eng):
        """One Strang sub-step (``tensor_propagator.py:224-271``)."""
        psik = [k * pk for k, pk in zip(eng['kin'], self.psik)]
        psi = ifft_2d(psik, self.dr)
        psi, dens = norm(psi, self.dv_r, self.atom_num)
        g = self.g_sc
        int_eng = [g['uu'] * dens[0] + g['ud'] * dens[1],
                   g['dd'] * dens[1] + g['ud'] * dens[0]]
        int_op = evolution_op(t_step / 2, int_eng)
        psi = [o * p for o, p in zip(int_op, psi)]
        if self.is_coupling:
            psi = self._apply_coupling(eng['coupl'], psi)
        psi = [v * p for v, p in zip(eng['pot'], psi)]
        if self.is_coupling:
            psi = self._apply_coupling(eng['coupl'], psi)
        psi = [o * p for o, p in zip(int_op, psi)]     # same int_op (:262-267)
        psik = fft_2d(psi, self.dr)
        psik = [k * pk for k, pk in zip(eng['kin'], psik)]
        self.psik, _ = norm(psik, self.dv_k, self.atom_num)

    def full_step(self):
        """Outer, inner, outer sub-steps (``tensor_propagator.py:214-222``)."""
        self.single_step(self.dt_out, self.eng_out)
        self.single_step(self.dt_in, self.eng_in)
        self.single_step(self.dt_out, self.eng_out)

    def run(self, n_steps, record_pops=True):
        """``n_steps`` full steps with per-step populations, as the loop in
        ``prop_loop`` (``tensor_propagator.py:185-194``) without sampling."""
        pops = np.empty((n_steps, 2))
        for i in range(n_steps):
            self.full_step()
            if record_pops:
                pops[i] = calc_pops(self.psik, self.dv_k)
        return pops

    def psik_numpy(self):
        return np.array([p.cpu().numpy() for p in self.psik])
