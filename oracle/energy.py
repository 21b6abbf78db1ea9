"""FP64 energy functional of a spinor on the CPU (NumPy).

TEST INFRASTRUCTURE ONLY: the checker of the device energy reductions.

Physical energy of the Hamiltonian the propagator applies
(spinor_gpe/pspinor/tensor_propagator.py:224-271):
  E_kin = sum_k K_c |psik_c|^2 dv_k,  E_pot = sum V_c n_c dv_r,
  E_int = sum (g_uu n0^2/2 + g_dd n1^2/2 + g_ud n0 n1) dv_r,
  E_cpl = sum 2 Re(conj(psi_0) h psi_1) dv_r, h = (Omega/2) exp(-i theta),
  mu = (E_kin + E_pot + E_cpl + 2 E_int) / N,
with psi = ifft_2d(psik) (tensor_tools.py:231-258).  Also the sums of the
original's reporting convention (tensor_propagator.py:308-324): grid sums
without dv_r, interaction without 1/2, coupling Omega Re(conj(psi_0) psi_1),
and a spectral kinetic term sum_k ((kx^2+ky^2)/2 + kL kx) |psik|^2 dv_k / dv_r.
"""
import numpy as np


def _ifft_2d(psik, dr):
    scale = dr[0] * dr[1] / (2 * np.pi)
    return [np.fft.ifftn(np.fft.ifftshift(p)) / scale for p in psik]


def energy_functional(psik, kin, pot, coupling, theta, g, dr, dv_r, dv_k):
    """[E_kin, E_pot, E_int, E_cpl, E_total, mu, N_k, N_r, S1, S2]."""
    psik = [np.asarray(p, dtype=np.complex128) for p in psik]
    densk = [np.abs(p)**2 for p in psik]
    e_kin = sum(float(np.sum(k * d)) for k, d in zip(kin, densk)) * dv_k
    n_k = sum(float(np.sum(d)) for d in densk) * dv_k
    psi = _ifft_2d(psik, dr)
    n0, n1 = np.abs(psi[0])**2, np.abs(psi[1])**2
    e_pot = float(np.sum(pot[0] * n0 + pot[1] * n1)) * dv_r
    s1 = float(np.sum(g[0] * n0**2 + g[1] * n1**2)) * dv_r
    s2 = float(np.sum(g[2] * n0 * n1)) * dv_r
    h = np.asarray(coupling) / 2 * np.exp(-1.0j * np.asarray(theta))
    e_cpl = float(np.sum(2 * np.real(np.conj(psi[0]) * h * psi[1]))) * dv_r
    n_r = float(np.sum(n0 + n1)) * dv_r
    e_int = 0.5 * s1 + s2
    total = e_kin + e_pot + e_int + e_cpl
    mu = (e_kin + e_pot + e_cpl + 2 * e_int) / n_r
    return np.array([e_kin, e_pot, e_int, e_cpl, total, mu, n_k, n_r, s1, s2])


def reference_convention(psik, kx, ky, kl, is_coupling, pot, coupling, g, dr,
                         dv_r, dv_k):
    """[E_tot, E_kin, E_pot, E_int] in the original's convention with a
    spectral kinetic term."""
    psik = [np.asarray(p, dtype=np.complex128) for p in psik]
    w = (kx**2 + ky**2) / 2 + (kl * kx if is_coupling else 0.0)
    kin = sum(float(np.sum(w * np.abs(p)**2)) for p in psik) * dv_k / dv_r
    psi = _ifft_2d(psik, dr)
    n0, n1 = np.abs(psi[0])**2, np.abs(psi[1])**2
    pot_e = float(np.sum(pot[0] * n0 + pot[1] * n1))
    int_e = float(np.sum(g[0] * n0**2 + g[1] * n1**2 + g[2] * n0 * n1))
    cpl = float(np.sum(np.real(np.conj(psi[0]) * psi[1] + np.conj(psi[1]) * psi[0])
                       * coupling / 2))
    return [kin + pot_e + int_e + cpl, kin, pot_e, int_e]
