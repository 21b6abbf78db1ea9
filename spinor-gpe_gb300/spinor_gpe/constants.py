"""Physical constants (SI) used by the problem set-up, with the Rb-87 data
of spinor-gpe (``spinor_gpe/constants.py:14-35``)."""
import scipy.constants as const

h = const.h
hbar = const.hbar
c = const.c
eps0 = const.epsilon_0
a0 = const.physical_constants['Bohr radius'][0]
e = const.elementary_charge

Rb87 = {}
Rb87['m'] = 87 * 1.66e-27                      # mass [kg]
Rb87['D2'] = 780.1e-9                          # D2 line wavelength [m]
Rb87['a_sc'] = 100.4 * a0                      # scattering length [m]
Rb87['g'] = 4 * const.pi * (hbar**2) * Rb87['a_sc'] / Rb87['m']
Rb87['k_r'] = 2 * const.pi / Rb87['D2']        # resonant recoil wavenumber [1/m]
Rb87['E_r'] = (h / (2 * Rb87['m'])) * (1 / Rb87['D2'])**2   # recoil energy [Hz]
Rb87['D1_alpha'] = h * 1.22306e-5              # D1 scalar polarizability [Hz m^2/V^2]
Rb87['gJ_S12'] = 2.002331
Rb87['gJ_P12'] = 0.666
Rb87['gJ_P32'] = 1.3362
Rb87['delta_FS'] = 6.834682e9                  # ground-state hyperfine splitting [Hz]
