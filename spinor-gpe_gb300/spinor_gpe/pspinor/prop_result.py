"""``PropResult``: the result container returned by propagation
(``spinor_gpe/pspinor/prop_result.py:19-82``).

Holds NumPy copies of the final real- and k-space spinor, the final energies,
the per-step populations and the path of the sampled-wavefunction file, plus
the derived densities and phases.  The matplotlib plotting and movie methods
of the original are outside this package and raise ``NotImplementedError``.
"""
import numpy as np

from . import tensor_tools as ttools


class PropResult:
    """Result of a propagation (see the module docstring)."""

    def __init__(self, psi_final, psik_final, eng_final, pops,
                 sampled_path=None, derived=None):
        """``derived`` (optional): the densities, k-space densities, masked
        phases and FP64 separation sums already computed on the device
        (``TensorPropagator.analysis``); without it they are computed here
        from the NumPy arrays as in the original."""
        self.psi = psi_final
        self.psik = psik_final
        self.eng_final = eng_final
        self.pops = pops
        self.sampled_path = sampled_path
        self._sep_sums = None

        if derived is not None:
            self.dens = list(derived['dens'])
            self.densk = list(derived['densk'])
            self.phase = list(derived['phase'])
            self._sep_sums = tuple(float(v) for v in derived['sums'][:3])
        else:
            self.dens = ttools.density(self.psi)
            self.densk = ttools.density(self.psik)
            self.phase = ttools.phase(self.psi, uwrap=False, dens=self.dens)

        self.paths = dict()
        self.time_scale = None
        self.space = dict()

    def calc_separation(self):
        """Phase-separation measure 1 - sum(n0 n1)/sqrt(sum n0^2 sum n1^2)
        (prop_result.py:84-88); from the device's FP64 sums when the result
        came with them."""
        if self._sep_sums is not None:
            s01, s00, s11 = self._sep_sums
            return 1 - s01 / np.sqrt(s00 * s11)
        return 1 - (np.sum(ttools.prod(self.dens))
                    / np.sqrt(np.sum(self.dens[0]**2)
                              * np.sum(self.dens[1]**2)))

    def _no_plotting(self, *_, **__):
        raise NotImplementedError('plotting is not part of this package; '
                                  'use the NumPy arrays on this object')

    plot_spins = plot_total = plot_eng = plot_pops = make_movie = _no_plotting
