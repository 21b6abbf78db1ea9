"""The golden-vector checks detect each parity-critical detail of the step.

Mistakes are planted in copies of the CPU oracle (never in the solver): each
variant changes one detail that the original propagator has
(spinor_gpe/pspinor/tensor_propagator.py:101, 138-149, 224-271), and its
result must miss the original's golden vectors by more than ten times the
complex128 tolerance of the GPU parity tests (1e-10), while the unmodified
oracle reproduces them to 1e-12.  (In real time at dt = 1e-3 a wrong
sub-step ratio changes 20 steps by ~2e-9 only: the splitting error is of
higher order in dt, so such a mistake is visible to the complex128 checks
and to the imaginary-time cases, not to the complex64 tolerance.)
"""
import pytest

from conftest import case_params, load_cases, rel_l2
from oracle import OraclePropagator, inputs_from_arrays
from oracle.split_step import coupling_op, evolution_op, ifft_2d, fft_2d, norm

CASES = load_cases()


class _Fresh(OraclePropagator):
    """Second interaction half step from the density after coupling and
    potential (the original reuses the first operator, :262-267)."""

    def single_step(self, t_step, eng):
        psik = [k * pk for k, pk in zip(eng['kin'], self.psik)]
        psi = ifft_2d(psik, self.dr)
        psi, dens = norm(psi, self.dv_r, self.atom_num)
        g = self.g_sc

        def int_op(d):
            return evolution_op(t_step / 2, [g['uu'] * d[0] + g['ud'] * d[1],
                                             g['dd'] * d[1] + g['ud'] * d[0]])
        psi = [o * p for o, p in zip(int_op(dens), psi)]
        if self.is_coupling:
            psi = self._apply_coupling(eng['coupl'], psi)
        psi = [v * p for v, p in zip(eng['pot'], psi)]
        if self.is_coupling:
            psi = self._apply_coupling(eng['coupl'], psi)
        dens2 = [(p.abs() ** 2).real for p in psi]
        psi = [o * p for o, p in zip(int_op(dens2), psi)]
        psik = fft_2d(psi, self.dr)
        psik = [k * pk for k, pk in zip(eng['kin'], psik)]
        self.psik, _ = norm(psik, self.dv_k, self.atom_num)


class _PlainStrang(OraclePropagator):
    """Three equal sub-steps instead of gamma = 1/(2 + 2^(1/3)) (:101)."""
    MAGIC_GAMMA = 1.0 / 3.0


def _coupling_full_angle(orc, inp):
    """Outer coupling with the full angle (the original halves it, :142)."""
    import torch
    coupling = torch.as_tensor(inp.coupling, dtype=torch.float64)
    expon = 2 * inp.kL_recoil * torch.as_tensor(inp.x_mesh)
    orc.eng_out['coupl'] = coupling_op(orc.dt_out, coupling, expon)


def _run(orc_cls, case, n_steps, tweak=None):
    p = case_params(case)
    inp = inputs_from_arrays(case)
    orc = orc_cls(inp, p['dt'], p['time'], 128)
    if tweak is not None:
        tweak(orc, inp)
    for _ in range(n_steps):
        orc.full_step()
    return orc.psik_numpy()


@pytest.mark.parametrize('name', ['imag_raman_64x32', 'real_raman_32'])
def test_unmodified_oracle_is_the_control(name):
    case = CASES[name]
    got = _run(OraclePropagator, case, case_params(case)['n_steps'])
    assert rel_l2(got, case['psik_final']) <= 1e-12


@pytest.mark.parametrize('name', ['imag_raman_64x32', 'real_raman_32'])
@pytest.mark.parametrize('variant', ['fresh_interaction', 'plain_strang', 'coupling_angle'])
def test_planted_mistake_is_detected(name, variant):
    case = CASES[name]
    n = case_params(case)['n_steps']
    if variant == 'fresh_interaction':
        got = _run(_Fresh, case, n)
    elif variant == 'plain_strang':
        got = _run(_PlainStrang, case, n)
    else:
        got = _run(OraclePropagator, case, n, _coupling_full_angle)
    assert rel_l2(got, case['psik_final']) > 1e-9
