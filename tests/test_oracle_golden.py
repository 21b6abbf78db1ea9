"""The CPU oracle against golden vectors from the original spinor-gpe.

The fixtures were produced by ``tests/golden/make_golden.py`` running the
original package on the CPU; the oracle restatement must reproduce them
(it performs the same torch operations in the same order, so agreement is
at the level of FP64 rounding or exact).
"""
import itertools

import numpy as np
import pytest
import torch

from conftest import prop_case_names, case_params, load_cases, rel_l2
from oracle import (OraclePropagator, calc_pops, fft_1d, fft_2d, ifft_1d,
                    ifft_2d, inputs_from_arrays)

CASES = load_cases()
PROP_CASES = prop_case_names(CASES)


@pytest.mark.parametrize('name', PROP_CASES)
def test_oracle_matches_reference_propagation(name):
    case = CASES[name]
    p = case_params(case)
    tol = 1e-12 if p['dtype'] == 128 else 1e-6
    orc = OraclePropagator(inputs_from_arrays(case), p['dt'], p['time'],
                           p['dtype'])
    saved = [q.clone() for q in orc.psik]
    orc.single_step(orc.dt_out, orc.eng_out)
    assert rel_l2(orc.psik_numpy(), case['psik_single_out']) <= tol
    orc.psik = saved
    pops = np.empty((p['n_steps'], 2))
    for i in range(p['n_steps']):
        orc.full_step()
        pops[i] = calc_pops(orc.psik, orc.dv_k)
        if i == 0:
            assert rel_l2(orc.psik_numpy(), case['psik_step1']) <= tol
    assert rel_l2(orc.psik_numpy(), case['psik_final']) <= tol
    np.testing.assert_allclose(pops, case['pops'], rtol=tol, atol=tol)


def test_oracle_fft_helpers_match_reference():
    f = CASES['fft']
    psi = [torch.as_tensor(a) for a in f['in']]
    dr = torch.as_tensor(f['dr'])
    for fn, key in [(fft_2d, 'fft_2d'), (ifft_2d, 'ifft_2d')]:
        got = np.array([t.numpy() for t in fn(psi, dr)])
        assert rel_l2(got, f[key]) < 1e-14
    for fn, key, ax in [(fft_1d, 'fft_1d_x', 0), (fft_1d, 'fft_1d_y', 1),
                        (ifft_1d, 'ifft_1d_x', 0), (ifft_1d, 'ifft_1d_y', 1)]:
        got = np.array([t.numpy() for t in fn(psi, dr, ax)])
        assert rel_l2(got, f[key]) < 1e-14


# The invariants of the original's FFT tests (spinor_gpe/tests/fft_func_tests.py):
# all-ones grids over every shape in {128..1024}^2, tolerance 10 eps.
SHAPES = list(itertools.product([128, 256, 512, 1024], repeat=2))


@pytest.mark.parametrize('shape', SHAPES)
def test_oracle_fft_invariants(shape):
    eps = torch.finfo(torch.complex128).eps * 10
    grid = [torch.ones(shape, dtype=torch.complex128)] * 2
    dr = (1, 1)
    grid_k = fft_2d(grid, dr)
    grid_r = ifft_2d(grid_k, dr)
    for g, r in zip(grid, grid_r):          # for_back_torch_2d (:27-55)
        assert float(torch.max(torch.abs(r - g))) <= eps
    n = np.prod(shape)
    atoms = [sum(calc_pops(grid, 1.0)), sum(calc_pops(grid_r, 1.0))]
    assert abs(atoms[0] - atoms[1]) <= eps * n
    vol = 4 * np.pi**2 / n                  # compare_norm_torch (:453-472)
    atoms_k = sum(calc_pops(grid_k, vol))
    assert abs(atoms[0] - atoms_k) <= eps * n


def test_oracle_energy_convention_matches_reference():
    """The original's eng_expect on a phase-smooth ground state (golden,
    recorded with an identity phase unwrap, exact without wraps): potential
    and interaction terms agree exactly; the spectral kinetic term agrees with
    the original's finite differences to their O(dx^2) truncation (dx = 0.25)."""
    from oracle.energy import reference_convention
    e = CASES['energy']
    c = CASES['imag_plain_32']
    sc = c['scalars']
    got = reference_convention(e['psik'], e['kx_mesh'], e['ky_mesh'], sc[1],
                               bool(sc[3]), c['pot_eng_spin'], c['coupling'],
                               c['g'], c['dr'], c['dv'][0], c['dv'][1])
    ref = e['eng_expect']
    np.testing.assert_allclose(got[2:], ref[2:], rtol=1e-12)
    assert abs(got[1] - ref[1]) / ref[1] < 0.03
    assert abs(got[0] - ref[0]) / ref[0] < 1e-3
