"""Full-length validation of the solver on the named problem set-ups.

Test infrastructure (needs a CUDA GPU; not collected by pytest): each
set-up is run through the drop-in propagator and through the oracle, the
original algorithm restated in torch, here executed on the GPU in complex128.
Printed per set-up as one JSON line: relative L2 error of the final psik,
energy / chemical potential / atom number of both (FP64 functional), the
solver's steps/s.

    python tests/validate_configs.py [ground_state_256 raman_quench_1024 vortex_2048]

* ground_state_256: 256^2, complex128, 1000 imaginary steps, dt = 0.02.
* raman_quench_1024: 1024^2, complex64, 3000 imaginary steps at dt = 0.01,
  then delta 0 -> 0.5 and 10000 real steps at dt = 1e-3; real-time energy
  drift of both.
* vortex_2048: 2048^2, complex64 with FP32 DFTs, complex64 with the
  split-BF16 tensor-core DFT16 stages, and complex128; 2000 imaginary steps
  at dt = 0.01, 8 seeded vortices.
* curve_quench_1024, curve_vortex_2048: the error against the complex128
  oracle every 500 steps over the whole run (the quench: 3000 imaginary
  steps, then 10000 real-time steps, each implementation continuing from
  its own ground state; the vortex start: 2000 imaginary steps), for the
  solver in each precision (complex64, complex128, double-float), the
  original's own complex64 arithmetic, and
  two diagnostic complex128 oracle runs that isolate one FP32 effect each:
  the state rounded to complex64 after every sub-step (FP32 storage alone),
  and the operator tables rounded to complex64 (FP32 tables alone).  Besides
  the relative L2 error, the error after removing the best global phase is
  recorded.
"""
import json
import os
import sys
import tempfile
import time

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
for p in (os.path.join(REPO, 'spinor-gpe_gb300'), REPO):
    if p not in sys.path:
        sys.path.insert(0, p)

from oracle import OracleInputs, OraclePropagator          # noqa: E402
from oracle.energy import energy_functional                # noqa: E402
from spinor_gpe import workloads                           # noqa: E402
from spinor_gpe.pspinor import pspinor as spin             # noqa: E402
from spinor_gpe.pspinor import tensor_propagator as tprop  # noqa: E402
from spinor_gpe.pspinor import tensor_tools as ttools      # noqa: E402


def inputs(ps):
    return OracleInputs(
        psik=[np.asarray(p) for p in ps.psik],
        kin_eng_spin=[np.asarray(k) for k in ps.kin_eng_spin],
        pot_eng_spin=[np.asarray(v) for v in ps.pot_eng_spin],
        coupling=np.asarray(ps.coupling, dtype=np.float64),
        x_mesh=ps.space['x_mesh'], dr=ps.space['dr'],
        dv_r=float(ps.space['dv_r']), dv_k=float(ps.space['dv_k']),
        g_sc=dict(ps.g_sc), atom_num=float(ps.atom_num),
        kL_recoil=float(ps.kL_recoil), rot_coupling=bool(ps.rot_coupling),
        is_coupling=bool(ps.is_coupling))


def oracle_energy(ps, psik):
    theta = 0.0 if ps.rot_coupling else 2 * ps.kL_recoil * ps.space['x_mesh']
    g = (ps.g_sc['uu'], ps.g_sc['dd'], ps.g_sc['ud'])
    return energy_functional(psik, ps.kin_eng_spin, ps.pot_eng_spin,
                             np.asarray(ps.coupling, dtype=np.float64), theta, g,
                             ps.space['dr'], float(ps.space['dv_r']),
                             float(ps.space['dv_k']))


def rel_l2(a, b):
    return float(np.linalg.norm((np.asarray(a) - np.asarray(b)).ravel())
                 / np.linalg.norm(np.asarray(b).ravel()))


def run_solver(ps, dt, n, time_mode, dtype, tensor_core_dft=False):
    prop = tprop.TensorPropagator(ps, dt, n, 'cuda', time=time_mode, dtype=dtype,
                                  tensor_core_dft=tensor_core_dft)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    prop.full_steps(n)
    psik = [p.cpu().numpy().astype(np.complex128) for p in prop.psik]
    dt_s = time.perf_counter() - t0
    return prop, psik, n / dt_s


def run_oracle(ps, dt, n, time_mode, dtype=128):
    orc = OraclePropagator(inputs(ps), dt, time_mode, dtype, device='cuda')
    for _ in range(n):
        orc.full_step()
    return orc.psik_numpy()


def summary(name, ps, mine, ref, rate, extra=None):
    em = oracle_energy(ps, mine)
    er = oracle_energy(ps, ref)
    out = {'config': name, 'psik_rel_l2': rel_l2(mine, ref),
           'energy': em[4], 'energy_oracle': er[4],
           'energy_rel_err': abs(em[4] - er[4]) / abs(er[4]),
           'mu': em[5], 'mu_oracle': er[5], 'mu_rel_err': abs(em[5] - er[5]) / abs(er[5]),
           'atoms': em[7], 'atoms_oracle': er[7], 'steps_per_s': rate}
    if extra:
        out.update(extra)
    print(json.dumps(out), flush=True)


def ground_state_256(tmp):
    ps = workloads.ground_state_256(spin.PSpinor, ttools.fft_2d, tmp + '/c1/')
    _, mine, rate = run_solver(ps, 0.02, 1000, 'imag', 128)
    ref = run_oracle(ps, 0.02, 1000, 'imag')
    summary('ground_state_256 (complex128, 1000 imaginary steps)', ps, mine,
            ref, rate)


def raman_quench_1024(tmp):
    ps = workloads.raman_quench_1024(spin.PSpinor, ttools.fft_2d, tmp + '/c2/')
    prop, mine_g, rate_i = run_solver(ps, 0.01, 3000, 'imag', 64)
    ref_g = run_oracle(ps, 0.01, 3000, 'imag')
    ref_g64 = run_oracle(ps, 0.01, 3000, 'imag', 64)
    ground_err = rel_l2(mine_g, ref_g)
    print(json.dumps({'config': 'raman_quench_1024 ground state (complex64, 3000 imaginary steps)',
                      'psik_rel_l2': ground_err,
                      'original_complex64_psik_rel_l2': rel_l2(ref_g64, ref_g)}), flush=True)
    # quench from the same (oracle) ground state for both
    ps.psik = list(ref_g)
    ps.detuning_uniform(0.5)
    e0 = oracle_energy(ps, ref_g)[4]
    prop, mine, rate = run_solver(ps, 1e-3, 10000, 'real', 64)
    ref = run_oracle(ps, 1e-3, 10000, 'real')
    ref64 = run_oracle(ps, 1e-3, 10000, 'real', 64)
    summary('raman_quench_1024 (complex64, 3000 imag + 10000 real steps)', ps,
            mine, ref, rate,
            {'ground_state_psik_rel_l2': ground_err, 'imag_steps_per_s': rate_i,
             'original_complex64_psik_rel_l2': rel_l2(ref64, ref),
             'energy_drift_solver': (oracle_energy(ps, mine)[4] - e0) / abs(e0),
             'energy_drift_original_complex64': (oracle_energy(ps, ref64)[4] - e0) / abs(e0),
             'energy_drift_oracle': (oracle_energy(ps, ref)[4] - e0) / abs(e0)})


def vortex_2048(tmp):
    ps = workloads.vortex_2048(spin.PSpinor, ttools.fft_2d, tmp + '/c3/')
    ref = run_oracle(ps, 0.01, 2000, 'imag')
    ref64 = run_oracle(ps, 0.01, 2000, 'imag', 64)
    for dtype, tc in ((64, False), (64, True), (128, False)):
        _, mine, rate = run_solver(ps, 0.01, 2000, 'imag', dtype, tc)
        variant = 'split-BF16 tensor-core DFT16' if tc else 'FP32 DFT' if dtype == 64 else 'FP64'
        summary(f'vortex_2048 (complex{dtype}, {variant}, 2000 imaginary steps)', ps,
                mine, ref, rate, {'original_complex64_psik_rel_l2': rel_l2(ref64, ref)})


# ----------------------------------------------------- error-vs-step curves

class RoundedStateOracle(OraclePropagator):
    """complex128 oracle whose psik is rounded to complex64 after every
    sub-step: the effect of FP32 storage of the state alone."""

    def single_step(self, t_step, eng):
        super().single_step(t_step, eng)
        self.psik = [p.to(torch.complex64).to(torch.complex128) for p in self.psik]


class RoundedTablesOracle(OraclePropagator):
    """complex128 oracle whose pre-computed operator tables (kinetic,
    potential, coupling) are rounded to complex64: the effect of FP32 tables
    alone."""

    def __init__(self, *a, **k):
        super().__init__(*a, **k)

        def rnd(t):
            return t.to(torch.complex64).to(torch.complex128)
        for eng in (self.eng_out, self.eng_in):
            eng['kin'] = [rnd(e) for e in eng['kin']]
            eng['pot'] = [rnd(e) for e in eng['pot']]
            eng['coupl'] = [[rnd(e) for e in row] for row in eng['coupl']]


def phase_aligned_rel_l2(a, b):
    """min over a global phase phi of ||a e^{i phi} - b|| / ||b||."""
    a = np.asarray(a).ravel()
    b = np.asarray(b).ravel()
    ov = np.vdot(a, b)
    ph = ov / abs(ov) if abs(ov) > 0 else 1.0
    return float(np.linalg.norm(a * ph - b) / np.linalg.norm(b))


class OracleRunner:
    """Checkpointed run of one oracle class (complex128 unless dtype 64)."""

    def __init__(self, cls=OraclePropagator, dtype=128):
        self.cls, self.dtype = cls, dtype

    def start(self, ps, dt, time_mode):
        self.orc = self.cls(inputs(ps), dt, time_mode, self.dtype, device='cuda')

    def steps(self, n):
        for _ in range(n):
            self.orc.full_step()

    def psik(self):
        return self.orc.psik_numpy().astype(np.complex128)


class SolverRunner:
    """Checkpointed run of the drop-in propagator in one precision."""

    def __init__(self, dtype, **kw):
        self.dtype, self.kw = dtype, kw
        self.busy = 0.0

    def start(self, ps, dt, time_mode):
        self.prop = tprop.TensorPropagator(ps, dt, 1, 'cuda', time=time_mode,
                                           dtype=self.dtype, **self.kw)

    def steps(self, n):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        self.prop.full_steps(n)
        torch.cuda.synchronize()
        self.busy += time.perf_counter() - t0

    def psik(self):
        return np.array([p.cpu().numpy() for p in self.prop.psik]).astype(np.complex128)


def error_curve(name, build, phases, runners, every=500):
    """Run every runner through ``phases`` [(dt, n_steps, time, prepare)],
    where ``prepare(ps)`` (or None) changes the problem before a phase and
    each runner continues from its own state; print the error against the
    first runner (the complex128 oracle) every ``every`` steps."""
    tmp = tempfile.mkdtemp(prefix='sgpe_curve_')
    ref_points = None
    for i, (label, runner) in enumerate(runners):
        ps = build(tmp + f'/run{i}/')
        points, step = [], 0
        for dt, n, time_mode, prepare in phases:
            if step > 0:
                ps.psik = list(runner.psik())
            if prepare is not None:
                prepare(ps)
            runner.start(ps, dt, time_mode)
            done = 0
            while done < n:
                k = min(every, n - done)
                runner.steps(k)
                done += k
                step += k
                points.append((step, time_mode, runner.psik()))
        if ref_points is None:
            ref_points = points
            continue
        curve = [{'step': st, 'time': tm, 'psik_rel_l2': rel_l2(pk, rp[2]),
                  'phase_aligned_rel_l2': phase_aligned_rel_l2(pk, rp[2])}
                 for (st, tm, pk), rp in zip(points, ref_points)]
        out = {'config': name, 'variant': label, 'curve': curve}
        if isinstance(runner, SolverRunner):
            out['solver_steps_per_s'] = step / runner.busy
        print(json.dumps(out), flush=True)
        del points


def curve_runners(variants):
    """The complex128 oracle (reference), then the named variants."""
    table = {
        'original complex64': lambda: OracleRunner(dtype=64),
        'oracle complex128, state rounded to complex64 each sub-step':
            lambda: OracleRunner(RoundedStateOracle),
        'oracle complex128, operator tables rounded to complex64':
            lambda: OracleRunner(RoundedTablesOracle),
        'solver complex64': lambda: SolverRunner(64),
        'solver complex128': lambda: SolverRunner(128),
        'solver double-float': lambda: SolverRunner('double-float'),
    }
    return [('oracle complex128', OracleRunner())] + [(v, table[v]()) for v in variants]


CURVE_VARIANTS = ['original complex64',
                  'oracle complex128, state rounded to complex64 each sub-step',
                  'oracle complex128, operator tables rounded to complex64',
                  'solver complex64', 'solver complex128', 'solver double-float']


def curve_quench_1024(tmp, variants=None):
    def build(path):
        return workloads.raman_quench_1024(spin.PSpinor, ttools.fft_2d, path)
    error_curve('raman_quench_1024 (3000 imag + 10000 real steps)', build,
                [(0.01, 3000, 'imag', None),
                 (1e-3, 10000, 'real', lambda ps: ps.detuning_uniform(0.5))],
                curve_runners(variants or CURVE_VARIANTS))


def curve_vortex_2048(tmp, variants=None):
    def build(path):
        return workloads.vortex_2048(spin.PSpinor, ttools.fft_2d, path)
    error_curve('vortex_2048 (2000 imag steps)', build,
                [(0.01, 2000, 'imag', None)], curve_runners(variants or CURVE_VARIANTS))


CONFIGS = {'ground_state_256': ground_state_256,
           'curve_quench_1024': curve_quench_1024,
           'curve_vortex_2048': curve_vortex_2048,
           'raman_quench_1024': raman_quench_1024,
           'vortex_2048': vortex_2048}

if __name__ == '__main__':
    # python tests/validate_configs.py [config ...] [--variants "name" ...]
    argv = sys.argv[1:]
    variants = None
    if '--variants' in argv:
        k = argv.index('--variants')
        variants = argv[k + 1:]
        argv = argv[:k]
    names = argv or list(CONFIGS)
    tmp = tempfile.mkdtemp(prefix='sgpe_validate_')
    for n in names:
        if n.startswith('curve_'):
            CONFIGS[n](tmp, variants)
        else:
            CONFIGS[n](tmp)
