"""Benchmark of the GB300 split-step solver.

Workload (default): the real-time Raman-dressed quench on a 1024x1024
two-component grid over [-32,32)^2 in complex64: g_uu = g_dd = 1000,
g_ud = 990, Omega = 1, k_L = 3 (theta = 2 k_L x), prepared by 3000
imaginary-time steps at dt = 0.01 before the timed region, then quenched to
delta = 0.5 and propagated in real time at dt = 1e-3.  A step is one full
Strang step (three sub-steps) of one solve; the metric is full steps per
second.

To keep the timed working set larger than the 129 MB L2, R independent
copies of the solve (replicas, 16 MiB of state each) are stepped round-robin,
so consecutive steps never reuse a cached state; R is chosen so that the
replicas' states are at least twice the L2 size.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl native|reference]

Under torchrun each rank runs its own replicas on its own GPU ("replicas
only": a solve is never split across GPUs); the time is the maximum over
ranks and the value counts the steps of all ranks.

``--impl reference`` times the original algorithm's CPU path (the oracle's
restatement of spinor-gpe's torch propagator) on the host cores, on the same
workload, and also its torch CUDA path on the same GPU.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, 'spinor-gpe_gb300'))

METRIC = 'full Strang steps/s @1024^2 complex64 (real-time Raman quench)'
UNIT = 'steps/s'
L2_BYTES = 129 * 2**20
FALLBACK_HBM_GBS = 6800.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=1000)
    ap.add_argument('--warmup', type=int, default=10)
    ap.add_argument('--impl', default='native', choices=['native', 'reference'])
    ap.add_argument('--grid', '--n', dest='n', type=int, default=1024,
                    help='grid side')
    ap.add_argument('--prep-steps', type=int, default=3000)
    ap.add_argument('--no-cpu-baseline', action='store_true')
    ap.add_argument('--workload', default='raman_quench',
                    choices=['raman_quench', 'batched_uneven', 'served'],
                    help='raman_quench (headline); batched_uneven (independent '
                         'ground states stepped as one batch against the same '
                         'solves run one after another); served (a Poisson '
                         'request stream through the continuous-batching loop '
                         'against the same requests solved one after another)')
    ap.add_argument('--solves', type=int, default=96)
    ap.add_argument('--batch-extra-steps', type=int, default=50,
                    help='raman_quench: also time the batched uneven solves for this '
                         'many steps (0: skip) and report them in the same line')
    ap.add_argument('--precision-modes', nargs='*', default=['double-float', '128'],
                    help='raman_quench: also time these precisions on the same '
                         'workload and report them in the same line')
    ap.add_argument('--breakdown', action='store_true',
                    help='batched_uneven: also time each grid-size class alone '
                         '(one solve, the class sequentially, the class batched)')
    ap.add_argument('--batch-steps', type=int, default=2000)
    ap.add_argument('--serve-rate', type=float, default=200.0)
    ap.add_argument('--serve-window', type=float, default=0.5)
    ap.add_argument('--max-active', type=int, default=64)
    ap.add_argument('--serve-max-queue', type=float, default=None,
                    help='served: shed requests that waited longer than this many '
                         'seconds for admission (default: never shed)')
    ap.add_argument('--serve-seq-sample', type=int, default=0,
                    help='served: run the sequential baseline on a seeded sample of '
                         'this many served requests (0: all of them)')
    ap.add_argument('--dtype', default='64', choices=['64', '128', 'double-float'],
                    help='raman_quench: precision of the timed solves (complex64, '
                         'complex128, or double-float: FP32 head + tail pairs)')
    ap.add_argument('--tensor-core-dft', action='store_true',
                    help='raman_quench: run the split-BF16 tensor-core DFT16 '
                         'variant (precision study; not the headline)')
    ap.add_argument('--kernel-shapes', type=int, nargs=2, default=None, metavar=('ROW', 'COL'),
                    help='raman_quench: run the solves in these kernel shapes instead of the '
                         'defaults (sgpe_shape_count lists them)')
    ap.add_argument('--batch-sizes', type=int, nargs='+', default=None,
                    help='batched_uneven: draw the grid sides from these (default '
                         '128 192 256 384 512 768 1024)')
    ap.add_argument('--batch-queue', action='store_true',
                    help='batched_uneven: step the batch with the work-queue kernel (one '
                         'persistent launch per graph) instead of grouped launches')
    ap.add_argument('--no-batch-autotune', action='store_true',
                    help='batched_uneven: keep every solve in its default kernel shapes '
                         '(no PropagatorBatch.autotune)')
    ap.add_argument('--host-setup', action='store_true',
                    help='served: build each request with the host PSpinor '
                         'set-up instead of the device set-up')
    return ap.parse_args()


# ------------------------------------------------------------------ helpers

def dist_setup():
    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    if world > 1:
        import torch.distributed as dist
        import torch
        backend = 'nccl' if torch.cuda.is_available() else 'gloo'
        dist.init_process_group(backend)
    return world, rank, local


def max_over_ranks(x, world):
    """Maximum of a float over all ranks (x itself when world == 1)."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = 'cuda' if dist.get_backend() == 'nccl' else 'cpu'
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def measured_peaks():
    path = os.path.join(REPO, 'MEASURED_PEAKS.json')
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d['hbm_gbs']), 'measured'
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM_GBS, 'fallback'


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during a region."""

    FIELDS = ('index,clocks.sm,clocks.max.sm,power.draw,'
              'clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,'
              'clocks_event_reasons.hw_thermal_slowdown,'
              'clocks_event_reasons.sw_thermal_slowdown,'
              'clocks_event_reasons.sw_power_cap')

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix='.csv')
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ['nvidia-smi', '-i', str(self.gpu), '--query-gpu=' + self.FIELDS,
                 '--format=csv,noheader,nounits', '-lms', '100'],
                stdout=open(self.path, 'w'), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['unsampled']}
        sm, smax, reasons = [], [], set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown',
                 'sw_power_cap']
        for line in open(self.path):
            parts = [p.strip() for p in line.split(',')]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == 'active':
                    reasons.add(name)
        os.unlink(self.path)
        if not sm:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['unsampled']}
        return {'sm_mhz': statistics.median(sm), 'sm_max_mhz': max(smax),
                'samples': len(sm), 'reasons': sorted(reasons)}


def build_problem(tmpdir, n, prep_steps, device, dtype=64):
    """The 1024^2 quench workload: imaginary-time preparation at delta = 0
    (untimed), then delta -> 0.5.  Returns the PSpinor ready for real time."""
    import torch
    from spinor_gpe import workloads
    from spinor_gpe.pspinor import pspinor as spin
    from spinor_gpe.pspinor import tensor_tools as ttools
    from spinor_gpe.pspinor import tensor_propagator as tprop
    ps = workloads.raman_quench_1024(spin.PSpinor, ttools.fft_2d,
                                     os.path.join(tmpdir, 'quench') + '/',
                                     n=n, delta=0.0)
    if prep_steps > 0 and device is not None:
        prop = tprop.TensorPropagator(ps, 0.01, prep_steps, device,
                                      time='imag', dtype=dtype)
        prop.full_steps(prep_steps)
        ps.psik = [p.cpu().numpy() for p in prop.psik]
        del prop
        torch.cuda.synchronize()
    ps.detuning_uniform(0.5)
    return ps


# ------------------------------------------------------------- CPU baseline

def cpu_reference_rate(ps, budget_s=12.0, max_steps=50, dtype=64):
    """Full steps/s of the original algorithm on the host cores (the oracle's
    torch restatement, all intra-op threads), on a bounded sample."""
    import torch
    sys.path.insert(0, REPO)
    from oracle import OraclePropagator, OracleInputs
    torch.set_num_threads(os.cpu_count() or 1)
    inp = OracleInputs(
        psik=[np.asarray(p) for p in ps.psik],
        kin_eng_spin=[np.asarray(k) for k in ps.kin_eng_spin],
        pot_eng_spin=[np.asarray(v) for v in ps.pot_eng_spin],
        coupling=np.asarray(ps.coupling, dtype=np.float64),
        x_mesh=ps.space['x_mesh'], dr=ps.space['dr'],
        dv_r=float(ps.space['dv_r']), dv_k=float(ps.space['dv_k']),
        g_sc=dict(ps.g_sc), atom_num=float(ps.atom_num),
        kL_recoil=float(ps.kL_recoil), rot_coupling=bool(ps.rot_coupling),
        is_coupling=bool(ps.is_coupling))
    orc = OraclePropagator(inp, 1e-3, 'real', dtype)
    orc.full_step()                       # warm-up
    t0 = time.perf_counter()
    orc.full_step()
    one = time.perf_counter() - t0
    n = int(max(2, min(max_steps, budget_s / max(one, 1e-6))))
    t0 = time.perf_counter()
    for _ in range(n):
        orc.full_step()
    dt = time.perf_counter() - t0
    return {'value': n / dt, 'unit': UNIT, 'cores': torch.get_num_threads(),
            'kind': 'port',
            'sample': f'{n} real-time full steps of one {ps.psik[0].shape[0]}^2 '
                      f'complex64 solve (the oracle, torch CPU, '
                      f'{torch.get_num_threads()} threads)'}, inp


def torch_cuda_reference_rate(inp, steps=30, warmup=3, dtype=64):
    """Full steps/s of the original algorithm's torch CUDA path (the oracle's
    restatement run on the GPU: torch.fft, ATen element-wise kernels and the
    original's host synchronisations)."""
    import torch
    from oracle import OraclePropagator
    orc = OraclePropagator(inp, 1e-3, 'real', dtype, device='cuda')
    for _ in range(warmup):
        orc.full_step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        orc.full_step()
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    return steps / dt


# --------------------------------------------------------------- native arm

def precision_mode_rate(ps, mode, n, device, world, k, warmup):
    """Full steps/s of the same workload in another precision: replicas
    stepped round-robin as in the headline (inputs larger than L2), CUDA
    events on the stream, every replica warmed into graph replay first."""
    import torch
    from spinor_gpe.pspinor import tensor_propagator as tprop
    dtype = mode if mode == 'double-float' else int(mode)
    elem = 8 if dtype == 64 else 16
    n_rep = max(1, math.ceil(2 * L2_BYTES / (2 * n * n * elem)) + 1)
    props = [tprop.TensorPropagator(ps, 1e-3, k, device, time='real', dtype=dtype)
             for _ in range(n_rep)]
    for _ in range(3):
        for p in props:
            p.full_steps(1)
    for i in range(warmup):
        props[i % n_rep].full_steps(1)
    stream = torch.cuda.current_stream()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for i in range(k):
        props[i % n_rep].full_steps(1)
    ev1.record(stream)
    torch.cuda.synchronize()
    t = max_over_ranks(ev0.elapsed_time(ev1) / 1e3, world)
    del props
    return {'value': world * k / t, 'unit': UNIT, 'steps': k, 'replicas': n_rep,
            'dtype': {'double-float': 'double-float (fp32 head + tail pairs, ~48 bits)',
                      '128': 'c128 (fp64)', '64': 'c64'}[str(mode)]}



def run_native(args, world, rank, local):
    import torch
    from spinor_gpe.pspinor import tensor_propagator as tprop
    torch.cuda.set_device(local)
    device = f'cuda:{local}'
    n = args.n
    tmp = tempfile.mkdtemp(prefix='sgpe_bench_')
    ps = build_problem(tmp, n, args.prep_steps, device)
    dtype = args.dtype if args.dtype == 'double-float' else int(args.dtype)
    elem = 8 if dtype == 64 else 16       # bytes per complex value of the state
    host_ctype = torch.complex64 if dtype == 64 else torch.complex128
    state_bytes = 2 * n * n * elem
    n_rep = max(1, math.ceil(2 * L2_BYTES / state_bytes) + 1)
    psik_host = [torch.as_tensor(np.asarray(p), dtype=host_ctype)
                 .pin_memory() for p in ps.psik]
    shapes = tuple(args.kernel_shapes) if args.kernel_shapes else None
    props = [tprop.TensorPropagator(ps, 1e-3, args.steps, device, time='real',
                                    dtype=dtype, tensor_core_dft=args.tensor_core_dft,
                                    kernel_shapes=shapes)
             for _ in range(n_rep)]
    stream = torch.cuda.current_stream()

    # warm-up.  Every replica first takes three single steps: the first is
    # eager (the state arrives in k-space form), the second captures the
    # plan's one-step graph (allocating its merged kinetic tables before the
    # capture), the third replays it.  Only then are all replicas in the
    # steady state the timed region measures; --warmup adds round-robin
    # steps on top.
    for _ in range(3):
        for p in props:
            p.full_steps(1)
    for i in range(args.warmup):
        props[i % n_rep].full_steps(1)
    torch.cuda.synchronize()

    # ---- device-timed region: K steps round-robin over the replicas
    k = args.steps
    barrier(world)
    torch.cuda.synchronize()
    # events also split the region into 10 windows (median window reported
    # beside the whole-region value)
    n_win = 10 if k >= 10 else 1
    bounds = [round(w * k / n_win) for w in range(n_win + 1)]
    with ClockSampler(local) as clk:
        evs = [torch.cuda.Event(enable_timing=True) for _ in range(n_win + 1)]
        evs[0].record(stream)
        w = 1
        for i in range(k):
            props[i % n_rep].full_steps(1)
            if i + 1 == bounds[w]:
                evs[w].record(stream)
                w += 1
        torch.cuda.synchronize()
    barrier(world)
    ev0, ev1 = evs[0], evs[-1]
    t_dev = ev0.elapsed_time(ev1) / 1e3
    t_max = max_over_ranks(t_dev, world)
    value = world * k / t_max
    win_rates = [(bounds[w + 1] - bounds[w]) / (evs[w].elapsed_time(evs[w + 1]) / 1e3)
                 for w in range(n_win)]
    median_window = world * statistics.median(win_rates)

    # ---- per-pass roofline (same workload, events around every pass)
    col_ms, row_ms = props[0]._plan.time_passes(torch, 50, props[0]._device)

    # ---- end to end through the public API, host buffers
    pops_dev = [torch.empty((k, 2), dtype=torch.float64, device=device)
                for _ in range(n_rep)]
    pops_host = torch.empty((k, 2), dtype=torch.float64).pin_memory()
    out_host = [[torch.empty((n, n), dtype=host_ctype).pin_memory()
                 for _ in range(2)] for _ in range(n_rep)]
    # the state loads run on one side stream and the final reads on another,
    # ordered against the steps by events, so copies overlap the steps of
    # the other replicas (the psik setter and getter work on the caller's
    # current stream)
    h2d_stream = torch.cuda.Stream(device)
    d2h_stream = torch.cuda.Stream(device)
    loaded = [torch.cuda.Event() for _ in range(n_rep)]
    stepped = [torch.cuda.Event() for _ in range(n_rep)]
    last = {i % n_rep: i for i in range(max(0, k - n_rep), k)}

    def end_to_end():
        """Load every replica's state, take the K steps, read the states
        back; returns the host wall time of the whole sequence."""
        barrier(world)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        with torch.cuda.stream(h2d_stream):
            for r in range(n_rep):
                props[r].psik = [h.to(device, non_blocking=True) for h in psik_host]
                loaded[r].record(h2d_stream)
        for i in range(k):
            r = i % n_rep
            j = i // n_rep
            if j == 0:
                stream.wait_event(loaded[r])
            props[r].full_steps(1, pops_dev[r][j:j + 1])
            if j > 0:   # populations of the replica's previous step are final now
                pops_host[i - n_rep].copy_(pops_dev[r][j - 1], non_blocking=True)
            if last.get(r) == i:
                stepped[r].record(stream)
                with torch.cuda.stream(d2h_stream):
                    d2h_stream.wait_event(stepped[r])
                    for c in range(2):
                        out_host[r][c].copy_(props[r].psik[c], non_blocking=True)
        for r in range(n_rep):
            if r not in last:      # replicas that took no step (k < n_rep)
                with torch.cuda.stream(d2h_stream):
                    d2h_stream.wait_event(loaded[r])
                    for c in range(2):
                        out_host[r][c].copy_(props[r].psik[c], non_blocking=True)
        torch.cuda.synchronize()
        return time.perf_counter() - t0

    # once untimed, so that the side streams' device allocations are cached
    end_to_end()
    t_e2e = max_over_ranks(end_to_end(), world)
    h2d = n_rep * state_bytes / k
    d2h = (n_rep * state_bytes + 16 * (k - n_rep)) / k
    assert np.isfinite(out_host[0][0].numpy()).all()

    peak, peak_kind = measured_peaks()
    pass_bytes = 4 * n * n * elem         # read + write of both components
    dom_ms, dom_name = max((row_ms, 'row_kernel'), (col_ms, 'col_kernel'))
    achieved = pass_bytes / (dom_ms / 1e3) / 1e9
    step_bytes = 48 * n * n * elem        # 12 sweeps per full step (reference count)
    traffic = None
    traffic_note = None
    tpath = os.path.join(REPO, 'profiles', 'traffic.json')
    if os.path.exists(tpath):
        try:
            tj = json.load(open(tpath))
            traffic = tj.get(dom_name)
            traffic_note = tj.get('note')
        except ValueError:
            traffic = None

    # the other precisions on the same workload (fewer timed steps)
    modes = {}
    for mode in args.precision_modes:
        modes[mode] = precision_mode_rate(ps, mode, n, device, world,
                                          max(20, k // 5), args.warmup)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu, _ = cpu_reference_rate(ps)

    shapes0 = list(props[0].kernel_shapes)
    batched = None
    if args.batch_extra_steps > 0:
        del props
        b = measure_batched(world, rank, local, args.solves, args.batch_extra_steps,
                            args.warmup)
        batched = {'value': b['value'], 'unit': b['unit'],
                   'sequential_plain': b['sequential_plain']['value'],
                   'speedup_vs_sequential': b['speedup_vs_sequential'],
                   'solves': args.solves, 'steps': args.batch_extra_steps,
                   'what': 'the batched uneven ground states (sides 128-1024, '
                           'seeded parameters, complex64) advanced together by '
                           'PropagatorBatch (autotuned kernel shapes) against the '
                           'same solves one after another (bench.py --workload '
                           'batched_uneven runs it alone)'}
        if b.get('work_queue'):
            batched['work_queue'] = {k: b['work_queue'][k] for k in
                                     ('value', 'speedup_vs_sequential', 'what')}

    line = {
        'metric': METRIC, 'value': value, 'unit': UNIT, 'n_gpus': world,
        'steps': k, 'warmup': args.warmup,
        'ms_per_step': 1e3 * t_max / k * 1.0,
        'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
        'dtype': ('c64 (split-BF16 tensor-core DFT16 stages)' if args.tensor_core_dft
                  else 'c64 (fp32 butterflies; fp64 reductions)' if dtype == 64
                  else 'c128 (fp64)' if dtype == 128
                  else 'double-float (fp32 head + tail pairs, ~48 bits; fp64 reductions)'),
        'data': 'synthetic (seeded Thomas-Fermi + phase noise, 3000-step '
                'imaginary-time preparation)',
        'config': {'workload': f'raman_quench_{n}', 'grid': [n, n],
                   'time': 'real', 'dt': 1e-3, 'delta': 0.5, 'omega': 1.0,
                   'k_L': 3.0, 'g': [1000.0, 1000.0, 990.0],
                   'replicas_per_gpu': n_rep,
                   'kernel_shapes': shapes0,
                   'l2': f'inputs larger than L2: {n_rep} replica states of '
                         f'{state_bytes >> 20} MiB stepped round-robin',
                   'parallelism': f'replicas x{world}'},
        'grid_point_steps_per_s': value * n * n,
        'median_window': {'value': median_window, 'unit': UNIT, 'windows': n_win,
                          'what': 'median over equal windows of the timed steps, CUDA events'},
        'e2e': {'value': world * k / t_e2e, 'unit': UNIT,
                'h2d_bytes_per_step': h2d, 'd2h_bytes_per_step': d2h,
                'path': 'TensorPropagator.psik= (H2D from pinned memory, on a '
                        'side stream) / full_steps(1) per step with per-step '
                        'populations D2H / psik D2H after each replica\'s last '
                        'step (on a second side stream); events order the '
                        'copies against the steps, so the copies of one replica '
                        'overlap the steps of the others; the first step of each '
                        'replica after its psik load runs eagerly (the state '
                        'arrives in k-space form), the rest replay its captured '
                        'graph; the whole sequence runs once untimed first (the '
                        'side streams allocate their buffers), then timed'},
        'roofline': {'bound': 'hbm', 'kernel': dom_name,
                     'achieved': achieved, 'peak': peak, 'unit': 'GB/s',
                     'frac': achieved / peak, 'traffic': traffic,
                     'traffic_source': traffic_note,
                     'peak_kind': peak_kind,
                     'algorithmic_bytes': pass_bytes,
                     'col_pass_ms': col_ms, 'row_pass_ms': row_ms},
        'step_roofline': {'bytes_per_step': step_bytes,
                          'achieved': value / world * step_bytes / 1e9,
                          'peak': peak, 'unit': 'GB/s',
                          'frac': value / world * step_bytes / 1e9 / peak},
        'gpu_launches': 6 * k,
        'clocks': clk.summary(),
    }
    if modes:
        line['precision_modes'] = modes
    if batched is not None:
        line['batched_uneven'] = batched
    if cpu is not None:
        line['cpu_baseline'] = cpu
    if rank == 0:
        print(json.dumps(line))


# ---------------------------------------------------- batched uneven solves

def run_batched(args, world, rank, local):
    """Independent imaginary-time ground states with uneven grids (sides
    128..1024, dx = 0.125) and seeded parameters, complex64, dt = 0.02: all
    solves advanced together through ``PropagatorBatch`` (one CUDA graph with
    a branch per solve), against the plain single-solve drop-in stepping the
    same solves one after another.  Metric: aggregate grid-point-steps/s."""
    line = measure_batched(world, rank, local, args.solves, args.batch_steps,
                           args.warmup, not args.no_batch_autotune and not args.batch_queue,
                           args.breakdown, queue=args.batch_queue, sizes=args.batch_sizes)
    if rank == 0:
        print(json.dumps(line))


def measure_batched(world, rank, local, n_solves, k, warmup, autotune=True,
                    with_breakdown=False, queue=False, sizes=None):
    """The batched-uneven measurement (see ``run_batched``); returns its JSON
    line as a dict."""
    import torch
    from spinor_gpe import workloads
    from spinor_gpe.batch import PropagatorBatch
    from spinor_gpe.pspinor import pspinor as spin
    from spinor_gpe.pspinor import tensor_propagator as tprop
    from spinor_gpe.pspinor import tensor_tools as ttools
    torch.cuda.set_device(local)
    device = f'cuda:{local}'
    tmp = tempfile.mkdtemp(prefix='sgpe_batch_')
    extra = {} if sizes is None else {'sizes': tuple(sizes)}
    spins = workloads.batched_uneven(spin.PSpinor, ttools.fft_2d, tmp + '/',
                                     n_solves=n_solves, seed=4 + rank, **extra)
    props = [tprop.TensorPropagator(s, 0.02, k, device, time='imag', dtype=64)
             for s in spins]
    points = sum(s.psik[0].size for s in spins)
    stream = torch.cuda.current_stream()

    def timed(fn):
        barrier(world)
        torch.cuda.synchronize()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        fn()
        ev1.record(stream)
        torch.cuda.synchronize()
        barrier(world)
        return max_over_ranks(ev0.elapsed_time(ev1) / 1e3, world)

    # plain solves one after another (warm-up captures each plan's graphs)
    for p in props:
        p.full_steps(max(warmup, 9))
    t_seq = timed(lambda: [p.full_steps(k) for p in props])

    breakdown = None
    if with_breakdown:
        breakdown = {}
        kb = max(20, k // 10)
        for n in sorted({s.psik[0].shape[0] for s in spins}):
            cls = [p for p, s in zip(props, spins) if s.psik[0].shape[0] == n]
            t_one = timed(lambda: cls[0].full_steps(kb)) / kb
            cb = PropagatorBatch(cls)
            cb.full_steps(9)
            t_grp = timed(lambda: cb.full_steps(kb)) / kb
            cb.close()
            breakdown[str(n)] = {'solves': len(cls), 'one_alone_us': 1e6 * t_one,
                                 'sequential_us': 1e6 * t_one * len(cls),
                                 'batched_us': 1e6 * t_grp}

    batch = PropagatorBatch(props, queue=queue)
    tuned = None
    if autotune:
        # kernel shapes per size class for grouped stepping (set-up, untimed)
        t0 = time.perf_counter()
        tuned = batch.autotune()
        tune_s = time.perf_counter() - t0
        if breakdown is not None:
            for (_, _, nx), times in tuned.items():
                shapes = props[[p._shape[1] for p in props].index(nx)].kernel_shapes
                breakdown[str(nx)]['batched_tuned_us'] = times[shapes]
                breakdown[str(nx)]['tuned_shapes'] = list(shapes)
    batch.full_steps(max(warmup, 9))
    with ClockSampler(local) as clk:
        t_bat = timed(lambda: batch.full_steps(k))
    if queue:
        batch.check_device()
    for p in props[:4]:
        assert all(torch.isfinite(c).all().item() for c in p.psik)
    work_queue = None
    if not queue:
        # the same solves through the work-queue kernel (one persistent
        # launch per 8 steps), beside the grouped launches
        batch.close()
        qb = PropagatorBatch(props, queue=True)
        qb.full_steps(max(warmup, 9))
        t_q = timed(lambda: qb.full_steps(k))
        qb.check_device()
        qb.close()
        work_queue = {'value': world * points * k / t_q, 'unit': 'grid-point-steps/s',
                      'ms_per_step': 1e3 * t_q / k,
                      'speedup_vs_sequential': t_seq / t_q,
                      'what': 'PropagatorBatch(queue=True): one persistent cooperative '
                              'launch per 8 steps whose blocks claim pass items from a '
                              'device work queue'}
    sizes = {}
    for s in spins:
        sizes[s.psik[0].shape[0]] = sizes.get(s.psik[0].shape[0], 0) + 1
    value = world * points * k / t_bat
    seq = world * points * k / t_seq
    line = {
        'metric': 'grid-point-steps/s, batched uneven imaginary-time solves '
                  '(complex64)',
        'value': value, 'unit': 'grid-point-steps/s', 'n_gpus': world,
        'steps': k, 'warmup': max(warmup, 9), 'ms_per_step': 1e3 * t_bat / k,
        'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
        'dtype': 'c64 (fp32 butterflies; fp64 reductions)',
        'data': 'synthetic (seeded sizes and parameters, Thomas-Fermi + '
                'phase noise)',
        'config': {'workload': f'batched_uneven_{n_solves}',
                   'solves_per_gpu': n_solves, 'grid_sides': sizes,
                   'grid_points_per_gpu': points, 'dt': 0.02, 'time': 'imag',
                   'l2': f'inputs larger than L2: {points * 16 >> 20} MiB of '
                         f'state per GPU',
                   'parallelism': f'replicas x{world}'},
        'sequential_plain': {'value': seq, 'unit': 'grid-point-steps/s',
                             'what': 'the same solves, each advanced alone '
                                     'with TensorPropagator.full_steps (default '
                                     'kernel shapes)'},
        'speedup_vs_sequential': value / seq,
        'batch_kernel_shapes': (None if tuned is None else {
            f'{ny}x{nx}': list(props[[p._shape for p in props].index((ny, nx))].kernel_shapes)
            for (_, ny, nx) in tuned}),
        'batch_autotune_s': None if tuned is None else tune_s,
        'batch_mode': ('work queue: one persistent launch per graph (8 steps)' if queue
                       else 'grouped launches per size class, parallel graph branches'),
        'gpu_launches': (-(-k // 8) if queue else 6 * k * n_solves),
        'per_class_step_us': breakdown,
        'work_queue': work_queue,
        'clocks': clk.summary(),
    }
    batch.close()
    return line


# ------------------------------------------------------ served request stream

def run_served(args, world, rank, local):
    """A seeded Poisson request stream (70% ground states at 256^2/512^2 run
    to |dE| < 1e-8 per step or 3000 steps, 30% real-time quenches at 1024^2
    for 5000 steps; complex64) served by the continuous-batching loop under
    a 150 GB admission cap (requests set up on the device unless
    --host-setup), then the same requests solved one after another by the
    plain drop-in.  Reports latency percentiles (arrival to result),
    offered and served load, aggregate grid-point-steps/s of both."""
    import torch
    from spinor_gpe import serve, workloads
    torch.cuda.set_device(local)
    device = f'cuda:{local}'
    tmp = tempfile.mkdtemp(prefix='sgpe_serve_')
    stream = workloads.served_stream(rate=args.serve_rate,
                                     window=args.serve_window, seed=5 + rank)
    reqs = serve.requests_from_stream(stream, tmp + '/', device=device,
                                      device_setup=not args.host_setup)
    offered_max = sum(r.max_steps * r.grid_points for r in reqs)
    # warm-up: one small solve through the loop (library load, first graphs)
    serve.SolveServer(device, max_active=2).run(reqs[:1], realtime=False)
    barrier(world)
    torch.cuda.synchronize()
    srv = serve.SolveServer(device, hbm_cap=150e9, max_active=args.max_active,
                            max_queue_s=args.serve_max_queue)
    with ClockSampler(local) as clk:
        res = srv.run(reqs, realtime=True)
    st = dict(srv.stats)
    wall = max_over_ranks(st['wall_s'], world)
    barrier(world)
    # sequential baseline: the served requests (or a seeded sample of them),
    # each solved alone with the same stopping rules
    served_ids = [r.rid for r in res if not r.shed]
    if args.serve_seq_sample and args.serve_seq_sample < len(served_ids):
        rng = np.random.default_rng(11 + rank)
        served_ids = sorted(rng.choice(served_ids, args.serve_seq_sample, replace=False).tolist())
    by_id = {r.rid: r for r in reqs}
    sample = [by_id[i] for i in served_ids]
    seq, t_seq, t_seq_wall = serve.run_sequential(sample, device, with_wall=True)
    t_seq = max_over_ranks(t_seq, world)
    t_seq_wall = max_over_ranks(t_seq_wall, world)
    res_by_id = {r.rid: r for r in res}
    same = all((res_by_id[b.rid].steps, res_by_id[b.rid].converged) == (b.steps, b.converged)
               for b in seq)
    seq_gps = sum(b.steps * b.grid_points for b in seq)
    gps = st['grid_point_steps']
    kinds = {}
    for r in res:
        if r.shed:
            continue
        k = kinds.setdefault(f'{r.kind}_{int(round(r.grid_points ** 0.5))}',
                             {'n': 0, 'steps': 0, 'converged': 0, 'lat': []})
        k['n'] += 1
        k['steps'] += r.steps
        k['converged'] += int(r.converged)
        k['lat'].append(r.latency)
    for k in kinds.values():
        lat = np.array(k.pop('lat'))
        k['p50_ms'] = float(np.percentile(lat, 50) * 1e3)
        k['p99_ms'] = float(np.percentile(lat, 99) * 1e3)
    line = {
        'metric': 'served request stream: p50/p99 latency (ms) and aggregate '
                  'grid-point-steps/s (complex64)',
        'value': world * gps / wall, 'unit': 'grid-point-steps/s',
        'p50_ms': st['p50_ms'], 'p99_ms': st['p99_ms'],
        'n_gpus': world, 'steps': len(res), 'warmup': 1,
        'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
        'dtype': 'c64 (fp32 butterflies; fp64 reductions)',
        'data': 'synthetic (seeded Poisson stream; Thomas-Fermi starts)',
        'config': {'workload': f'served_stream_{args.serve_rate:g}rps_'
                               f'{args.serve_window:g}s',
                   'requests': len(res), 'rate_per_s': args.serve_rate,
                   'window_s': args.serve_window, 'hbm_cap_bytes': 150e9,
                   'max_active': args.max_active,
                   'setup': 'host PSpinor' if args.host_setup else
                            'DeviceSpinor (set-up kernels on the GPU)',
                   'parallelism': f'replicas x{world}'},
        'offered': {'requests_per_s': args.serve_rate,
                    'grid_point_steps_upper_bound': offered_max,
                    'grid_point_steps_per_s_upper_bound':
                        offered_max / args.serve_window},
        'served': {'grid_point_steps': gps, 'wall_s': wall,
                   'requests_served': st['served'], 'requests_shed': st['shed'],
                   'max_queue_s': args.serve_max_queue,
                   'requests_per_s': st['served'] / wall,
                   'peak_active': st['peak_active'],
                   'peak_admitted_bytes': st['peak_admitted_bytes'],
                   'by_kind': kinds,
                   'host_loop': st['host']},
        'sequential_plain': {'value': world * seq_gps / t_seq,
                             'unit': 'grid-point-steps/s',
                             'device_s': t_seq, 'requests': len(seq),
                             'with_host_setup': {'value': world * seq_gps / t_seq_wall,
                                                 'wall_s': t_seq_wall},
                             'what': 'served requests (all, or a seeded sample) with '
                                     'the same stopping rules, each solved alone by '
                                     'the plain drop-in: device time of the stepping '
                                     '(host set-up excluded), and host wall time '
                                     'including each set-up'},
        'speedup_vs_sequential': (gps / wall) / (seq_gps / t_seq),
        'speedup_vs_sequential_with_setup': (gps / wall) / (seq_gps / t_seq_wall),
        'same_steps_alone_and_in_mix': same,
        'clocks': clk.summary(),
    }
    if rank == 0:
        print(json.dumps(line))


# ------------------------------------------------------------ reference arm

def run_reference(args, world, rank, local):
    """The original algorithm on the host cores (rank 0 only)."""
    if rank != 0:
        return
    import torch
    tmp = tempfile.mkdtemp(prefix='sgpe_ref_')
    has_gpu = torch.cuda.is_available()
    # no preparation here: this arm runs none of the native kernels, and the
    # step cost does not depend on the state's values
    ps = build_problem(tmp, args.n, 0, None)
    cpu, inp = cpu_reference_rate(ps, budget_s=min(60.0, 3.0 * max(args.steps, 1)),
                                  max_steps=max(args.steps, 2))
    line = {
        'impl': 'reference', 'metric': METRIC, 'value': cpu['value'],
        'unit': UNIT, 'n_gpus': world, 'steps': args.steps,
        'warmup': args.warmup, 'ms_per_step': 1e3 / cpu['value'],
        'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
        'dtype': 'c64', 'data': 'synthetic',
        'config': {'workload': f'raman_quench_{args.n}',
                   'grid': [args.n, args.n], 'time': 'real', 'dt': 1e-3},
        'cpu_baseline': cpu,
        'e2e': {'value': cpu['value'], 'unit': UNIT, 'h2d_bytes_per_step': 0,
                'd2h_bytes_per_step': 0},
    }
    if has_gpu:
        line['torch_cuda_same_gpu'] = {
            'value': torch_cuda_reference_rate(inp), 'unit': UNIT,
            'what': 'original algorithm on torch CUDA (torch.fft + ATen, with '
                    'its per-sub-step host synchronisations), complex64'}
        line['torch_cuda_same_gpu_c128'] = {
            'value': torch_cuda_reference_rate(inp, steps=10, dtype=128), 'unit': UNIT,
            'what': 'the same in complex128 (the original\'s default precision)'}
    print(json.dumps(line))


def main():
    args = parse()
    world, rank, local = dist_setup()
    if args.impl == 'reference':
        run_reference(args, world, rank, local)
    elif args.workload == 'batched_uneven':
        run_batched(args, world, rank, local)
    elif args.workload == 'served':
        run_served(args, world, rank, local)
    else:
        run_native(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == '__main__':
    main()
