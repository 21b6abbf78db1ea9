"""A request loop that serves independent solves on one GPU with continuous
batching.

Requests (ground states run to an energy tolerance, real-time quenches run
for a step count) arrive over time.  The loop admits each one as soon as a
slot and device memory allow, keeps its wavefunction and operators resident
on the GPU while it runs, advances every admitted solve in chunks of steps on
its own CUDA stream, so the chunks of different solves overlap on the device,
and retires each solve when its own stopping rule says so.  Requests that
arrive while others run join the mix at once; a finished solve frees its slot
and memory for the next one.

A solve's arithmetic depends only on the solve: every chunk is the same
sequence of native calls whether the solve runs alone or among others, so a
result is the same in both cases (bit for bit: the kernels are deterministic
and the solves share no device memory).

Stopping rules
  * ``tol``  (imaginary time): after every chunk of ``chunk`` steps the FP64
    energy is evaluated after the chunk's last two steps; the solve retires
    when |E(n) - E(n-1)| < tol, or at ``max_steps``.
  * no ``tol`` (real time): the solve runs ``max_steps`` steps.

Load shedding: with ``max_queue_s`` a request that has waited longer than
that for admission is rejected (reported with ``shed=True`` and no steps)
instead of joining an ever longer queue, so an overloaded stream keeps a
bounded latency for the requests it serves.

Host set-up (building a propagator: FP64 operators on the host, plan
creation and uploads) runs on a helper thread, so the loop that feeds the GPU
never waits on it.  Freeing device memory synchronises the device, so a
retired solve's plan is parked rather than destroyed; parked plans are freed
only when admission needs their memory, and at the end of the run.
"""
import collections
import concurrent.futures
import dataclasses
import time
from typing import Callable, Optional

import numpy as np
import torch


def solve_footprint(ny, nx, bits):
    """Device bytes one admitted solve holds: the plan's state, transform
    scratch and energy buffers (6 fields of two components), the cached
    k-space spinor (2 fields) and about 2 MiB of tables and partial sums."""
    return 8 * ny * nx * (bits // 8) + (2 << 20)


@dataclasses.dataclass
class SolveRequest:
    """One solve.  ``make`` builds its propagator (a ``TensorPropagator`` or
    an object with its ``full_steps`` / ``energy_to`` / ``psik`` interface);
    it is called once, at admission, on a helper thread."""
    rid: int
    arrival: float              # seconds after the stream starts
    make: Callable[[], object]
    footprint: int              # device bytes while admitted
    max_steps: int
    tol: Optional[float] = None
    chunk: int = 100
    grid_points: int = 0
    kind: str = ''


@dataclasses.dataclass
class SolveResult:
    rid: int
    kind: str
    steps: int
    converged: bool
    energy: Optional[float]
    d_energy: Optional[float]
    arrival: float
    admitted: float
    finished: float
    grid_points: int
    psik: Optional[list] = None
    shed: bool = False

    @property
    def latency(self):
        return self.finished - self.arrival


class _Solve:
    """A solve in flight: its propagator, stream and stopping rule."""

    def __init__(self, req, prop, stream, device):
        self.req = req
        self.prop = prop
        self.stream = stream
        self.steps = 0
        self.e_prev = None          # energy after the previous chunk
        self.d_energy = None
        self.energy = None
        self.done = False
        self.converged = False
        self.n_last = 0
        self.admitted = 0.0
        with torch.cuda.stream(stream):
            self.dev = torch.empty((2, 10), dtype=torch.float64, device=device)
        self.host = torch.empty((2, 10), dtype=torch.float64).pin_memory()
        self.event = torch.cuda.Event()

    def enqueue(self):
        """Queue the next chunk (and its energy evaluations) on the stream."""
        req = self.req
        n = min(req.chunk, req.max_steps - self.steps)
        self.n_last = n
        with torch.cuda.stream(self.stream):
            if req.tol is not None and n >= 2:
                self.prop.full_steps(n - 1)
                self.prop.energy_to(self.dev[0])
                self.prop.full_steps(1)
                self.prop.energy_to(self.dev[1])
            else:
                if n > 0:
                    self.prop.full_steps(n)
                if req.tol is not None or self.steps + n >= req.max_steps:
                    self.prop.energy_to(self.dev[1])
            self.host.copy_(self.dev, non_blocking=True)
            self.event.record(self.stream)

    def ready(self):
        return self.event.query()

    def process(self):
        """Read the finished chunk's results; decide whether to stop."""
        req = self.req
        n = self.n_last
        self.steps += n
        vals = self.host.numpy()
        if req.tol is not None:
            e1 = float(vals[1, 4])
            e0 = float(vals[0, 4]) if n >= 2 else self.e_prev
            self.energy = e1
            if e0 is not None:
                self.d_energy = abs(e1 - e0)
                if self.d_energy < req.tol:
                    self.converged = True
            self.e_prev = e1
        elif self.steps >= req.max_steps:
            self.energy = float(vals[1, 4])
        self.done = self.converged or self.steps >= req.max_steps
        return self.done


class SolveServer:
    """Continuous-batching loop over ``SolveRequest`` objects on one GPU.

    ``hbm_cap``: device bytes the admitted solves may hold together;
    ``max_active``: solves admitted at once (one CUDA stream each);
    ``keep_psik``: return each final k-space spinor (device tensors);
    ``build_workers``: helper threads building admitted solves;
    ``max_queue_s``: shed requests that waited longer than this for admission
    (None: never shed).
    """

    def __init__(self, device='cuda', hbm_cap=150e9, max_active=64,
                 keep_psik=False, build_workers=4, clock=time.perf_counter,
                 max_queue_s=None):
        self.device = torch.device(device)
        self.max_queue_s = None if max_queue_s is None else float(max_queue_s)
        self.hbm_cap = float(hbm_cap)
        self.max_active = int(max_active)
        self.keep_psik = keep_psik
        self.build_workers = int(build_workers)
        self.clock = clock
        self._streams = None        # created on the first run
        self.stats = {}

    # helper-thread work ------------------------------------------------
    def _build(self, req):
        torch.cuda.set_device(self.device)
        prop = req.make()
        torch.cuda.current_stream(self.device).synchronize()
        return prop

    def _release(self, parked):
        """Destroy parked solves (their plans free device memory)."""
        for solve in parked:
            solve.stream.synchronize()
            solve.prop = None
            solve.dev = None

    def run(self, requests, realtime=True):
        """Serve ``requests`` (any order; each becomes visible at its
        ``arrival`` time when ``realtime``, else all at once) and return the
        results in request order.  Fills ``self.stats``; its ``host`` entry
        gives the loop's own cost: chunks submitted, seconds spent queueing
        them (``enqueue_s``) and reading their results (``process_s``),
        seconds asleep waiting for the GPU (``asleep_s``) and the longest
        loop iteration spent working, during which no finished solve is
        resubmitted."""
        for r in requests:
            if r.footprint > self.hbm_cap:
                raise ValueError(f'request {r.rid} needs {r.footprint} bytes, '
                                 f'more than the cap {self.hbm_cap:.0f}')
        if self.device.index is None:
            self.device = torch.device('cuda', torch.cuda.current_device())
        torch.cuda.set_device(self.device)
        if self._streams is None:
            self._streams = [torch.cuda.Stream(device=self.device)
                             for _ in range(self.max_active)]
        order = sorted(requests, key=lambda r: (r.arrival, r.rid))
        arrivals = collections.deque(order)
        pending = collections.deque()
        free_streams = list(self._streams)
        building = {}               # future -> (req, stream, admit time)
        active = []
        results = {}
        used = 0.0                  # bytes of admitted solves
        parked, parked_bytes = [], 0.0
        peak_used = 0.0
        peak_active = 0
        releases = 0
        pool = concurrent.futures.ThreadPoolExecutor(
            max_workers=self.build_workers)
        # host-side cost of the loop: time in chunk submission and result
        # reads, time asleep waiting for the GPU, longest busy iteration
        t_enqueue = t_process = t_sleep = 0.0
        chunks = iterations = 0
        busy_max = 0.0
        t0 = self.clock()
        while arrivals or pending or building or active:
            iterations += 1
            t_iter = self.clock()
            now = t_iter - t0
            while arrivals and (not realtime or arrivals[0].arrival <= now):
                pending.append(arrivals.popleft())
            if self.max_queue_s is not None:
                while pending and now - pending[0].arrival > self.max_queue_s:
                    req = pending.popleft()
                    results[req.rid] = SolveResult(
                        req.rid, req.kind, 0, False, None, None, req.arrival,
                        now, now, req.grid_points, None, shed=True)
            # admission: first come, first served, under slots and memory
            if (pending and free_streams and parked
                    and used + parked_bytes + pending[0].footprint > self.hbm_cap):
                self._release(parked)
                parked, parked_bytes = [], 0.0
                releases += 1
            while (pending and free_streams
                   and used + parked_bytes + pending[0].footprint <= self.hbm_cap):
                req = pending.popleft()
                used += req.footprint
                peak_used = max(peak_used, used)
                fut = pool.submit(self._build, req)
                building[fut] = (req, free_streams.pop(), now)
            progressed = False
            for fut in [f for f in building if f.done()]:
                req, stream, t_adm = building.pop(fut)
                solve = _Solve(req, fut.result(), stream, self.device)
                solve.admitted = t_adm
                t_a = self.clock()
                solve.enqueue()
                t_enqueue += self.clock() - t_a
                chunks += 1
                active.append(solve)
                progressed = True
            peak_active = max(peak_active, len(active))
            still = []
            for s in active:
                if not s.ready():
                    still.append(s)
                    continue
                progressed = True
                t_a = self.clock()
                finished = s.process()
                t_process += self.clock() - t_a
                if finished:
                    t_fin = self.clock() - t0
                    psik = None
                    if self.keep_psik:
                        with torch.cuda.stream(s.stream):
                            psik = [p.clone() for p in s.prop.psik]
                        s.stream.synchronize()
                    results[s.req.rid] = SolveResult(
                        s.req.rid, s.req.kind, s.steps, s.converged, s.energy,
                        s.d_energy, s.req.arrival, s.admitted, t_fin,
                        s.req.grid_points, psik)
                    used -= s.req.footprint
                    parked.append(s)
                    parked_bytes += s.req.footprint
                    free_streams.append(s.stream)
                else:
                    t_a = self.clock()
                    s.enqueue()
                    t_enqueue += self.clock() - t_a
                    chunks += 1
                    still.append(s)
            active = still
            t_a = self.clock()
            busy_max = max(busy_max, t_a - t_iter)
            if not progressed:
                if not active and not building and arrivals and realtime:
                    time.sleep(max(0.0, min(arrivals[0].arrival - now, 0.01)))
                else:
                    time.sleep(20e-6)
                t_sleep += self.clock() - t_a
        torch.cuda.synchronize(self.device)
        wall = self.clock() - t0
        pool.shutdown(wait=True)
        self._release(parked)
        res = [results[r.rid] for r in requests]
        done = [r for r in res if not r.shed]
        lat = np.array([r.latency for r in done]) if done else np.zeros(1)
        gps = sum(r.steps * r.grid_points for r in res)
        self.stats = {'requests': len(res), 'served': len(done),
                      'shed': len(res) - len(done), 'wall_s': wall,
                      'grid_point_steps': gps,
                      'grid_point_steps_per_s': gps / wall if wall > 0 else 0.0,
                      'p50_ms': float(np.percentile(lat, 50) * 1e3),
                      'p99_ms': float(np.percentile(lat, 99) * 1e3),
                      'peak_active': peak_active,
                      'peak_admitted_bytes': peak_used,
                      'parked_releases': releases,
                      'host': {'chunks': chunks, 'iterations': iterations,
                               'enqueue_s': t_enqueue, 'process_s': t_process,
                               'asleep_s': t_sleep,
                               'busy_s': wall - t_sleep,
                               'longest_busy_iteration_ms': 1e3 * busy_max}}
        return res


def run_sequential(requests, device='cuda', with_wall=False):
    """The same requests solved one after another with the plain propagator
    and the same stopping rules, on the current stream.  Returns the results
    and the device time of the stepping (set-up excluded), in seconds; with
    ``with_wall`` also the host wall time including each request's set-up."""
    device = torch.device(device)
    if device.index is None:
        device = torch.device('cuda', torch.cuda.current_device())
    torch.cuda.set_device(device)
    stream = torch.cuda.current_stream(device)
    total = 0.0
    out = []
    t_wall = time.perf_counter()
    for req in sorted(requests, key=lambda r: (r.arrival, r.rid)):
        prop = req.make()
        torch.cuda.synchronize(device)
        s = _Solve(req, prop, stream, device)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        while True:
            s.enqueue()
            s.event.synchronize()
            if s.process():
                break
        e1.record(stream)
        e1.synchronize()
        total += e0.elapsed_time(e1) / 1e3
        out.append(SolveResult(req.rid, req.kind, s.steps, s.converged,
                               s.energy, s.d_energy, req.arrival, 0.0, 0.0,
                               req.grid_points))
        del s, prop
    torch.cuda.synchronize(device)
    if with_wall:
        return out, total, time.perf_counter() - t_wall
    return out, total


def poisson_arrivals(rate, window, seed):
    """Seeded Poisson arrival times (seconds) in [0, window)."""
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= window:
            return out
        out.append(t)



def requests_from_stream(stream, path, device='cuda', dtype=64,
                         ground_chunk=100, quench_chunk=500, device_setup=False):
    """``SolveRequest`` objects for ``workloads.served_stream`` descriptions:
    each builds its PSpinor (``device_setup``: a ``DeviceSpinor``, set up on
    the GPU) and drop-in propagator when admitted."""
    from . import workloads
    from .pspinor import pspinor as spin
    from .pspinor import tensor_propagator as tprop
    from .pspinor import tensor_tools as ttools
    bits = 64 if dtype in (64, torch.complex64) else 128

    def maker(d):
        def make():
            if device_setup:
                ps = workloads.request_spin_device(path, d, device=device, dtype=bits)
            else:
                ps = workloads.request_spin(spin.PSpinor, ttools.fft_2d, path, d)
            return tprop.TensorPropagator(ps, d['dt'], d['max_steps'], device,
                                          time=d['time'], dtype=bits)
        return make
    out = []
    for d in stream:
        n = d['n']
        out.append(SolveRequest(
            rid=d['rid'], arrival=d['arrival'], make=maker(d),
            footprint=solve_footprint(n, n, bits), max_steps=d['max_steps'],
            tol=d['tol'],
            chunk=ground_chunk if d['tol'] is not None else quench_chunk,
            grid_points=n * n, kind=d['kind']))
    return out
