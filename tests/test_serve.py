"""The request loop: arrival streams and footprints on the CPU; on the GPU,
every result is the same alone and in the mix, admission respects the slot
and memory limits."""
import numpy as np
import pytest
import torch

from spinor_gpe import serve, workloads


def test_served_stream_is_seeded_and_mixed():
    a = workloads.served_stream(rate=200, window=2.0, seed=5)
    b = workloads.served_stream(rate=200, window=2.0, seed=5)
    assert a == b
    t = np.array([d['arrival'] for d in a])
    assert np.all(np.diff(t) > 0) and t[-1] < 2.0
    assert 300 < len(a) < 500                      # Poisson(400)
    kinds = [d['kind'] for d in a]
    assert 0.6 < kinds.count('ground') / len(a) < 0.8
    for d in a:
        if d['kind'] == 'ground':
            assert d['n'] in (256, 512) and d['tol'] == 1e-8
            assert d['max_steps'] == 3000 and d['time'] == 'imag'
            assert 0.5 <= d['lam'] <= 2 and 100 <= d['g'][0] <= 2000
            assert d['g'][1] == 0.995 * d['g'][0] and d['g'][2] == 0.99 * d['g'][0]
        else:
            assert d['n'] == 1024 and d['max_steps'] == 5000
            assert d['time'] == 'real' and 0.1 <= d['delta'] <= 1.0


def test_poisson_arrivals_rate():
    t = serve.poisson_arrivals(200.0, 50.0, 3)
    assert abs(len(t) / 50.0 - 200.0) < 10.0


def test_footprint():
    assert serve.solve_footprint(1024, 1024, 64) == 8 * 1024 * 1024 * 8 + (2 << 20)
    assert serve.solve_footprint(256, 256, 128) == 8 * 256 * 256 * 16 + (2 << 20)


def _small_requests(tmp_path):
    from spinor_gpe.pspinor import pspinor as spin
    from spinor_gpe.pspinor import tensor_propagator as tprop
    from spinor_gpe.pspinor import tensor_tools as ttools
    specs = [('ground', 64, 0.02, 120, 1e-4), ('ground', 128, 0.02, 90, 1e-9),
             ('quench', 128, 1e-3, 70, None), ('ground', 192, 0.02, 60, 1e-9),
             ('quench', 64, 1e-3, 50, None)]
    reqs = []
    for i, (kind, n, dt, steps, tol) in enumerate(specs):
        def make(i=i, n=n, dt=dt, steps=steps, tol=tol):
            ps = workloads.build(spin.PSpinor, ttools.fft_2d,
                                 str(tmp_path / f'r{i}') + '/', nx=n, ny=n,
                                 half_x=n / 16, half_y=n / 16,
                                 g=(500.0 + 100 * i, 497.0, 495.0), lam=1.1,
                                 omega=0.7, k_l=3.0, delta=0.2, seed=40 + i)
            return tprop.TensorPropagator(ps, dt, steps, 'cuda',
                                          time='imag' if tol else 'real',
                                          dtype=64)
        reqs.append(serve.SolveRequest(
            rid=i, arrival=0.001 * i, make=make,
            footprint=serve.solve_footprint(n, n, 64), max_steps=steps,
            tol=tol, chunk=16, grid_points=n * n, kind=kind))
    return reqs


@pytest.mark.gpu
def test_results_same_alone_and_in_the_mix(tmp_path):
    reqs = _small_requests(tmp_path)
    mix = serve.SolveServer(max_active=3, keep_psik=True)
    together = mix.run(reqs, realtime=True)
    assert mix.stats['peak_active'] <= 3
    # the loop's own accounting: one submission per chunk of every solve
    host = mix.stats['host']
    assert host['chunks'] == sum(-(-got.steps // req.chunk) for req, got in zip(reqs, together))
    assert 0.0 <= host['enqueue_s'] <= host['busy_s']
    assert 0.0 <= host['process_s'] <= host['busy_s']
    assert host['busy_s'] + host['asleep_s'] == pytest.approx(mix.stats['wall_s'])
    for req, got in zip(reqs, together):
        alone = serve.SolveServer(max_active=1, keep_psik=True).run([req])[0]
        assert (alone.steps, alone.converged) == (got.steps, got.converged)
        assert alone.energy == got.energy
        for a, b in zip(alone.psik, got.psik):
            assert torch.equal(a, b)
        assert got.finished >= got.admitted >= got.arrival - 1e-9
    # the loop's stopping rules: tolerance or step count
    for req, got in zip(reqs, together):
        if got.converged:
            assert got.d_energy < req.tol and got.steps <= req.max_steps
        else:
            assert got.steps == req.max_steps
    assert together[2].steps == 70 and not together[2].converged


@pytest.mark.gpu
def test_admission_respects_memory_cap(tmp_path):
    reqs = _small_requests(tmp_path)
    cap = 2.5 * serve.solve_footprint(128, 128, 64)
    reqs = [r for r in reqs if r.footprint <= cap]
    srv = serve.SolveServer(max_active=8, hbm_cap=cap)
    res = srv.run(reqs, realtime=False)
    assert srv.stats['peak_admitted_bytes'] <= cap
    assert len(res) == len(reqs)
    seq, t = serve.run_sequential(reqs)
    assert t > 0
    for a, b in zip(sorted(res, key=lambda r: r.rid), seq):
        assert (a.steps, a.energy) == (b.steps, b.energy)


def test_oversize_request_rejected():
    srv = serve.SolveServer(hbm_cap=1e6)
    req = serve.SolveRequest(0, 0.0, lambda: None, int(2e6), 10)
    with pytest.raises(ValueError):
        srv.run([req])


@pytest.mark.gpu
def test_served_requests_with_device_set_up(tmp_path):
    stream = workloads.served_stream(rate=200, window=0.02, seed=9,
                                     ground_sizes=(64,), quench_size=64)
    for d in stream:
        d['max_steps'] = 30
    reqs = serve.requests_from_stream(stream, str(tmp_path) + '/', device_setup=True,
                                      ground_chunk=10, quench_chunk=10)
    res = serve.SolveServer(max_active=4).run(reqs, realtime=False)
    assert len(res) == len(reqs) and all(r.steps > 0 for r in res)
    assert all(np.isfinite(r.energy) for r in res)


@pytest.mark.gpu
def test_requests_past_the_queue_limit_are_shed(tmp_path):
    """With one slot and a queue-time limit shorter than one request's
    set-up, the requests behind the first are shed (no steps, flagged), and
    the one served matches the same request served alone."""
    import time as _time
    reqs = _small_requests(tmp_path)
    slow = []
    for r in reqs:
        def make(m=r.make):
            _time.sleep(0.3)             # a set-up longer than the queue limit
            return m()
        slow.append(serve.SolveRequest(r.rid, 0.0, make, r.footprint, r.max_steps,
                                       r.tol, r.chunk, r.grid_points, r.kind))
    srv = serve.SolveServer(max_active=1, max_queue_s=0.1)
    res = srv.run(slow, realtime=True)
    assert srv.stats['served'] == 1 and srv.stats['shed'] == len(slow) - 1
    assert not res[0].shed and res[0].steps > 0
    assert all(r.shed and r.steps == 0 for r in res[1:])
    alone = serve.SolveServer(max_active=1).run([reqs[0]])[0]
    assert (alone.steps, alone.energy) == (res[0].steps, res[0].energy)
