"""The N > 1 host path of bench.py on CPU ranks (gloo, world size 2).

Solves are never split across GPUs ("replicas only"): the multi-rank code
is the barrier, the maximum of the timed region over ranks, and rank 0 alone
printing (and, for the reference arm, alone doing the work)."""
import json
import os
import socket
import subprocess
import sys

import torch
import torch.multiprocessing as mp

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port),
                      RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, REPO)
    import bench
    w, r, _ = bench.dist_setup()
    assert (w, r) == (world, rank)
    bench.barrier(w)
    out[rank] = bench.max_over_ranks(1.5 + rank, w)
    import torch.distributed as dist
    dist.destroy_process_group()


def test_max_over_ranks_gloo_world_2():
    ctx = mp.get_context('spawn')
    with ctx.Manager() as m:
        out = m.dict()
        mp.start_processes(_worker, args=(2, _free_port(), out), nprocs=2,
                           start_method='spawn')
        assert dict(out) == {0: 2.5, 1: 2.5}


def test_reference_arm_two_ranks_prints_one_line():
    env = dict(os.environ, CUDA_VISIBLE_DEVICES='')
    cmd = [sys.executable, '-m', 'torch.distributed.run', '--nnodes=1',
           '--nproc-per-node', '2', '--master-addr', '127.0.0.1',
           '--master-port', str(_free_port()), 'bench.py', '--impl',
           'reference', '--gpus', '2', '--grid', '64', '--steps', '2',
           '--warmup', '1']
    r = subprocess.run(cmd, cwd=REPO, env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith('{')]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d['impl'] == 'reference' and d['n_gpus'] == 2
    assert d['cpu_baseline']['kind'] == 'port' and d['value'] > 0
    assert d['e2e']['h2d_bytes_per_step'] == 0
