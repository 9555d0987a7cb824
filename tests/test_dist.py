"""The N > 1 host path of bench.py on CPU ranks (gloo, world size 2): the
barrier and max-over-ranks timing, and the reference arm under torchrun,
where rank 0 alone runs and prints one line."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group('gloo', init_method=f'tcp://127.0.0.1:{port}',
                            rank=rank, world_size=world)
    d = bench.Dist(world)
    d.barrier()
    q.put((rank, d.allmax(1.5 + rank), d.allmax(-float(rank))))
    d.barrier()
    dist.destroy_process_group()


def test_dist_barrier_and_allmax_two_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == [(0, 2.5, 0.0), (1, 2.5, 0.0)]


@pytest.mark.timeout(300)
def test_reference_arm_under_torchrun_prints_once():
    pytest.importorskip('torch')
    env = dict(os.environ, OMP_NUM_THREADS='2')
    cmd = [sys.executable, '-m', 'torch.distributed.run', '--nnodes=1',
           '--nproc-per-node', '2', '--master-addr', '127.0.0.1',
           '--master-port', str(_free_port()), 'bench.py', '--impl',
           'reference', '--gpus', '2', '--steps', '1', '--warmup', '1',
           '--cpu-sample', '3']
    out = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True,
                         text=True, timeout=280)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith('{')]
    assert len(lines) == 1
    rec = json.loads(lines[0])
    assert rec['impl'] == 'reference' and rec['value'] > 0
    assert rec['e2e']['h2d_bytes_per_step'] == 0
