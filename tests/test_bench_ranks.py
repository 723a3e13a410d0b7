"""bench.py's host logic on the CPU: the multi-rank path (two gloo ranks stand for two replicas) and the reference
arm's JSON line.

Under torchrun every rank runs an independent replica of the workload. The job's time is the slowest rank's (a MAX
all-reduce), its rate counts the units of all ranks, and the reference arm runs on rank 0 alone.
"""

import contextlib
import io
import multiprocessing as mp
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def _replica(rank, ws, port, q):
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench as b
    dist.init_process_group('gloo', rank=rank, world_size=ws)
    try:
        t = b.slowest_rank(10.0 + 5.0 * rank, ws, 'cpu')   # rank r's timed region: 10 + 5 r ms
        q.put((rank, t, b.whole_job_rate(ws, 1_000_000, 1024, t)))
    finally:
        dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank_and_all_ranks_units():
    ws, port = 2, _free_port()
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    procs = [ctx.Process(target=_replica, args=(r, ws, port, q)) for r in range(ws)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in range(ws))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, rate in got:
        assert t == 15.0                                   # every rank sees the slowest rank's time
        assert rate == pytest.approx(2 * 1_000_000 * 1024 / 15e-3 / 1e9)


def test_one_rank_needs_no_process_group():
    assert bench.slowest_rank(3.5, 1) == 3.5
    assert bench.whole_job_rate(1, 12_582_912, 1024, 4.0) == pytest.approx(12_582_912 * 1024 / 4e-3 / 1e9)


def test_reference_arm_runs_on_rank_zero_only():
    class Args:
        workload, n = 'hex32', None
    out = io.StringIO()
    with contextlib.redirect_stdout(out):
        bench.reference_arm(Args(), 2, 1)
    assert out.getvalue() == ''


def test_reference_arm_prints_the_contract_line():
    """`bench.py --impl reference` (the reference's CPU formulation, the oracle port) prints one JSON line with the
    bench keys, the reference tag, its CPU baseline and an end-to-end figure with no device copies."""
    import json
    import subprocess
    out = subprocess.run([sys.executable, os.path.join(ROOT, 'bench.py'), '--impl', 'reference', '--steps', '1',
                          '--warmup', '0', '--n', '20000'], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith('{')]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ('metric', 'value', 'unit', 'n_gpus', 'steps', 'warmup', 'ms_per_step', 'higher_is_better', 'scaling',
              'vs_baseline', 'dtype', 'data', 'config', 'cpu_baseline', 'e2e'):
        assert k in d, k
    assert d['impl'] == 'reference' and d['metric'] == bench.METRIC and d['higher_is_better'] is True
    assert d['value'] > 0 and d['cpu_baseline']['kind'] == 'port' and d['cpu_baseline']['cores'] >= 1
    assert d['e2e'] == {'value': d['value'], 'unit': d['unit'], 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}
