"""The multi-rank logic of bench.py on the CPU: two gloo ranks stand for two replicas.

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
