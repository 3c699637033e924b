"""Runs with one process per GPU (bench.py under torchrun): the path is not
sharded, ranks only agree on timings.  Two gloo ranks on the CPU check that
every rank receives the slowest rank's time and that the whole-job rate uses
it (the same helpers bench.py calls with NCCL)."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from igap4_gb300.replicas import job_rate, max_over_ranks

    ms = 10.0 + 5.0 * rank  # rank 1 is the slower replica
    m = max_over_ranks(ms)
    dist.barrier()
    q.put((rank, m, job_rate(1000, m, world)))
    dist.destroy_process_group()


def test_replicas_report_the_slowest_rank():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
    assert all(p.exitcode == 0 for p in procs)
    assert [o[1] for o in out] == [15.0, 15.0]
    assert out[0][2] == out[1][2] == 2 * 1000 / 15e-3


def test_single_process_is_its_own_maximum():
    from igap4_gb300.replicas import job_rate, max_over_ranks

    assert max_over_ranks(7.5) == 7.5
    assert job_rate(131072, 256.0, 1) == 131072 / 0.256
