"""Replica runs over several ranks (acvd_gb300.replicas), as two gloo ranks on CPU: the
timing reduces to the slowest rank's, the throughput counts every rank's units."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, ws, port, out):
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(ws),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    from acvd_gb300 import replicas
    replicas.init("gloo")
    assert replicas.world() == (ws, rank, rank)
    ms = replicas.max_over_ranks(10.0 + 5.0 * rank)       # rank 1 is the slowest replica
    rate = replicas.aggregate_rate(1000.0, ms)
    replicas.barrier()
    out.put((rank, ms, rate))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_gloo_replicas():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [15.0, 15.0]
    assert all(abs(r[2] - 2 * 1000.0 / 0.015) < 1e-6 for r in res)


def test_single_rank_needs_no_group(monkeypatch):
    for k in ("RANK", "LOCAL_RANK", "WORLD_SIZE"):
        monkeypatch.delenv(k, raising=False)
    from acvd_gb300 import replicas
    replicas.init("gloo")
    assert replicas.world() == (1, 0, 0)
    assert replicas.max_over_ranks(3.0) == 3.0
    assert replicas.aggregate_rate(10.0, 2.0) == 5000.0
