"""Batch sharded by mesh over ranks (acvd_gb300.shards), on CPU: the partition covers
every mesh once and balances the items; two gloo ranks each solve their share of a
small batch with the oracle's restatement (the GPU solve is the same per-mesh
function), the per-mesh results are gathered on rank 0 and equal a single-process
run mesh for mesh."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp

from acvd_gb300 import batch as B
from acvd_gb300 import shards
from acvd_gb300 import synth


def test_partition_covers_and_balances():
    specs = synth.batch_specs(256, 0)
    sizes = [B.spec_items(s) for s in specs]
    for n in (1, 2, 3, 4, 8):
        parts = shards.balanced_partition(sizes, n)
        assert len(parts) == n
        flat = sorted(m for p in parts for m in p)
        assert flat == list(range(256))
        assert all(p == sorted(p) for p in parts)
        loads = shards.part_loads(sizes, parts)
        # largest-first greedy: the busiest part exceeds the average by less than one mesh
        assert max(loads) - sum(loads) / n <= max(sizes)
        assert shards.balanced_partition(sizes, n) == parts       # deterministic
    assert shards.balanced_partition([5, 5, 5], 2) == [[0, 2], [1]]
    with pytest.raises(ValueError):
        shards.balanced_partition(sizes, 0)


def test_split_packed_and_single_rank_gather():
    specs = synth.batch_specs(6, 3, lo=200, hi=900)
    b = B.batch_from_specs(specs)
    per = shards.split_packed(b.labels0, b.v_off, b.k_off, b.ks)
    for m in range(6):
        np.testing.assert_array_equal(per[m], b.mesh_labels(b.labels0, m))
    got = shards.gather_meshes({m: m * m for m in range(6)}, 6, 0, 1)
    assert got == [m * m for m in range(6)]
    with pytest.raises(RuntimeError):
        shards.gather_meshes({0: 1}, 2, 0, 1)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


SPECS = dict(n=10, seed=5, lo=300, hi=3000)


def _solve_mesh(spec):
    """One mesh of the batch: the reference's sampling and sequential solve (oracle)."""
    from oracle import oracle
    m = B.mesh_from_spec(spec, False)
    k = max(1, m.n_points // 20)
    p = oracle.Port("qem", m.points, m.faces, k, 0.0, unconstrained_init=1)
    p.init(None)
    p.run()
    return p.labels(), p.global_energy()


def _rank(rank, ws, port, out):
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(ws),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    from acvd_gb300 import replicas
    replicas.init("gloo")
    specs = synth.batch_specs(SPECS["n"], SPECS["seed"], SPECS["lo"], SPECS["hi"])
    parts = shards.balanced_partition([B.spec_items(s) for s in specs], ws)
    local = {m: _solve_mesh(specs[m]) for m in parts[rank]}
    res = shards.gather_meshes(local, len(specs), rank, ws)
    if rank == 0:
        out.put([(lab.tolist(), e) for lab, e in res])
    else:
        assert res is None
        out.put(None)
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_gloo_ranks_gather_every_mesh(oracle_lib):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = [q.get(timeout=300) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res = next(g for g in got if g is not None)
    specs = synth.batch_specs(SPECS["n"], SPECS["seed"], SPECS["lo"], SPECS["hi"])
    assert len(res) == len(specs)
    for m, spec in enumerate(specs):
        lab, e = _solve_mesh(spec)
        assert res[m][0] == lab.tolist() and res[m][1] == e, m
