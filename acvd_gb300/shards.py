"""Batched clustering sharded by mesh over the GPUs of one node.

The meshes of a batch are independent: nothing is exchanged between them while
they are clustered.  A multi-GPU batch run therefore splits the meshes over the
ranks (one process per GPU, as torchrun launches them), every rank packs its share
into one CSR and clusters it (acvd_gb300.batch), and the per-mesh labels and
energies are gathered on rank 0 afterwards.  No collective runs on the data path.
The reference's CPU analogue hands one label's mesh to each host thread
(DiscreteRemeshing/Examples/VolumeAnalysis.cxx:108-300, threads at :153).

The split balances the items per rank: meshes are dealt largest first, each to the
rank with the fewest items so far (ties to the lower rank), so that the busiest rank
holds at most the average plus one mesh.
"""
from __future__ import annotations

import numpy as np


def balanced_partition(sizes, n_parts: int) -> list[list[int]]:
    """Mesh indices per part, each part in increasing mesh order.  Largest mesh first
    to the least-loaded part (lowest part index on ties); deterministic."""
    if n_parts < 1:
        raise ValueError("n_parts must be at least 1")
    sizes = [int(s) for s in sizes]
    order = sorted(range(len(sizes)), key=lambda m: (-sizes[m], m))
    load = [0] * n_parts
    parts: list[list[int]] = [[] for _ in range(n_parts)]
    for m in order:
        p = min(range(n_parts), key=lambda r: (load[r], r))
        parts[p].append(m)
        load[p] += sizes[m]
    return [sorted(p) for p in parts]


def part_loads(sizes, parts) -> list[int]:
    return [int(sum(int(sizes[m]) for m in p)) for p in parts]


def gather_meshes(local: dict, n_meshes: int, rank: int, ws: int):
    """Gathers {mesh index: result} from every rank on rank 0 and returns the results
    in mesh order there (None on the other ranks).  Every mesh must come from exactly
    one rank."""
    if ws == 1:
        merged = dict(local)
    else:
        import torch.distributed as dist
        got = [None] * ws if rank == 0 else None
        dist.gather_object(local, got, dst=0)
        if rank != 0:
            return None
        merged = {}
        for part in got:
            for m, r in part.items():
                if m in merged:
                    raise RuntimeError(f"mesh {m} came from two ranks")
                merged[m] = r
    missing = [m for m in range(n_meshes) if m not in merged]
    if missing:
        raise RuntimeError(f"meshes missing from the gather: {missing[:8]}")
    return [merged[m] for m in range(n_meshes)]


def split_packed(labels: np.ndarray, v_off, k_off, ks) -> list[np.ndarray]:
    """Per-mesh labels in each mesh's own numbering (null = its own K) from a packed
    batch clustering."""
    out = []
    for m in range(len(ks)):
        lab = labels[v_off[m]:v_off[m + 1]].astype(np.int64) - int(k_off[m])
        k = int(ks[m])
        lab[(lab < 0) | (lab >= k)] = k
        out.append(lab.astype(np.int32))
    return out
