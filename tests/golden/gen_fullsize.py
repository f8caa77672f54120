"""Writes the full-size energy fixtures (tests/golden/fullsize/*.json).

TEST INFRASTRUCTURE: runs the oracle's restatement of the reference's sequential
MinimizeEnergy (oracle/acvd_port.cpp, pinned bit for bit to the reference's own
headers compiled against the VTK shim) on the benchmark configurations whose CPU
solves are too long for a test or a bench run:

* heightfield_4096_aniso -- quadric-anisotropic metric, heightfield 4096^2
  (16,777,216 items), K = 200,000, gradation 1.5;
* batch_256_qem -- the 256 meshes of the batched QEM workload, each solved on its own;
* torus_1024x512_qem -- ACVDQ torus 1024x512, K = 20,000, gradation 1.5 (cheap; kept
  for the full-size parity test).

For each mesh the fixture holds the SHA-256 of the initial clustering that the
reference's ComputeInitialRandomSampling gives (Common/vtkUniformClustering.h:1178-1316,
run by the oracle), and the energy that the reference's evaluation
(Init + ReComputeStatistics with the placement on, :353-403, ComputeGlobalEnergy
:1319-1346) assigns to the CPU run's converged clustering.  A GPU run from the same
initial clustering must land within 0.1 % of that energy.

    python tests/golden/gen_fullsize.py [torus_1024x512_qem] [heightfield_4096_aniso] [batch_256_qem]
"""
from __future__ import annotations

import hashlib
import json
import multiprocessing as mp
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
OUT = os.path.join(HERE, "fullsize")

SINGLE = {
    # name: (generator, generator kwargs, metric, K, gradation, unconstrained init, density)
    "torus_1024x512_qem": ("torus", {"nu": 1024, "nv": 512, "seed": 0}, "qem", 20000, 1.5, 1),
    "heightfield_4096_aniso": ("heightfield", {"n": 4096, "seed": 0}, "aniso", 200000, 1.5, 0),
}
BATCH = {"batch_256_qem": dict(n_meshes=256, seed=0, metric="qem", gradation=0.0, uinit=1, items_per_cluster=20)}


def labels_sha(lab: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(lab, dtype=np.int32).tobytes()).hexdigest()


def solve(metric, points, faces, k, gradation, ind, pd, uinit):
    """The reference's default initial sampling, a converged sequential solve, and the
    reference's evaluation of the result."""
    from oracle import oracle
    p = oracle.Port(metric, points, faces, k, gradation, ind, pd, unconstrained_init=uinit)
    p.init(None)
    lab0 = p.labels()
    secs = p.run()
    lab = p.labels()
    ev = oracle.Port(metric, points, faces, k, gradation, ind, pd)
    ev.evaluate(lab, 1)
    e = ev.global_energy()
    connected = ev.clean() == 0
    return lab0, lab, e, secs, connected


def gen_single(name):
    from acvd_gb300 import synth
    kind, kw, metric, k, grad, uinit = SINGLE[name]
    m = synth.make(kind, **kw)
    use_ind = grad != 0.0 if metric == "aniso" else grad > 0.0
    ind = m.indicator if use_ind else None
    pd = m.principal_dirs if metric == "aniso" else None
    t0 = time.time()
    lab0, lab, e, secs, connected = solve(metric, m.points, m.faces, k, grad, ind, pd, uinit)
    rec = {"workload": name, "items": int(m.n_points), "clusters": int(k), "metric": metric, "gradation": grad,
           "unconstrained_init": uinit, "labels0_sha256": labels_sha(lab0),
           "reference_energy": e, "reference_connected": bool(connected),
           "reference_assigned": bool(np.all(lab < k)),
           "cpu_minimize_s": secs, "wall_s": time.time() - t0,
           "generator": f"synth.{kind}({kw}), analytic curvature"}
    return rec


def _batch_job(a):
    kind, kw, metric, grad, uinit, ipc = a
    from acvd_gb300 import synth
    curv = grad != 0.0 or metric == "aniso"
    m = synth.make(kind, with_curvature=curv, **kw)
    k = max(1, m.n_points // ipc)
    use_ind = grad != 0.0 if metric == "aniso" else grad > 0.0
    lab0, lab, e, secs, connected = solve(metric, m.points, m.faces, k, grad, m.indicator if use_ind else None,
                                          None, uinit)
    return {"kind": kind, "params": kw, "items": int(m.n_points), "clusters": int(k),
            "labels0_sha256": labels_sha(lab0), "reference_energy": e, "reference_connected": bool(connected),
            "cpu_minimize_s": secs}


def gen_batch(name):
    from acvd_gb300 import synth
    from oracle import oracle
    b = BATCH[name]
    specs = synth.batch_specs(b["n_meshes"], b["seed"])
    jobs = [(kind, kw, b["metric"], b["gradation"], b["uinit"], b["items_per_cluster"]) for kind, kw in specs]
    oracle.build(ref=False)
    t0 = time.time()
    # largest meshes first so that the pool ends evenly
    order = sorted(range(len(jobs)), key=lambda j: -_size_hint(jobs[j]))
    with mp.get_context("spawn").Pool(os.cpu_count() or 1) as pool:
        res = pool.map(_batch_job, [jobs[j] for j in order], chunksize=1)
    meshes = [None] * len(jobs)
    for j, r in zip(order, res):
        meshes[j] = r
    return {"workload": name, "meshes": meshes, "metric": b["metric"], "gradation": b["gradation"],
            "unconstrained_init": b["uinit"], "items_per_cluster": b["items_per_cluster"],
            "wall_s": time.time() - t0, "generator": f"synth.batch_specs({b['n_meshes']}, {b['seed']})"}


def _size_hint(job):
    kind, kw = job[0], job[1]
    if kind == "icosphere":
        return 10 * 4 ** kw["level"]
    if kind == "torus":
        return kw["nu"] * kw["nv"]
    return kw["n"] ** 2


def main():
    from oracle import oracle
    oracle.build(ref=False)
    os.makedirs(OUT, exist_ok=True)
    names = sys.argv[1:] or list(SINGLE) + list(BATCH)
    for name in names:
        rec = gen_batch(name) if name in BATCH else gen_single(name)
        with open(os.path.join(OUT, name + ".json"), "w") as f:
            json.dump(rec, f, indent=1)
        print(name, "done in", round(rec["wall_s"], 1), "s", flush=True)


if __name__ == "__main__":
    main()
