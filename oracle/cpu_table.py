"""ORACLE / TEST INFRASTRUCTURE ONLY: the CPU baseline table of the benchmark
configurations, timed on the host it runs on.

For each configuration: the reference's sequential engine (vtkUniformClustering,
restated in acvd_port.cpp and pinned to the reference's own code) on one core, and
ACVDQP (vtkThreadedClustering, restated, pinned by energy) with every host core as a
thread, each from the reference's own initial sampling (the seeded single-item seeds
for the icosphere).  The time is the reference's clustering timer's span
(MinimizeEnergy); the energy is the reference's evaluation of the final clustering.
The 4096^2 heightfield's sequential solve takes about a quarter of an hour and is
skipped unless --with-slow is given (its converged energy and time from one x86 core
are in tests/golden/fullsize/heightfield_4096_aniso.json).  The batch solves every
mesh on its own, one mesh per core at a time.

    python oracle/cpu_table.py [--with-slow] > table.json
"""
from __future__ import annotations

import json
import multiprocessing as mp
import os
import platform
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
# run as a script, this directory would shadow the oracle package: the repository root instead
sys.path[0] = os.path.dirname(HERE)

import numpy as np  # noqa: E402

CONFIGS = {
    # name: (generator, kwargs, metric, K, gradation, unconstrained init, seeds, density)
    "C1 icosphere L5 iso": ("icosphere", {"level": 5, "seed": 0}, "iso", 1000, 0.0, 0, True, False),
    "C2 torus 1024x512 QEM": ("torus", {"nu": 1024, "nv": 512, "seed": 0}, "qem", 20000, 1.5, 1, False, False),
    "C3 heightfield 4096^2 aniso": ("heightfield", {"n": 4096, "seed": 0}, "aniso", 200000, 1.5, 0, False, False),
    "C5 torus 512x512 QEM": ("torus", {"nu": 512, "nv": 512, "seed": 0}, "qem", 10000, 1.0, 1, False, True),
}


def _mesh(cfg):
    from acvd_gb300 import synth
    kind, kw, metric, k, grad, uinit, seeds, dens = cfg
    m = synth.make(kind, **kw)
    ind = m.indicator
    if dens:
        ind = np.random.default_rng(1).uniform(0.5, 2.0, size=m.n_points)
    use_ind = grad != 0.0 if metric == "aniso" else grad > 0.0
    return m, (ind if use_ind else None), (m.principal_dirs if metric == "aniso" else None)


def solve(cfg, threads):
    from acvd_gb300 import synth
    from oracle import oracle
    kind, kw, metric, k, grad, uinit, seeds, dens = cfg
    m, ind, pd = _mesh(cfg)
    p = oracle.Port(metric, m.points, m.faces, k, grad, ind, pd, unconstrained_init=uinit)
    if threads:
        p.set_option("threads", threads)
    p.init(synth.seed_labels(m.n_points, k, seed=0) if seeds else None)
    secs = p.run()
    ev = oracle.Port(metric, m.points, m.faces, k, grad, ind, pd)
    ev.evaluate(p.labels(), 1)
    return {"items": int(m.n_points), "seconds": secs, "items_per_s": m.n_points / secs,
            "energy": ev.global_energy(), "connected": bool(ev.clean() == 0)}


def _batch_job(a):
    spec, ipc = a
    from acvd_gb300 import batch as B
    from oracle import oracle
    m = B.mesh_from_spec(spec, False)
    k = max(1, m.n_points // ipc)
    p = oracle.Port("qem", m.points, m.faces, k, 0.0, unconstrained_init=1)
    p.init(None)
    return m.n_points, p.run()


def main():
    from oracle import oracle
    from acvd_gb300 import synth
    oracle.build(ref=False)
    cores = os.cpu_count() or 1
    slow = "--with-slow" in sys.argv
    out = {"host": platform.machine(), "processor": platform.processor(), "cores": cores, "rows": []}
    try:
        with open("/proc/cpuinfo") as f:
            model = [ln.split(":", 1)[1].strip() for ln in f if ln.lower().startswith(("model name", "cpu part"))]
        out["cpu"] = model[0] if model else None
    except OSError:
        out["cpu"] = None
    for name, cfg in CONFIGS.items():
        heavy = cfg[0] == "heightfield" and cfg[1]["n"] >= 4096
        for threads in (0, cores):
            if heavy and threads == 0 and not slow:
                continue
            t0 = time.time()
            r = solve(cfg, threads)
            r.update({"config": name, "engine": "ACVDQP" if threads else "sequential", "threads": threads or 1,
                      "wall_s": time.time() - t0})
            out["rows"].append(r)
            print(json.dumps(r), file=sys.stderr, flush=True)
    # the batch: every mesh solved on its own, one mesh per core
    specs = synth.batch_specs(256, 0)
    t0 = time.time()
    from acvd_gb300 import batch as B
    jobs = sorted(((s, 20) for s in specs), key=lambda j: -B.spec_items(j[0]))
    with mp.get_context("spawn").Pool(cores) as pool:
        res = pool.map(_batch_job, jobs, chunksize=1)
    wall = time.time() - t0
    total = sum(r[1] for r in res)
    out["rows"].append({"config": "C4 batch of 256 QEM", "engine": "sequential per mesh", "threads": cores,
                        "items": int(sum(r[0] for r in res)), "seconds_summed_1_core": total,
                        "meshes_per_s_1_core": 256 / total, "wall_s_all_cores": wall,
                        "meshes_per_s_all_cores": 256 / wall})
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
